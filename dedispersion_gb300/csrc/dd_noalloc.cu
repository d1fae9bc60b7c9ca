// dd_noalloc.cu -- single-step dedispersion that allocates no device memory.
//
// Some callers cannot call cudaMalloc at the point where they dedisperse: a
// real-time beamformer loop that must never block (cudaMalloc and cudaFree
// can synchronize the whole device), or a host framework that owns all device
// memory through its own pool and caps it, so a library allocating behind its
// back could fail or fragment the pool.  dd_dedispersion_noalloc serves them:
// the caller passes device input and output buffers it already owns, and the
// engine's own per-call working memory -- the group and row descriptor tables
// the kernel reads and the status word it writes -- lives in one file-scope
// `__device__` array of fixed size (kScratchBytes, about 1 MiB), which every
// GPU that loads the library holds until the process exits.
//
// Limits: at most kMaxGroups synthesized beams and kMaxEntries live rows
// (synthesized beams x non-zapped channels) per call; larger requests are
// rejected with DD_ERR_UNSUPPORTED.  Every call shares the one array and it
// keeps the last call's contents, so calls that overlap on the GPU (two host
// threads, or two streams) race; host threads are serialized by a mutex here,
// but work queued on different streams by other means is not.  Each call
// waits on its stream for its own kernel (it reads the status word back)
// before it returns; the stream must belong to the current device.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>

#include "../../include/dedisp_gb300.h"
#include "dd_internal.h"

namespace dd {
void set_last_error(const char *message);
}

namespace {

constexpr size_t kMaxGroups = 4096;
constexpr size_t kMaxEntries = 61440;
constexpr size_t kStatusBytes = 256;
constexpr size_t kGroupOffset = kStatusBytes;
constexpr size_t kEntryOffset = kGroupOffset + kMaxGroups * sizeof(dd::GroupDesc);
constexpr size_t kScratchBytes = kEntryOffset + kMaxEntries * sizeof(dd::EntryDesc);
constexpr int kMaxDevices = 64;

// The scratch array.  In host code its name is only a stand-in: the device
// address comes from cudaGetSymbolAddress, once per device.
static __device__ __align__(256) unsigned char dd_noalloc_scratch[kScratchBytes];

std::mutex g_mutex;                         // serializes calls and guards what follows
void *g_scratch_addr[kMaxDevices] = {};     // device address of the array, per device
alignas(64) unsigned char g_stage[kScratchBytes];  // host image of the tables

dd_status fail(dd_status code, const char *fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  dd::set_last_error(buf);
  return code;
}

dd_status cuda_fail(cudaError_t e, const char *what) {
  (void)cudaGetLastError();
  return fail(e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver ? DD_ERR_NO_DEVICE
                                                                        : DD_ERR_CUDA,
              "%s: %s", what, cudaGetErrorString(e));
}

uint64_t pad_to(uint64_t v, uint64_t p) { return p == 0 ? v : (v + p - 1) / p * p; }

}  // namespace

extern "C" dd_status dd_dedispersion_noalloc(const dd_observation *o, const uint32_t *zapped,
                                             const uint32_t *beam_mapping, const void *d_input,
                                             float *d_output, const float *shifts,
                                             uint32_t padding, uint32_t input_bits,
                                             void *stream) {
  if (!o || !zapped || !beam_mapping || !shifts)
    return fail(DD_ERR_INVALID_ARGUMENT, "NULL host table");
  if (o->downsampling != 1) return fail(DD_ERR_UNSUPPORTED, "downsampling must be 1");
  if (o->nr_channels == 0) return fail(DD_ERR_INVALID_ARGUMENT, "nr_channels is 0");
  if (!(o->first_dm >= 0.0f) || !(o->dm_step >= 0.0f))
    return fail(DD_ERR_INVALID_ARGUMENT, "DM first/step must be non-negative");
  const uint32_t bits = input_bits;
  if (!(bits == 1 || bits == 2 || bits == 4 || bits == 8 || bits == 16 || bits == 32))
    return fail(DD_ERR_UNSUPPORTED, "input_bits %u not supported", bits);
  const uint32_t C = o->nr_channels, G = o->nr_synthesized_beams;
  const uint32_t D = o->nr_dms, S = o->nr_samples_per_batch;
  if (G > kMaxGroups)
    return fail(DD_ERR_UNSUPPORTED, "%u synthesized beams exceed the no-alloc limit of %zu", G,
                kMaxGroups);
  uint64_t live = 0;
  for (uint32_t c = 0; c < C; c++) live += zapped[c] == 0;
  if (live * G > kMaxEntries)
    return fail(DD_ERR_UNSUPPORTED,
                "%llu live rows (synthesized beams x non-zapped channels) exceed the no-alloc "
                "limit of %zu",
                (unsigned long long)(live * G), kMaxEntries);
  if (D == 0 || S == 0 || G == 0) return DD_OK;
  if (!d_input || !d_output) return fail(DD_ERR_INVALID_ARGUMENT, "NULL device buffer");

  // The default compiled configuration of this input width (registry order).
  int nk = 0;
  const dd::KernelInfo *reg = dd::kernel_registry(&nk), *k = nullptr;
  const int fam_bits = bits <= 8 ? 8 : (int)bits;
  for (int i = 0; i < nk && !k; i++)
    if (reg[i].elem_bits == fam_bits) k = &reg[i];
  if (!k) return fail(DD_ERR_UNSUPPORTED, "no kernel for %u-bit input", bits);

  // Reference layout of one single-step batch (include/Dedispersion.hpp:70-109).
  uint64_t row_bytes;
  if (bits < 8) {
    const uint32_t per = 8 / bits;
    row_bytes = pad_to((o->nr_samples_per_dispersed_batch + per - 1) / per, padding);
  } else {
    row_bytes = pad_to(o->nr_samples_per_dispersed_batch, padding / (bits / 8)) * (bits / 8);
  }
  const uint64_t out_row = pad_to(S, padding / 4);
  const uint64_t map_row = pad_to(C, padding / 4);

  std::lock_guard<std::mutex> lock(g_mutex);
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_fail(e, "current device");
  if (dev < 0 || dev >= kMaxDevices) return fail(DD_ERR_UNSUPPORTED, "device %d", dev);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (s != nullptr) {
    // The scratch address and the kernel launch are the current device's:
    // a stream of another device would be handed a foreign address.
    int sdev = -1;
    e = cudaStreamGetDevice(s, &sdev);
    if (e != cudaSuccess) return cuda_fail(e, "device of the stream");
    if (sdev != dev)
      return fail(DD_ERR_INVALID_ARGUMENT,
                  "the stream belongs to device %d but device %d is current", sdev, dev);
  }
  if (!g_scratch_addr[dev]) {
    // Set-up, once per device, with that device current: the first call on
    // a device does it, so that first call should come before any stream
    // capture begins.
    void *addr = nullptr;
    e = cudaGetSymbolAddress(&addr, dd_noalloc_scratch);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(dd_noalloc_scratch)");
    g_scratch_addr[dev] = addr;
  }
  unsigned char *scratch = static_cast<unsigned char *>(g_scratch_addr[dev]);

  // Group and row descriptors, built in the host image of the array.
  dd::GroupDesc *groups = reinterpret_cast<dd::GroupDesc *>(g_stage + kGroupOffset);
  dd::EntryDesc *entries = reinterpret_cast<dd::EntryDesc *>(g_stage + kEntryOffset);
  uint32_t ne = 0, max_delay = 0, spread = 0;
  for (uint32_t g = 0; g < G; g++) {
    groups[g].entry_begin = ne;
    groups[g].out_offset = (uint64_t)g * D * out_row;
    for (uint32_t c = 0; c < C; c++) {
      if (zapped[c] != 0) continue;
      const uint64_t beam = beam_mapping[(uint64_t)g * map_row + c];
      if (beam >= o->nr_beams)
        return fail(DD_ERR_INVALID_ARGUMENT, "beam mapping[%u][%u] = %llu >= nr_beams %u", g, c,
                    (unsigned long long)beam, o->nr_beams);
      const float sh = shifts[c];
      if (!(sh >= 0.0f) || !std::isfinite(sh))
        return fail(DD_ERR_INVALID_ARGUMENT, "shift[%u] must be finite and >= 0", c);
      entries[ne].row_offset = (beam * C + c) * row_bytes;
      entries[ne].shift = sh;
      entries[ne].delay_row = 0;
      ne++;
    }
    groups[g].entry_count = ne - groups[g].entry_begin;
  }
  const uint32_t tiles_d = (D + k->tile_d - 1) / k->tile_d;
  const uint32_t tiles_t = (S + k->tile_t - 1) / k->tile_t;
  for (uint32_t c = 0; c < C; c++) {
    if (zapped[c] != 0) continue;
    const float sh = shifts[c];
    max_delay = std::max(max_delay, dd::host_delay(o->first_dm, o->dm_step, D - 1, sh));
    for (uint32_t t = 0; t < tiles_d; t++) {
      const uint32_t d0 = t * k->tile_d, d1 = std::min(d0 + k->tile_d, D) - 1;
      spread = std::max(spread, dd::host_delay(o->first_dm, o->dm_step, d1, sh) -
                                    dd::host_delay(o->first_dm, o->dm_step, d0, sh));
    }
  }
  if ((uint64_t)S + max_delay > o->nr_samples_per_dispersed_batch)
    return fail(DD_ERR_INVALID_ARGUMENT,
                "rows hold %u samples but %u output samples + max delay %u are needed",
                o->nr_samples_per_dispersed_batch, S, max_delay);
  const uint32_t a = dd::window_alignment_samples(bits);
  const uint32_t win = ((k->tile_t + spread + a + 8) + 15) / 16 * 16;
  const size_t smem = dd::kernel_smem_bytes(*k, win, bits);
  int smem_max = 0;
  e = cudaDeviceGetAttribute(&smem_max, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  if (e != cudaSuccess) return cuda_fail(e, "query shared memory");
  if (smem > (size_t)smem_max)
    return fail(DD_ERR_UNSUPPORTED, "window of %u samples needs %zu bytes of shared memory", win,
                smem);
  e = cudaFuncSetAttribute(k->func, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_max);
  if (e != cudaSuccess) return cuda_fail(e, "set kernel shared memory");

  // The status word must start at zero; the tables are overwritten in full.
  e = cudaMemsetAsync(scratch, 0, sizeof(uint32_t), s);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(scratch + kGroupOffset, g_stage + kGroupOffset,
                        G * sizeof(dd::GroupDesc), cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess && ne)
    e = cudaMemcpyAsync(scratch + kEntryOffset, g_stage + kEntryOffset,
                        ne * sizeof(dd::EntryDesc), cudaMemcpyHostToDevice, s);
  if (e != cudaSuccess) return cuda_fail(e, "upload descriptor tables");

  dd::ProblemDesc P{};
  P.in = static_cast<const uint8_t *>(d_input);
  P.out = d_output;
  P.groups = reinterpret_cast<const dd::GroupDesc *>(scratch + kGroupOffset);
  P.entries = reinterpret_cast<const dd::EntryDesc *>(scratch + kEntryOffset);
  P.status = reinterpret_cast<uint32_t *>(scratch);
  P.row_bytes = row_bytes;
  P.out_dm_stride = out_row;
  P.nr_groups = G;
  P.nr_dms = D;
  P.nr_samples = S;
  P.bits = bits;
  P.first_dm = o->first_dm;
  P.dm_step = o->dm_step;
  P.win_samples = win;
  P.tiles_t = tiles_t;
  P.tiles_d = tiles_d;
  P.tma = (row_bytes % 16 == 0 && reinterpret_cast<uintptr_t>(d_input) % 16 == 0) ? 1u : 0u;
  P.out_vec4 = (out_row % 4 == 0 && reinterpret_cast<uintptr_t>(d_output) % 16 == 0) ? 1u : 0u;
  P.mul_hi8 = 1u << 24;
  const uint64_t tiles = (uint64_t)G * tiles_d * tiles_t;
  if (tiles > 0x7fffffffull) return fail(DD_ERR_UNSUPPORTED, "too many tiles");
  k->launch(P, (unsigned)tiles, smem, s);
  e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, "launch dedispersion kernel");

  // Wait for this call and read its status word.
  uint32_t status = 0;
  e = cudaMemcpyAsync(&status, scratch, sizeof(status), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return cuda_fail(e, "wait for dedispersion");
  if (status & dd::kStatusTimeout)
    return fail(DD_ERR_TIMEOUT, "a bounded wait for a staged row ran out on the device");
  if (status) return fail(DD_ERR_CUDA, "device status 0x%x", status);
  return DD_OK;
}
