// dd_subband.cu -- the subband method as one pipeline on the device: step one
// then step two, the intermediate kept in device memory the pipeline owns.
//
// The reference computes the two steps as separate calls with a float
// intermediate of [beam][coarse DM][subband][S1] (include/Dedispersion.hpp:
// 111-176); its drivers never chain them (src/DedispersionTest.cpp runs one
// step per invocation).  Here, when the step-one sums fit 16 bits (live
// channels per subband x (2^bits - 1) <= 65535, e.g. up to 257 channels of
// 8-bit input), the intermediate is packed: one 32-bit word per sample holds
// the exact sums of two coarse DMs (ProblemDesc::packed).  That halves its
// bytes (101 MB instead of 202 MB at 1536 channels, 32 subbands, 64 coarse
// DMs, 24649 samples), so the round trip through device memory halves too,
// and step two's pair tile adds both coarse DMs with one load and one add.
// Sums are integers below 2^24 either way, so the output equals the
// reference's float step one followed by its float step two bit for bit.
// Otherwise (16-bit or float input, or wider subbands) the pipeline runs the
// two float steps.  With one launch per step most of the intermediate goes
// through device memory; dd_subband_set_chunks runs the steps interleaved
// over time ranges so that step two reads it back from L2 (fewer DRAM bytes,
// more partial waves: slower on compute-bound shapes, hence opt-in).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <vector>

#include "../../include/dedisp_gb300.h"
#include "dd_kernels.cuh"

namespace dd {
void set_last_error(const char *message);
void plan_set_packed(dd_plan *p, const KernelInfo *k, uint32_t flush_rows);
void plan_clear_packed(dd_plan *p);
bool plan_ready(const dd_plan *p);
dd_status plan_problem(const dd_plan *p, const void *d_input, float *d_output,
                       ProblemDesc *out, uint64_t *rows_per_group);
dd_status plan_launch_range(const dd_plan *p, ProblemDesc P, uint32_t base, uint32_t count,
                            cudaStream_t stream);
dd_status plan_time_tiles(const dd_plan *p, uint32_t *tiles_t, uint32_t *tile_t,
                          uint32_t *max_delay);

// Largest step-one sum: live channels of the fullest subband x the largest
// sample of `bits`-bit input (0 when the width has no integer bound).
uint64_t subband_largest_sum(const dd_observation *o, const uint32_t *zapped, uint32_t bits) {
  const uint32_t C = o->nr_channels, SB = o->nr_subbands;
  if (SB == 0 || bits > 16) return 0;
  const uint32_t cps = C / SB;
  uint32_t live_max = 0;
  for (uint32_t sb = 0; sb < SB; sb++) {
    uint32_t live = 0;
    for (uint32_t c = sb * cps; c < (sb + 1) * cps; c++) live += (zapped && zapped[c]) ? 0u : 1u;
    live_max = std::max(live_max, live);
  }
  return (uint64_t)live_max * ((1ull << bits) - 1);
}

// Whether the packed intermediate holds this shape's step-one sums exactly.
bool subband_packable(const dd_observation *o, const uint32_t *zapped, uint32_t bits) {
  return bits <= 8 && o->nr_subbands && subband_largest_sum(o, zapped, bits) <= 0xFFFFu;
}

// Turns step plans `one` and `two` (tables set) into a packed pair where the
// sums fit and both build (else leaves them as float steps).  Returns whether
// they are packed.
bool subband_try_pack(dd_plan *one, dd_plan *two, const dd_observation *o, const uint32_t *zapped,
                      uint32_t bits, int pair_kernel) {
  if (!subband_packable(o, zapped, bits)) return false;
  const uint64_t big = subband_largest_sum(o, zapped, bits);
  const uint32_t flush = (uint32_t)std::max<uint64_t>(1, big ? 0xFFFFu / big : 0xFFFFu);
  int n = 0;
  const KernelInfo *pk = pair_kernels(&n);
  // The default step-one tile (short groups) takes subbands of at most 257
  // rows; sub-byte input packs wider subbands, which take the tile with
  // 32-bit totals instead.
  const KernelInfo *k1 = nullptr;
  const uint64_t rows = big / ((1ull << bits) - 1ull);
  if (rows > 257) {
    int nk = 0;
    const KernelInfo *reg = kernel_registry(&nk);
    for (int i = 0; i < nk && !k1; i++)
      if (std::strcmp(reg[i].name, "swar8_i2_d8_w8_c16_vkUnpackPermuteMad") == 0) k1 = &reg[i];
  }
  plan_set_packed(one, k1, 0);
  plan_set_packed(two, &pk[std::min(std::max(pair_kernel, 0), n - 1)], flush);
  if (plan_ready(one) && plan_ready(two)) return true;
  plan_clear_packed(one);
  plan_clear_packed(two);
  return false;
}
}  // namespace dd

namespace {

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
  if (e == cudaErrorMemoryAllocation)
    return fail(DD_ERR_OUT_OF_MEMORY, "%s: %s", what, cudaGetErrorString(e));
  return fail(DD_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

#define DDS_CUDA(call, what)                           \
  do {                                                 \
    cudaError_t e_ = (call);                           \
    if (e_ != cudaSuccess) return cuda_fail(e_, what); \
  } while (0)

}  // namespace

struct dd_subband {
  int device = 0;
  dd_observation obs{};
  uint32_t bits = 8, padding = 0;
  dd_plan *one = nullptr, *two = nullptr;
  bool packed = false;
  bool ready = false;
  int pair_kernel = 0;  // index into dd::pair_kernels
  bool overlap = false;  // step one as a programmatic dependent
  void *inter = nullptr;  // step-one output (packed or float)
  size_t inter_bytes = 0;
  uint32_t chunks = 0;              // dd_subband_set_chunks (0, 1: whole steps)
  cudaStream_t side = nullptr;      // step one of a chunked run
  std::vector<cudaEvent_t> events;  // fork, then one per chunk
  std::vector<float> shifts, shifts2;
  std::vector<uint32_t> zapped, mapping;
};

namespace {

void drop_plans(dd_subband *s) {
  if (s->one) dd_plan_destroy(s->one);
  if (s->two) dd_plan_destroy(s->two);
  s->one = s->two = nullptr;
}

dd_status make_plans(dd_subband *s) {
  drop_plans(s);
  dd_status st = dd_plan_create(&s->one, &s->obs, DD_STEP_ONE, s->bits, s->padding, nullptr,
                                s->device);
  if (!st) st = dd_plan_create(&s->two, &s->obs, DD_STEP_TWO, 32, s->padding, nullptr, s->device);
  if (!st) st = dd_plan_set_shifts(s->one, s->shifts.data(), s->shifts.size());
  if (!st) st = dd_plan_set_zapped(s->one, s->zapped.data(), s->zapped.size());
  if (!st) st = dd_plan_set_shifts(s->two, s->shifts2.data(), s->shifts2.size());
  if (!st) st = dd_plan_set_beam_mapping(s->two, s->mapping.data(), s->mapping.size());
  if (!st) st = dd_plan_set_overlap(s->one, s->overlap ? 1 : 0);
  return st;
}

// Builds both plans, packed where the sums fit, and sizes the intermediate.
dd_status build(dd_subband *s) {
  s->ready = false;
  dd_status st = make_plans(s);
  if (st) return st;
  s->packed = dd::subband_try_pack(s->one, s->two, &s->obs, s->zapped.data(), s->bits,
                                   s->pair_kernel);
  uint64_t adds = 0;  // builds the tables, reporting why they are invalid
  st = dd_plan_adds(s->one, &adds);
  if (!st) st = dd_plan_adds(s->two, &adds);
  if (st) return st;
  dd_layout lay;
  st = dd_get_layout(&s->obs, DD_STEP_ONE, s->bits, s->padding, nullptr, &lay);
  if (st) return st;
  const uint64_t D1 = s->obs.nr_dms_subbanding;
  size_t bytes = lay.output_bytes;
  if (s->packed && D1) bytes = lay.output_bytes / D1 * ((D1 + 1) / 2);
  if (bytes > s->inter_bytes) {
    if (s->inter) cudaFree(s->inter);
    s->inter = nullptr;
    s->inter_bytes = 0;
    DDS_CUDA(cudaSetDevice(s->device), "select device");
    DDS_CUDA(cudaMalloc(&s->inter, std::max<size_t>(bytes, 16)), "allocate intermediate");
    s->inter_bytes = bytes;
  }
  s->ready = true;
  return DD_OK;
}

// Per-thread state of the synchronous host-buffer call.
struct HostCache {
  dd_subband *pipe = nullptr;
  dd_observation obs{};
  uint32_t bits = 0, padding = 0;
  void *d_in = nullptr, *d_out = nullptr;
  uint64_t cap_in = 0, cap_out = 0;
  cudaStream_t stream = nullptr;
  void reset() {
    if (pipe) dd_subband_destroy(pipe);
    pipe = nullptr;
  }
  ~HostCache() {
    reset();
    if (d_in) cudaFree(d_in);
    if (d_out) cudaFree(d_out);
    if (stream) cudaStreamDestroy(stream);
  }
};
thread_local HostCache g_host;

}  // namespace

extern "C" {

dd_status dd_subband_create(dd_subband **pipeline, const dd_observation *obs,
                            uint32_t input_bits, uint32_t padding, int device) {
  if (!pipeline || !obs) return fail(DD_ERR_INVALID_ARGUMENT, "NULL argument");
  *pipeline = nullptr;
  if (obs->nr_subbands == 0) return fail(DD_ERR_INVALID_ARGUMENT, "observation has no subbands");
  // Validate geometry, bits and device through the step plans themselves.
  dd_plan *probe = nullptr;
  dd_status st = dd_plan_create(&probe, obs, DD_STEP_ONE, input_bits, padding, nullptr, device);
  if (st) return st;
  dd_plan_destroy(probe);
  st = dd_plan_create(&probe, obs, DD_STEP_TWO, 32, padding, nullptr, device);
  if (st) return st;
  dd_plan_destroy(probe);
  dd_subband *s = new dd_subband();
  s->device = device;
  s->obs = *obs;
  s->bits = input_bits;
  s->padding = padding;
  *pipeline = s;
  return DD_OK;
}

dd_status dd_subband_set_tables(dd_subband *s, const float *shifts, size_t n_shifts,
                                const float *shifts_step_two, size_t n_shifts2,
                                const uint32_t *zapped, size_t n_zapped,
                                const uint32_t *beam_mapping, size_t n_mapping) {
  if (!s || !shifts || !shifts_step_two || !zapped || !beam_mapping)
    return fail(DD_ERR_INVALID_ARGUMENT, "NULL argument");
  if (n_shifts < s->obs.nr_channels || n_zapped < s->obs.nr_channels ||
      n_shifts2 < s->obs.nr_subbands)
    return fail(DD_ERR_INVALID_ARGUMENT, "tables shorter than %u channels / %u subbands",
                s->obs.nr_channels, s->obs.nr_subbands);
  s->shifts.assign(shifts, shifts + n_shifts);
  s->shifts2.assign(shifts_step_two, shifts_step_two + n_shifts2);
  s->zapped.assign(zapped, zapped + n_zapped);
  s->mapping.assign(beam_mapping, beam_mapping + n_mapping);
  return build(s);
}

namespace {

// Chunked run: step two's time tiles in `chunks` ranges, each launched right
// after the step-one tiles it reads (its samples plus the largest step-two
// delay), so that the intermediate is read back while it is still in L2.
// Step one runs on a side stream one range ahead of step two: range k + 1's
// step one writes samples that range k's step two does not read.
dd_status run_chunked(dd_subband *s, const void *d_input, float *d_output, cudaStream_t stream) {
  dd::ProblemDesc P1, P2;
  dd_status st = dd::plan_problem(s->one, d_input, static_cast<float *>(s->inter), &P1, nullptr);
  if (!st) st = dd::plan_problem(s->two, s->inter, d_output, &P2, nullptr);
  uint32_t tt1 = 0, T1 = 0, md1 = 0, tt2 = 0, T2 = 0, md2 = 0;
  if (!st) st = dd::plan_time_tiles(s->one, &tt1, &T1, &md1);
  if (!st) st = dd::plan_time_tiles(s->two, &tt2, &T2, &md2);
  if (st) return st;
  const uint32_t K = std::max<uint32_t>(1, std::min<uint32_t>(s->chunks, tt2));
  DDS_CUDA(cudaSetDevice(s->device), "select device");
  if (!s->side)
    DDS_CUDA(cudaStreamCreateWithFlags(&s->side, cudaStreamNonBlocking), "create stream");
  while (s->events.size() < K + 1) {
    cudaEvent_t e = nullptr;
    DDS_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming), "create event");
    s->events.push_back(e);
  }
  // Step one of this run overwrites the intermediate the previous run's step
  // two reads: the side stream starts after the caller's stream.
  DDS_CUDA(cudaEventRecord(s->events[0], stream), "fork");
  DDS_CUDA(cudaStreamWaitEvent(s->side, s->events[0], 0), "fork");
  uint32_t done = 0;  // step-one time tiles launched
  for (uint32_t k = 0; k < K; k++) {
    const uint32_t a = (uint32_t)((uint64_t)tt2 * k / K), b = (uint32_t)((uint64_t)tt2 * (k + 1) / K);
    const uint64_t need_samples = (uint64_t)b * T2 + md2 + 1;
    const uint32_t need = k + 1 == K ? tt1
                                     : (uint32_t)std::min<uint64_t>(tt1, (need_samples + T1 - 1) / T1);
    if (need > done) {
      st = dd::plan_launch_range(s->one, P1, done, need - done, s->side);
      if (st) return st;
      done = need;
    }
    DDS_CUDA(cudaEventRecord(s->events[1 + k], s->side), "record step one");
    DDS_CUDA(cudaStreamWaitEvent(stream, s->events[1 + k], 0), "wait step one");
    st = dd::plan_launch_range(s->two, P2, a, b - a, stream);
    if (st) return st;
  }
  return DD_OK;
}

}  // namespace

dd_status dd_subband_run(dd_subband *s, const void *d_input, float *d_output, void *stream) {
  if (!s) return fail(DD_ERR_INVALID_ARGUMENT, "pipeline is NULL");
  if (!s->ready) return fail(DD_ERR_INVALID_ARGUMENT, "pipeline has no tables");
  if (s->chunks > 1) return run_chunked(s, d_input, d_output, static_cast<cudaStream_t>(stream));
  dd_status st = dd_plan_run(s->one, d_input, static_cast<float *>(s->inter), stream);
  if (!st) st = dd_plan_run(s->two, s->inter, d_output, stream);
  return st;
}

dd_status dd_subband_set_chunks(dd_subband *s, int chunks) {
  if (!s) return fail(DD_ERR_INVALID_ARGUMENT, "pipeline is NULL");
  if (chunks < 0 || chunks > 256)
    return fail(DD_ERR_INVALID_ARGUMENT, "chunks %d out of range (0..256)", chunks);
  s->chunks = (uint32_t)chunks;
  return DD_OK;
}

dd_status dd_subband_check(dd_subband *s, void *stream) {
  if (!s) return fail(DD_ERR_INVALID_ARGUMENT, "pipeline is NULL");
  if (!s->ready) return fail(DD_ERR_INVALID_ARGUMENT, "pipeline has no tables");
  dd_status st = dd_plan_check(s->one, stream);
  if (!st) st = dd_plan_check(s->two, stream);
  return st;
}

dd_status dd_subband_info(const dd_subband *s, int *packed, uint64_t *intermediate_bytes) {
  if (!s) return fail(DD_ERR_INVALID_ARGUMENT, "pipeline is NULL");
  if (!s->ready) return fail(DD_ERR_INVALID_ARGUMENT, "pipeline has no tables");
  if (packed) *packed = s->packed ? 1 : 0;
  if (intermediate_bytes) *intermediate_bytes = s->inter_bytes;
  return DD_OK;
}

dd_status dd_subband_set_pair_kernel(dd_subband *s, int index) {
  if (!s) return fail(DD_ERR_INVALID_ARGUMENT, "pipeline is NULL");
  int n = 0;
  (void)dd::pair_kernels(&n);
  if (index < 0 || index >= n)
    return fail(DD_ERR_INVALID_ARGUMENT, "pair kernel %d out of range (0..%d)", index, n - 1);
  s->pair_kernel = index;
  return s->shifts.empty() ? DD_OK : build(s);
}

dd_status dd_subband_set_overlap(dd_subband *s, int enable) {
  if (!s) return fail(DD_ERR_INVALID_ARGUMENT, "pipeline is NULL");
  s->overlap = enable != 0;
  return s->one ? dd_plan_set_overlap(s->one, enable) : DD_OK;
}

int dd_subband_pair_kernel_count(void) {
  int n = 0;
  (void)dd::pair_kernels(&n);
  return n;
}

dd_status dd_subband_destroy(dd_subband *s) {
  if (!s) return DD_OK;
  drop_plans(s);
  cudaSetDevice(s->device);
  if (s->inter) cudaFree(s->inter);
  for (cudaEvent_t e : s->events) cudaEventDestroy(e);
  if (s->side) cudaStreamDestroy(s->side);
  delete s;
  return DD_OK;
}

dd_status dd_subband_dedispersion(const dd_observation *obs, const uint32_t *zapped,
                                  const uint32_t *beam_mapping, const void *input, float *output,
                                  const float *shifts, const float *shifts_step_two,
                                  uint32_t padding, uint32_t input_bits) {
  if (!obs || !zapped || !beam_mapping || !input || !output || !shifts || !shifts_step_two)
    return fail(DD_ERR_INVALID_ARGUMENT, "NULL argument");
  dd_layout l1, l2;
  dd_status st = dd_get_layout(obs, DD_STEP_ONE, input_bits, padding, nullptr, &l1);
  if (!st) st = dd_get_layout(obs, DD_STEP_TWO, 32, padding, nullptr, &l2);
  if (st) return st;
  // One pipeline and buffers per thread, rebuilt when the geometry or a
  // table changes (repeated calls on the same observation build once).
  HostCache &c = g_host;
  const size_t n_map = (size_t)obs->nr_synthesized_beams * l2.mapping_row_elems;
  const bool same = c.pipe && c.bits == input_bits && c.padding == padding &&
                    std::memcmp(&c.obs, obs, sizeof(*obs)) == 0;
  if (!same) {
    c.reset();
    st = dd_subband_create(&c.pipe, obs, input_bits, padding, 0);
    if (st) return st;
    c.obs = *obs;
    c.bits = input_bits;
    c.padding = padding;
  }
  const bool tables = same && c.pipe->shifts.size() == l1.shifts_elems &&
                      std::memcmp(c.pipe->shifts.data(), shifts, l1.shifts_elems * 4) == 0 &&
                      c.pipe->shifts2.size() == l2.shifts_elems &&
                      std::memcmp(c.pipe->shifts2.data(), shifts_step_two, l2.shifts_elems * 4) == 0 &&
                      c.pipe->zapped.size() == l1.zapped_elems &&
                      std::memcmp(c.pipe->zapped.data(), zapped, l1.zapped_elems * 4) == 0 &&
                      c.pipe->mapping.size() == n_map &&
                      std::memcmp(c.pipe->mapping.data(), beam_mapping, n_map * 4) == 0;
  if (!tables) {
    st = dd_subband_set_tables(c.pipe, shifts, l1.shifts_elems, shifts_step_two, l2.shifts_elems,
                               zapped, l1.zapped_elems, beam_mapping, n_map);
    if (st) return st;
  }
  DDS_CUDA(cudaSetDevice(0), "select device");
  if (!c.stream) DDS_CUDA(cudaStreamCreateWithFlags(&c.stream, cudaStreamNonBlocking), "create stream");
  if (l1.input_bytes > c.cap_in) {
    if (c.d_in) cudaFree(c.d_in);
    c.d_in = nullptr;
    c.cap_in = 0;
    DDS_CUDA(cudaMalloc(&c.d_in, std::max<uint64_t>(l1.input_bytes, 16)), "allocate input");
    c.cap_in = l1.input_bytes;
  }
  if (l2.output_bytes > c.cap_out) {
    if (c.d_out) cudaFree(c.d_out);
    c.d_out = nullptr;
    c.cap_out = 0;
    DDS_CUDA(cudaMalloc(&c.d_out, std::max<uint64_t>(l2.output_bytes, 16)), "allocate output");
    c.cap_out = l2.output_bytes;
  }
  DDS_CUDA(cudaMemcpyAsync(c.d_in, input, l1.input_bytes, cudaMemcpyHostToDevice, c.stream),
           "copy input");
  DDS_CUDA(cudaMemsetAsync(c.d_out, 0, l2.output_bytes, c.stream), "clear output");
  st = dd_subband_run(c.pipe, c.d_in, static_cast<float *>(c.d_out), c.stream);
  if (st) return st;
  DDS_CUDA(cudaMemcpyAsync(output, c.d_out, l2.output_bytes, cudaMemcpyDeviceToHost, c.stream),
           "copy output");
  return dd_subband_check(c.pipe, c.stream);
}

}  // extern "C"
