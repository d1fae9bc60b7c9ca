// dd_api.cu -- host side of the C ABI (include/dedisp_gb300.h).
//
// Geometry and delay tables are computed on the host in the reference's float
// expression order (src/Shifts.cpp:20-42); plans turn an observation, a mode
// and the host tables (shifts, zapped mask, beam mapping) into the group and
// entry descriptors the kernels read (dd_internal.h), pick a compiled tile
// configuration, and launch it on the caller's stream.  There is no CPU path.
#include <cuda_runtime.h>

#include <algorithm>
#include <cctype>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/dedisp_gb300.h"
#include "dd_internal.h"
#include "dd_shared.cuh"
#include "dd_shared_plan.h"
#include "dd_tmem.cuh"

namespace {

thread_local std::string g_error;

dd_status fail(dd_status code, const char *fmt, ...) {
  char buf[1024];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_error = buf;
  return code;
}

dd_status cuda_fail(cudaError_t e, const char *what) {
  (void)cudaGetLastError();
  if (e == cudaErrorMemoryAllocation)
    return fail(DD_ERR_OUT_OF_MEMORY, "%s: %s", what, cudaGetErrorString(e));
  if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver)
    return fail(DD_ERR_NO_DEVICE, "%s: %s", what, cudaGetErrorString(e));
  return fail(DD_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

#define DD_CUDA(call, what)                       \
  do {                                            \
    cudaError_t e_ = (call);                      \
    if (e_ != cudaSuccess) return cuda_fail(e_, what); \
  } while (0)

bool bits_ok(uint32_t bits) {
  return bits == 1 || bits == 2 || bits == 4 || bits == 8 || bits == 16 ||
         bits == 32;
}

uint64_t pad(uint64_t v, uint64_t p) { return p == 0 ? v : (v + p - 1) / p * p; }

// AstroData::Observation frequency getters.  The subband frequency is that
// of the subband's highest channel, the channel step one dedisperses each
// subband to (include/Dedispersion.hpp:124).
float max_freq(const dd_observation *o) {
  volatile float span = (o->nr_channels - 1) * o->channel_bandwidth;
  return o->min_freq + span;
}
float subband_bandwidth(const dd_observation *o) {
  return (o->nr_channels / o->nr_subbands) * o->channel_bandwidth;
}
float subband_min_freq(const dd_observation *o) {
  volatile float span = ((o->nr_channels / o->nr_subbands) - 1) * o->channel_bandwidth;
  return o->min_freq + span;
}
float subband_max_freq(const dd_observation *o) {
  volatile float span = (o->nr_subbands - 1) * subband_bandwidth(o);
  return subband_min_freq(o) + span;
}

// src/Shifts.cpp:20-42, one table: frequencies f0 + k * step for k < n - 1,
// reference frequency fmax, last entry 0.
void shift_table(const dd_observation *o, float f0, float step, float fmax,
                 uint32_t n, float *out) {
  float inverseHighFreq = 1.0f / std::pow(fmax, 2.0f);
  float timeUnit = o->nr_samples_per_batch * o->sampling_time;
  for (uint32_t k = 0; k + 1 < n; k++) {
    volatile float offset = k * step;
    float inverseFreq = 1.0f / std::pow(f0 + offset, 2.0f);
    volatile float a = 4148.808f * (inverseFreq - inverseHighFreq);
    volatile float b = a * (o->nr_samples_per_batch / o->downsampling);
    out[k] = b / timeUnit;
  }
  out[n - 1] = 0;
}

uint64_t row_bytes_of(uint32_t samples, uint32_t bits, uint32_t padding) {
  if (bits < 8) {
    uint32_t per = 8 / bits;
    return pad((samples + per - 1) / per, padding);
  }
  uint32_t eb = bits / 8;
  return pad(samples, padding / eb) * eb;
}

dd_status check_obs(const dd_observation *o, dd_mode mode) {
  if (!o) return fail(DD_ERR_INVALID_ARGUMENT, "observation is NULL");
  if (o->downsampling != 1)
    return fail(DD_ERR_UNSUPPORTED, "downsampling must be 1 (got %u)", o->downsampling);
  if (o->nr_channels == 0) return fail(DD_ERR_INVALID_ARGUMENT, "nr_channels is 0");
  if (mode != DD_SINGLE_STEP && (o->nr_subbands == 0 || o->nr_subbands > o->nr_channels))
    return fail(DD_ERR_INVALID_ARGUMENT, "nr_subbands must be in 1..nr_channels");
  if (!(o->first_dm >= 0.0f) || !(o->dm_step >= 0.0f) ||
      !(o->first_dm_subbanding >= 0.0f) || !(o->dm_step_subbanding >= 0.0f))
    return fail(DD_ERR_INVALID_ARGUMENT, "DM first/step must be non-negative");
  if (mode < DD_SINGLE_STEP || mode > DD_STEP_TWO)
    return fail(DD_ERR_INVALID_ARGUMENT, "unknown mode %d", (int)mode);
  return DD_OK;
}

// Per-mode dimensions.
struct Dims {
  uint32_t nr_dms, nr_samples, row_samples;
  float first_dm, dm_step;
  uint64_t row_bytes, out_row, input_bytes, output_rows;
  uint64_t mapping_row, zapped_elems, shift_elems;
};

Dims dims_of(const dd_observation *o, dd_mode mode, uint32_t bits, uint32_t padding) {
  Dims d{};
  const uint64_t C = o->nr_channels;
  if (mode == DD_SINGLE_STEP) {
    d.nr_dms = o->nr_dms; d.nr_samples = o->nr_samples_per_batch;
    d.row_samples = o->nr_samples_per_dispersed_batch;
    d.first_dm = o->first_dm; d.dm_step = o->dm_step;
    d.row_bytes = row_bytes_of(d.row_samples, bits, padding);
    d.out_row = pad(d.nr_samples, padding / 4);
    d.input_bytes = o->nr_beams * C * d.row_bytes;
    d.output_rows = (uint64_t)o->nr_synthesized_beams * o->nr_dms;
    d.mapping_row = pad(C, padding / 4);
    d.zapped_elems = pad(C, padding / 4);
    d.shift_elems = pad(C, padding / 4);
  } else if (mode == DD_STEP_ONE) {
    d.nr_dms = o->nr_dms_subbanding; d.nr_samples = o->nr_samples_per_batch_subbanding;
    d.row_samples = o->nr_samples_per_dispersed_batch_subbanding;
    d.first_dm = o->first_dm_subbanding; d.dm_step = o->dm_step_subbanding;
    d.row_bytes = row_bytes_of(d.row_samples, bits, padding);
    d.out_row = pad(d.nr_samples, padding / 4);
    d.input_bytes = o->nr_beams * C * d.row_bytes;
    d.output_rows = (uint64_t)o->nr_beams * o->nr_dms_subbanding * o->nr_subbands;
    d.mapping_row = 0;
    d.zapped_elems = pad(C, padding / 4);
    d.shift_elems = pad(C, padding / 4);
  } else {
    d.nr_dms = o->nr_dms; d.nr_samples = o->nr_samples_per_batch;
    d.row_samples = o->nr_samples_per_batch_subbanding;
    d.first_dm = o->first_dm; d.dm_step = o->dm_step;
    d.row_bytes = pad(d.row_samples, padding / 4) * 4;
    d.out_row = pad(d.nr_samples, padding / 4);
    d.input_bytes = (uint64_t)o->nr_beams * o->nr_dms_subbanding * o->nr_subbands * d.row_bytes;
    d.output_rows = (uint64_t)o->nr_synthesized_beams * o->nr_dms_subbanding * o->nr_dms;
    d.mapping_row = pad(o->nr_subbands, padding / 4);
    d.zapped_elems = 0;
    d.shift_elems = pad(o->nr_subbands, padding / 4);
  }
  return d;
}

uint32_t family_bits(dd_mode mode, uint32_t bits) {
  if (mode == DD_STEP_TWO) return 32;
  return bits <= 8 ? 8 : bits;
}

const dd::KernelInfo *find_kernel(dd_mode mode, uint32_t bits, const dd_conf &c) {
  int n = 0;
  const dd::KernelInfo *reg = dd::kernel_registry(&n);
  const uint32_t fb = family_bits(mode, bits);
  for (int i = 0; i < n; i++) {
    const dd::KernelInfo &k = reg[i];
    if ((uint32_t)k.elem_bits != fb) continue;
    if (c.threads_d0 != 32u || c.threads_d1 != (uint32_t)k.warps_d) continue;
    if (c.items_d0 != (uint32_t)k.items_t || c.items_d1 != (uint32_t)k.items_d) continue;
    if (c.unroll != (uint32_t)k.channels) continue;
    // items_d2 = rows per shared partial sum marks the shared family, 2 the
    // short-group swar8 tiles.
    const bool shared = c.items_d2 == (uint32_t)dd::kSharedRows;
    if (shared != (k.family == dd::kFamilyShared8)) continue;
    // items_d2 = 3 marks the TMEM-window tile.
    const bool tmem = c.items_d2 == 3u;
    if (tmem != (k.family == dd::kFamilyTmem32)) continue;
    if ((c.items_d2 == 2u) != (k.max_rows != 0)) continue;
    if ((shared || tmem) && mode != DD_SINGLE_STEP) continue;
    return &k;
  }
  return nullptr;
}

// The default configuration of a mode and input width: the first registry
// entry of its family; for single-step input of 1-8 bits the first
// shared-partial-sum entry when `shared` (plans fall back to the direct
// entry where a shape does not fit the shared tables).
// Default tiles of the subband steps, where they differ from the first entry
// of their input width (fastest of a sweep of every registry entry at 1536
// channels, 32 subbands, 64 x 32 DMs, 24576 samples: step one's 64 coarse
// DMs favour 8 DMs per thread and, with 48 rows per subband, the short-group
// tile; step two's 32 subband rows 8 x 8 items).  A step-one shape whose
// subbands have more than 257 rows falls back to the other direct tiles.
const char *subband_default_name(dd_mode mode, uint32_t fb) {
  if (mode == DD_STEP_ONE && fb == 8) return "swar8s_i4_d8_w8_c8_vkUnpackPermuteMad";
  if (mode == DD_STEP_TWO) return "scalar32_i8_d8_w4_c16";
  return nullptr;
}

const dd::KernelInfo *default_kernel(dd_mode mode, uint32_t bits, bool shared) {
  int n = 0;
  const dd::KernelInfo *reg = dd::kernel_registry(&n);
  const uint32_t fb = family_bits(mode, bits);
  if (const char *name = subband_default_name(mode, fb))
    for (int i = 0; i < n; i++)
      if (std::strcmp(reg[i].name, name) == 0) return &reg[i];
  // `shared`: the preferred tile of plans without a configuration -- shared
  // partial sums for 1-8-bit single-step input, TMEM windows for float.
  const bool want_shared = shared && mode == DD_SINGLE_STEP && bits <= 8;
  const bool want_tmem = shared && mode == DD_SINGLE_STEP && bits == 32;
  for (int i = 0; i < n; i++)
    if ((uint32_t)reg[i].elem_bits == fb &&
        (reg[i].family == dd::kFamilyShared8) == want_shared &&
        (reg[i].family == dd::kFamilyTmem32) == want_tmem)
      return &reg[i];
  return nullptr;
}

dd_conf conf_of(const dd::KernelInfo &k) {
  dd_conf c{};
  c.split_batches = 0; c.local_mem = 1; c.unroll = k.channels;
  c.threads_d0 = 32; c.threads_d1 = k.warps_d; c.threads_d2 = 1;
  c.items_d0 = k.items_t; c.items_d1 = k.items_d;
  c.items_d2 = k.family == dd::kFamilyShared8  ? dd::kSharedRows
               : k.family == dd::kFamilyTmem32 ? 3
                                               : (k.max_rows ? 2 : 1);
  return c;
}

dd_status device_ok() {
  int n = 0;
  cudaError_t e = cudaGetDeviceCount(&n);
  if (e != cudaSuccess || n == 0) {
    (void)cudaGetLastError();
    return fail(DD_ERR_NO_DEVICE, "no CUDA device available (%s)",
                e == cudaSuccess ? "0 devices" : cudaGetErrorString(e));
  }
  return DD_OK;
}

// Restores the caller's current device on scope exit.
struct DeviceGuard {
  int prev = -1;
  bool ok = false;
  explicit DeviceGuard(int dev) {
    if (cudaGetDevice(&prev) != cudaSuccess) { (void)cudaGetLastError(); prev = -1; }
    ok = cudaSetDevice(dev) == cudaSuccess;
    if (!ok) (void)cudaGetLastError();
  }
  ~DeviceGuard() { if (prev >= 0) cudaSetDevice(prev); }
};

}  // namespace

struct dd_plan {
  int device = 0;
  dd_observation obs{};
  dd_mode mode = DD_SINGLE_STEP;
  uint32_t bits = 8, padding = 0;
  const dd::KernelInfo *kinfo = nullptr;
  Dims dims{};
  std::vector<float> shifts;
  std::vector<uint32_t> zapped, mapping;
  bool have_shifts = false;
  // derived
  uint32_t nr_groups = 0, tiles_t = 0, tiles_d = 0, win = 0;
  size_t smem = 0;
  uint64_t out_dm_stride = 0;
  std::vector<dd::GroupDesc> groups;
  std::vector<dd::EntryDesc> entries;
  dd::GroupDesc *d_groups = nullptr;
  dd::EntryDesc *d_entries = nullptr;
  size_t cap_groups = 0, cap_entries = 0;
  uint32_t *d_status = nullptr;
  // TMEM-window tile offsets (ProblemDesc::tmem_tab).
  std::vector<uint32_t> tmem_tab;
  uint32_t *d_tmem_tab = nullptr;
  size_t cap_tmem_tab = 0;
  // Precomputed delays (ProblemDesc::delay_base / delay_rel).
  std::vector<float> delay_shift;  // delay per unit DM of each delay row
  std::vector<uint16_t> delay_rel;
  uint16_t *d_delay_rel = nullptr;
  size_t cap_delay_rel = 0;
  bool use_delay_tables = false;
  // Shared-partial-sum tables (kFamilyShared8 only).
  dd::SharedTables shared;
  std::vector<uint4> stage_rows;  // [group][stage][32] row slots
  uint4 *d_stage_rows = nullptr;
  uint32_t *d_tile_stage = nullptr;
  uint16_t *d_pool = nullptr;
  size_t cap_stage_rows = 0, cap_tile_stage = 0, cap_pool = 0;
  std::string invalid;  // why the tables are not usable (empty when ready)
  bool ready = false;
  // Created without a configuration: a shape that the default shared kernel
  // cannot take runs on the default direct kernel instead.
  bool auto_kernel = false;
  // Tables changed since the last build: setters only record their table;
  // the first use (run, timing, queries) builds once.
  bool dirty = false;
  // Packed subband intermediate (ProblemDesc::packed): step one writes it,
  // step two (a pair tile) reads it; set by a subband pipeline only.
  bool packed = false;
  uint32_t flush_rows = 0;  // step two: rows per 16-bit lane flush
  uint32_t max_delay = 0;   // largest row delay of the built tables
  bool overlap = false;     // dd_plan_set_overlap
  // A kernel reading the device tables was enqueued since they were last
  // uploaded: the next upload first waits for the device (the run may still
  // be in flight on a non-blocking stream, which the synchronous upload
  // copies do not order against).
  mutable bool launched = false;
  uint32_t wait_ns = 0;     // dd_plan_set_wait_limit (0: the kernels' default)
};

namespace {

// Build the group/entry tables, the window size and upload them.
dd_status rebuild(dd_plan *p) {
  p->ready = false;
  if (!p->have_shifts) return DD_OK;
  const dd_observation *o = &p->obs;
  const Dims &d = p->dims;
  const uint32_t C = o->nr_channels;
  p->groups.clear();
  p->entries.clear();
  p->delay_shift.clear();
  auto zapped = [&](uint32_t c) { return !p->zapped.empty() && p->zapped[c] != 0; };
  // Entries of a group take consecutive delay rows; groups with the same
  // delays per unit DM share rows.
  if (p->mode == DD_SINGLE_STEP) {
    p->nr_groups = o->nr_synthesized_beams;
    p->out_dm_stride = d.out_row;
    for (uint32_t c = 0; c < C; c++)
      if (!zapped(c)) p->delay_shift.push_back(p->shifts[c]);
    for (uint32_t g = 0; g < p->nr_groups; g++) {
      dd::GroupDesc G{(uint32_t)p->entries.size(), 0, (uint64_t)g * d.nr_dms * d.out_row};
      uint32_t row = 0;
      for (uint32_t c = 0; c < C; c++) {
        if (zapped(c)) continue;
        uint64_t beam = p->mapping.empty() ? (o->nr_beams ? g % o->nr_beams : 0)
                                           : p->mapping[(uint64_t)g * d.mapping_row + c];
        if (beam >= o->nr_beams)
          return fail(DD_ERR_INVALID_ARGUMENT, "beam mapping[%u][%u] = %llu >= nr_beams %u",
                      g, c, (unsigned long long)beam, o->nr_beams);
        p->entries.push_back({(beam * C + c) * d.row_bytes, p->shifts[c], row++});
      }
      G.entry_count = (uint32_t)p->entries.size() - G.entry_begin;
      p->groups.push_back(G);
    }
  } else if (p->mode == DD_STEP_ONE) {
    const uint32_t SB = o->nr_subbands, cps = C / SB;
    // Packed: rows (beam, coarse DM pair, subband) of 32-bit words.
    const uint64_t dm_rows = p->packed ? (d.nr_dms + 1) / 2 : d.nr_dms;
    p->nr_groups = o->nr_beams * SB;
    p->out_dm_stride = (uint64_t)SB * d.out_row;
    std::vector<uint32_t> sb_row(SB);
    for (uint32_t sb = 0; sb < SB; sb++) {
      sb_row[sb] = (uint32_t)p->delay_shift.size();
      const float last = p->shifts[(sb + 1) * cps - 1];
      for (uint32_t c = sb * cps; c < (sb + 1) * cps; c++) {
        if (zapped(c)) continue;
        volatile float rel = p->shifts[c] - last;
        p->delay_shift.push_back(static_cast<float>(rel));
      }
    }
    for (uint32_t b = 0; b < o->nr_beams; b++)
      for (uint32_t sb = 0; sb < SB; sb++) {
        dd::GroupDesc G{(uint32_t)p->entries.size(), 0,
                        ((uint64_t)b * dm_rows * SB + sb) * d.out_row};
        uint32_t row = sb_row[sb];
        for (uint32_t c = sb * cps; c < (sb + 1) * cps; c++) {
          if (zapped(c)) continue;
          p->entries.push_back({((uint64_t)b * C + c) * d.row_bytes, p->delay_shift[row], row});
          row++;
        }
        G.entry_count = (uint32_t)p->entries.size() - G.entry_begin;
        p->groups.push_back(G);
      }
  } else {
    const uint32_t SB = o->nr_subbands, D1 = o->nr_dms_subbanding;
    // Packed: one group per pair of coarse DMs, reading the pair's rows.
    const uint32_t G1 = p->packed ? (D1 + 1) / 2 : D1;
    p->nr_groups = o->nr_synthesized_beams * G1;
    p->out_dm_stride = d.out_row;
    for (uint32_t sb = 0; sb < SB; sb++) p->delay_shift.push_back(p->shifts[sb]);
    for (uint32_t g = 0; g < o->nr_synthesized_beams; g++)
      for (uint32_t d1 = 0; d1 < G1; d1++) {
        const uint64_t first = p->packed ? 2ull * d1 : d1;  // coarse DM of the lanes' low half
        dd::GroupDesc G{(uint32_t)p->entries.size(), SB,
                        ((uint64_t)g * D1 * d.nr_dms + first * d.nr_dms) * d.out_row};
        for (uint32_t s = 0; s < SB; s++) {
          uint64_t beam = p->mapping.empty() ? (o->nr_beams ? g % o->nr_beams : 0)
                                             : p->mapping[(uint64_t)g * d.mapping_row + s];
          if (beam >= o->nr_beams)
            return fail(DD_ERR_INVALID_ARGUMENT, "beam mapping[%u][%u] = %llu >= nr_beams %u",
                        g, s, (unsigned long long)beam, o->nr_beams);
          p->entries.push_back({((beam * G1 + d1) * SB + s) * d.row_bytes, p->shifts[s], s});
        }
        p->groups.push_back(G);
      }
  }
  // Largest delay must stay inside the rows; window spread per DM tile.
  const dd::KernelInfo &k = *p->kinfo;
  std::vector<float> uniq;
  uniq.reserve(p->entries.size());
  for (auto &e : p->entries) uniq.push_back(e.shift);
  std::sort(uniq.begin(), uniq.end());
  uniq.erase(std::unique(uniq.begin(), uniq.end()), uniq.end());
  uint32_t max_delay = 0, spread = 0;
  p->tiles_d = d.nr_dms ? (d.nr_dms + k.tile_d - 1) / k.tile_d : 0;
  p->tiles_t = d.nr_samples ? (d.nr_samples + k.tile_t - 1) / k.tile_t : 0;
  for (float sh : uniq) {
    if (!(sh >= 0.0f) || !std::isfinite(sh))
      return fail(DD_ERR_INVALID_ARGUMENT, "delay per unit DM must be finite and >= 0 (got %g)", sh);
    if (d.nr_dms == 0) break;
    max_delay = std::max(max_delay, dd::host_delay(d.first_dm, d.dm_step, d.nr_dms - 1, sh));
    for (uint32_t t = 0; t < p->tiles_d; t++) {
      uint32_t d0 = t * k.tile_d, d1 = std::min(d0 + k.tile_d, d.nr_dms) - 1;
      uint32_t sp = dd::host_delay(d.first_dm, d.dm_step, d1, sh) -
                    dd::host_delay(d.first_dm, d.dm_step, d0, sh);
      spread = std::max(spread, sp);
    }
  }
  if (d.nr_dms && d.nr_samples && (uint64_t)d.nr_samples + max_delay > d.row_samples)
    return fail(DD_ERR_INVALID_ARGUMENT,
                "rows hold %u samples but %u output samples + max delay %u are needed",
                d.row_samples, d.nr_samples, max_delay);
  p->max_delay = max_delay;
  int dev_max = 0, sm_max = 0;
  {
    DeviceGuard g(p->device);
    DD_CUDA(cudaDeviceGetAttribute(&dev_max, cudaDevAttrMaxSharedMemoryPerBlockOptin, p->device),
            "query shared memory");
    DD_CUDA(cudaDeviceGetAttribute(&sm_max, cudaDevAttrMaxSharedMemoryPerMultiprocessor,
                                   p->device), "query shared memory");
  }
  const bool shared = k.family == dd::kFamilyShared8;
  if (k.max_rows)
    for (const dd::GroupDesc &G : p->groups)
      if (G.entry_count > (uint32_t)k.max_rows)
        return fail(DD_ERR_UNSUPPORTED, "tile %s takes groups of at most %d rows (a group has %u)",
                    k.name, k.max_rows, G.entry_count);
  if (p->packed && p->mode == DD_STEP_ONE) {
    if (k.family != dd::kFamilySwar8 || k.items_d % 2)
      return fail(DD_ERR_UNSUPPORTED, "a packed step one runs a swar8 tile (got %s)", k.name);
    const uint32_t SB = o->nr_subbands, cps = C / SB;
    uint32_t live_max = 0;
    for (uint32_t sb = 0; sb < SB; sb++) {
      uint32_t live = 0;
      for (uint32_t c = sb * cps; c < (sb + 1) * cps; c++) live += zapped(c) ? 0u : 1u;
      live_max = std::max(live_max, live);
    }
    if ((uint64_t)live_max * ((1u << p->bits) - 1u) > 0xFFFFu)
      return fail(DD_ERR_UNSUPPORTED,
                  "%u live channels of %u-bit input per subband can exceed 16-bit sums",
                  live_max, p->bits);
  } else if (p->packed && p->mode == DD_STEP_TWO) {
    if (k.family != dd::kFamilyPair16 || p->flush_rows == 0)
      return fail(DD_ERR_UNSUPPORTED, "a packed step two runs a pair tile");
  } else if (k.family == dd::kFamilyPair16) {
    return fail(DD_ERR_UNSUPPORTED, "pair tiles read a packed step-one intermediate only");
  }
  const bool tmem = k.family == dd::kFamilyTmem32;
  uint32_t rows_max = 0;
  for (const dd::GroupDesc &G : p->groups) rows_max = std::max(rows_max, G.entry_count);
  if (tmem) {
    if (p->mode != DD_SINGLE_STEP || p->bits != 32)
      return fail(DD_ERR_UNSUPPORTED, "kernel %s computes single-step float input only", k.name);
    if (dd::tmem_smem_bytes(rows_max) > (size_t)dev_max)
      return fail(DD_ERR_UNSUPPORTED, "tile %s holds the rows of a group in shared memory "
                  "(%u rows need %zu bytes, device allows %d)",
                  k.name, rows_max, dd::tmem_smem_bytes(rows_max), dev_max);
    if (d.input_bytes / 16 > 0xFFFFFFFFull)
      return fail(DD_ERR_UNSUPPORTED, "tile %s addresses rows in 16-byte units of 32 bits",
                  k.name);
    if (!dd::tmem_fits(uniq.data(), uniq.size(), d.first_dm, d.dm_step, d.nr_dms))
      return fail(DD_ERR_UNSUPPORTED, "tile %s: 16 DMs spread a row's delay by more than %u "
                  "samples", k.name, dd::kTmMaxOff - 3u);
    dd::tmem_tables(p->delay_shift, d.first_dm, d.dm_step, d.nr_dms, &p->tmem_tab);
  }
  if (shared) {
    if (p->mode != DD_SINGLE_STEP || p->bits > 8)
      return fail(DD_ERR_UNSUPPORTED, "kernel %s computes single-step 1/2/4/8-bit input only",
                  k.name);
    // One CTA per SM: the whole opt-in shared memory of a block.
    const size_t budget = (size_t)dev_max;
    (void)sm_max;
    const std::string why = dd::build_shared_tables(k, p->delay_shift, d.first_dm, d.dm_step,
                                                    d.nr_dms, p->bits, budget, &p->shared);
    if (!why.empty()) return fail(DD_ERR_UNSUPPORTED, "tile %s: %s", k.name, why.c_str());
  }
  const uint32_t bits = family_bits(p->mode, p->bits) == 8 ? p->bits : family_bits(p->mode, p->bits);
  const uint32_t a = dd::window_alignment_samples(bits);
  p->win = shared ? 0 : tmem ? rows_max : ((k.tile_t + spread + a + 8) + 15) / 16 * 16;
  p->smem = shared ? p->shared.smem : dd::kernel_smem_bytes(k, p->win, bits);
  if (p->smem > (size_t)dev_max)
    return fail(DD_ERR_UNSUPPORTED,
                "tile %s needs %zu bytes of shared memory (window %u samples), device allows %d; "
                "use a configuration with fewer DMs per tile",
                k.name, p->smem, p->win, dev_max);
  // Delay table: the offsets of each DM tile's delays from the delay of its
  // first DM, per delay row (the same float order as the device's
  // dev_delay).  16-bit offsets: skipped if a spread does not fit.
  const size_t rows = p->delay_shift.size();
  p->use_delay_tables = !shared && !tmem && spread < 65536 && rows > 0 && p->tiles_d > 0;
  if (p->use_delay_tables) {
    p->delay_rel.assign((size_t)p->tiles_d * rows * k.tile_d, 0);
    // DM values in the reference's order (firstDM + dm * dmStep, each op
    // rounded to float: this file is compiled with -ffp-contract=off), then
    // one product and truncation per entry; equal to dd::host_delay.
    std::vector<float> dm_value((size_t)p->tiles_d * k.tile_d);
    for (size_t i = 0; i < dm_value.size(); i++) {
      const uint32_t dm = std::min((uint32_t)i, d.nr_dms - 1);
      const float step_dm = static_cast<float>(dm) * d.dm_step;
      dm_value[i] = d.first_dm + step_dm;
    }
    for (uint32_t t = 0; t < p->tiles_d; t++) {
      const float *dv = &dm_value[(size_t)t * k.tile_d];
      for (size_t r = 0; r < rows; r++) {
        const float sh = p->delay_shift[r];
        const uint32_t base = static_cast<uint32_t>(dv[0] * sh);
        uint16_t *rel = &p->delay_rel[((size_t)t * rows + r) * k.tile_d];
        for (int j = 0; j < k.tile_d; j++)
          rel[j] = (uint16_t)(static_cast<uint32_t>(dv[j] * sh) - base);
      }
    }
  }
  // Upload.
  DeviceGuard g(p->device);
  if (p->launched) {
    DD_CUDA(cudaDeviceSynchronize(), "wait for runs reading the old tables");
    p->launched = false;
  }
  if (p->groups.size() > p->cap_groups) {
    if (p->d_groups) cudaFree(p->d_groups);
    p->d_groups = nullptr;
    DD_CUDA(cudaMalloc(&p->d_groups, std::max<size_t>(1, p->groups.size()) * sizeof(dd::GroupDesc)),
            "allocate group table");
    p->cap_groups = p->groups.size();
  }
  if (p->entries.size() > p->cap_entries || !p->d_entries) {
    if (p->d_entries) cudaFree(p->d_entries);
    p->d_entries = nullptr;
    DD_CUDA(cudaMalloc(&p->d_entries, std::max<size_t>(1, p->entries.size()) * sizeof(dd::EntryDesc)),
            "allocate entry table");
    p->cap_entries = std::max<size_t>(1, p->entries.size());
  }
  if (!p->groups.empty())
    DD_CUDA(cudaMemcpy(p->d_groups, p->groups.data(), p->groups.size() * sizeof(dd::GroupDesc),
                       cudaMemcpyHostToDevice), "upload group table");
  if (!p->entries.empty())
    DD_CUDA(cudaMemcpy(p->d_entries, p->entries.data(), p->entries.size() * sizeof(dd::EntryDesc),
                       cudaMemcpyHostToDevice), "upload entry table");
  if (tmem) {
    if (p->tmem_tab.size() > p->cap_tmem_tab || !p->d_tmem_tab) {
      if (p->d_tmem_tab) cudaFree(p->d_tmem_tab);
      p->d_tmem_tab = nullptr;
      DD_CUDA(cudaMalloc(&p->d_tmem_tab, std::max<size_t>(1, p->tmem_tab.size()) * sizeof(uint32_t)),
              "allocate TMEM tile offsets");
      p->cap_tmem_tab = std::max<size_t>(1, p->tmem_tab.size());
    }
    if (!p->tmem_tab.empty())
      DD_CUDA(cudaMemcpy(p->d_tmem_tab, p->tmem_tab.data(), p->tmem_tab.size() * sizeof(uint32_t),
                         cudaMemcpyHostToDevice), "upload TMEM tile offsets");
  }
  if (p->use_delay_tables) {
    if (p->delay_rel.size() > p->cap_delay_rel) {
      if (p->d_delay_rel) cudaFree(p->d_delay_rel);
    if (p->d_tmem_tab) cudaFree(p->d_tmem_tab);
      p->d_delay_rel = nullptr;
      DD_CUDA(cudaMalloc(&p->d_delay_rel, p->delay_rel.size() * sizeof(uint16_t)),
              "allocate delay table");
      p->cap_delay_rel = p->delay_rel.size();
    }
    DD_CUDA(cudaMemcpy(p->d_delay_rel, p->delay_rel.data(),
                       p->delay_rel.size() * sizeof(uint16_t), cudaMemcpyHostToDevice),
            "upload delay table");
  }
  if (shared) {
    auto upload = [&](auto **dptr, size_t *cap, const auto &v, const char *what) -> dd_status {
      using T = typename std::decay<decltype(v)>::type::value_type;
      const size_t n = std::max<size_t>(1, v.size());
      if (n > *cap || !*dptr) {
        if (*dptr) cudaFree(*dptr);
        *dptr = nullptr;
        DD_CUDA(cudaMalloc(reinterpret_cast<void **>(dptr), n * sizeof(T)), what);
        *cap = n;
      }
      if (!v.empty())
        DD_CUDA(cudaMemcpy(*dptr, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice), what);
      return DD_OK;
    };
    // Row slots of every stage for every group: the row's byte offset, its
    // subgroup's window start, the stage table's pool index.
    const std::vector<dd::SharedStage> &sts = p->shared.stages;
    p->stage_rows.assign((size_t)p->nr_groups * sts.size() * dd::kStageRows, uint4{0, 0, 0, 0});
    for (uint32_t gi = 0; gi < p->nr_groups; gi++)
      for (size_t si = 0; si < sts.size(); si++) {
        uint4 *slot = &p->stage_rows[((size_t)gi * sts.size() + si) * dd::kStageRows];
        for (uint32_t r = 0; r < (uint32_t)dd::kStageRows; r++) {
          slot[r].w = sts[si].pool;
          if (r >= sts[si].nrows) continue;
          const uint64_t off =
              p->entries[p->groups[gi].entry_begin + sts[si].row_first + r].row_offset;
          slot[r].x = (uint32_t)(off & 0xFFFFFFFFu);
          slot[r].y = (uint32_t)(off >> 32);
          slot[r].z = sts[si].bmin[sts[si].row_sub[r]] | dd::kRowPresent;
        }
      }
    dd_status us = upload(&p->d_stage_rows, &p->cap_stage_rows, p->stage_rows,
                          "upload stage rows");
    if (!us) us = upload(&p->d_tile_stage, &p->cap_tile_stage, p->shared.tile_stage,
                         "upload tile stage table");
    if (!us) us = upload(&p->d_pool, &p->cap_pool, p->shared.pool, "upload stage pool");
    if (us) return us;
  }
  // The attribute is a cap shared by every plan of this kernel: set it to the
  // device maximum (less the kernel's static shared memory) so that no plan
  // lowers it below another plan's need.
  cudaFuncAttributes fa{};
  DD_CUDA(cudaFuncGetAttributes(&fa, k.func), "query kernel attributes");
  if (p->smem + fa.sharedSizeBytes > (size_t)dev_max)
    return fail(DD_ERR_UNSUPPORTED, "tile %s needs %zu + %zu bytes of shared memory, device "
                "allows %d", k.name, p->smem, (size_t)fa.sharedSizeBytes, dev_max);
  DD_CUDA(cudaFuncSetAttribute(k.func, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               dev_max - (int)fa.sharedSizeBytes),
          "set kernel shared memory");
  p->ready = true;
  return DD_OK;
}

// rebuild(), and for plans created without a configuration: the default
// shared kernel while it saves enough adds (shared_worth_it), else the
// default direct kernel.  Where a tile does not fit (its tables or window
// outgrow shared memory): the direct default, then the other direct tiles of
// the same width, largest (samples x DMs x rows per stage) first.
// The shared-partial-sum tile pays for its stage machinery (row expansion,
// chains, barriers) per executed add; the direct tile does one packed add
// per direct-sum add.  Timed on the 40 uneven beams of the batched
// benchmark (384 and 1536 channels, 2/4/8-bit, DM steps 0.1-0.47): the
// shared tile is faster while its executed adds stay below ~0.34 of the
// direct sum (ratios 0.20-0.33: 0.46-0.90 of the direct time) and slower
// above (0.35-0.48: 1.02-2.12 of it).
constexpr double kSharedMaxAddsRatio = 0.34;

bool shared_worth_it(const dd_plan *p) {
  const uint64_t rows = p->nr_groups ? p->entries.size() / p->nr_groups : 0;
  const double direct = (double)rows * p->obs.nr_dms * p->kinfo->tile_t;
  const double shared = (double)(p->shared.adds_partial + p->shared.adds_series);
  return direct <= 0 || shared <= kSharedMaxAddsRatio * direct;
}

// The default direct tile has 8 warps and budgets two CTAs per SM.  Where a
// shape's window leaves room for only one (wide DM spreads of 8-bit rows:
// its staged rows and their four shifted copies grow with the spread), the
// SM would hold 8 warps; the 16-warp tile of the same samples per thread
// keeps 16.  Measured on 384-channel 8-bit beams with DM steps of 0.42-0.46:
// 0.334 against 0.429 ms and 0.997 against 1.525 ms.
void prefer_occupancy(dd_plan *p) {
  if (p->kinfo->family != dd::kFamilySwar8 || p->kinfo->warps_d != 8) return;
  int sm_max = 0;
  if (cudaDeviceGetAttribute(&sm_max, cudaDevAttrMaxSharedMemoryPerMultiprocessor,
                             p->device) != cudaSuccess) {
    (void)cudaGetLastError();
    return;
  }
  if (2 * (p->smem + 1024) <= (size_t)sm_max) return;
  int n = 0;
  const dd::KernelInfo *reg = dd::kernel_registry(&n);
  const dd::KernelInfo *eight = p->kinfo, *wide = nullptr;
  for (int i = 0; i < n && !wide; i++)
    if (reg[i].family == dd::kFamilySwar8 && !reg[i].max_rows && reg[i].warps_d == 16 &&
        reg[i].items_t == eight->items_t && reg[i].items_d == eight->items_d &&
        reg[i].channels == eight->channels && reg[i].variant == eight->variant)
      wide = &reg[i];
  if (!wide) return;
  p->kinfo = wide;
  if (rebuild(p) == DD_OK) return;
  p->kinfo = eight;
  (void)rebuild(p);
}

dd_status rebuild_auto(dd_plan *p) {
  if (p->auto_kernel) p->kinfo = default_kernel(p->mode, p->bits, true);
  dd_status st = rebuild(p);
  if (st == DD_OK && p->auto_kernel && p->kinfo->family == dd::kFamilyShared8 &&
      !shared_worth_it(p)) {
    const dd::KernelInfo *shared = p->kinfo;
    p->kinfo = default_kernel(p->mode, p->bits, false);
    st = rebuild(p);
    if (st == DD_OK && p->mode == DD_SINGLE_STEP) prefer_occupancy(p);
    if (st == DD_OK) return st;
    p->kinfo = shared;  // the direct tile does not fit: keep the shared one
    return rebuild(p);
  }
  if (st != DD_ERR_UNSUPPORTED || !p->auto_kernel) return st;
  const std::string first = g_error;
  const dd::KernelInfo *direct = default_kernel(p->mode, p->bits, false);
  std::vector<const dd::KernelInfo *> cands;
  if (p->kinfo != direct) cands.push_back(direct);
  int n = 0;
  const dd::KernelInfo *reg = dd::kernel_registry(&n);
  std::vector<const dd::KernelInfo *> rest;
  for (int i = 0; i < n; i++)
    if (&reg[i] != direct && reg[i].family == direct->family &&
        reg[i].elem_bits == direct->elem_bits)
      rest.push_back(&reg[i]);
  std::stable_sort(rest.begin(), rest.end(), [](const dd::KernelInfo *x, const dd::KernelInfo *y) {
    return (uint64_t)x->tile_t * x->tile_d * x->channels >
           (uint64_t)y->tile_t * y->tile_d * y->channels;
  });
  cands.insert(cands.end(), rest.begin(), rest.end());
  for (const dd::KernelInfo *k : cands) {
    p->kinfo = k;
    st = rebuild(p);
    if (st != DD_ERR_UNSUPPORTED) return st;
  }
  p->kinfo = default_kernel(p->mode, p->bits, true);
  return fail(DD_ERR_UNSUPPORTED, "no tile fits this shape: %s", first.c_str());
}

}  // namespace
extern "C" {
namespace {
dd_status rebuild_deferred(dd_plan *p);  // defined with the setters below
}  // namespace
}
namespace {

// Build the tables if a setter changed them since the last build.  Plans are
// logically const for their queries; the build is a cache.
dd_status ensure_built(const dd_plan *cp) {
  dd_plan *p = const_cast<dd_plan *>(cp);
  if (!p->dirty) return DD_OK;
  p->dirty = false;
  return rebuild_deferred(p);
}

}  // namespace

namespace dd {
cudaError_t launch_row_stats(const ProblemDesc &P, unsigned long long *accum, uint32_t rows,
                             cudaStream_t stream);
// Lets other translation units of the library report through dd_last_error.
void set_last_error(const char *message) { g_error = message; }

// Makes `p` a stage of a subband pipeline with the packed intermediate: step
// one writes pairs of coarse DMs; step two reads them with pair tile `k`,
// widening lanes every `flush_rows` rows.  Before the tables are built.
void plan_set_packed(dd_plan *p, const KernelInfo *k, uint32_t flush_rows) {
  p->packed = true;
  p->flush_rows = flush_rows;
  if (k) p->kinfo = k;
  p->auto_kernel = false;
  p->dirty = true;
  p->ready = false;
}

// Undoes plan_set_packed: float steps on the default kernel again.
void plan_clear_packed(dd_plan *p) {
  p->packed = false;
  p->flush_rows = 0;
  p->kinfo = default_kernel(p->mode, p->bits, true);
  p->auto_kernel = true;
  p->dirty = true;
  p->ready = false;
}

// Whether the plan's tables are built (a deferred error leaves them unbuilt).
bool plan_ready(const dd_plan *p) { return ensure_built(p) == DD_OK && p->ready; }

// Family of the kernel the plan runs.
int plan_family(const dd_plan *p) {
  (void)ensure_built(p);
  return p->kinfo->family;
}

// Launches `p`'s kernel over all its tiles with arguments `P` (from
// plan_problem, possibly with another status word) on `stream`.
dd_status plan_launch(const dd_plan *p, const ProblemDesc &P, cudaStream_t stream) {
  const uint64_t tiles = (uint64_t)p->nr_groups * p->tiles_d * p->tiles_t;
  if (tiles == 0) return DD_OK;
  p->launched = true;
  p->kinfo->launch(P, (unsigned)tiles, p->smem, stream);
  DD_CUDA(cudaGetLastError(), "launch dedispersion kernel");
  return DD_OK;
}

// Launches time tiles [base, base + count) of every group and DM tile.
dd_status plan_launch_range(const dd_plan *p, ProblemDesc P, uint32_t base, uint32_t count,
                            cudaStream_t stream) {
  if (base + (uint64_t)count > p->tiles_t)
    return fail(DD_ERR_INVALID_ARGUMENT, "time tiles %u..%u past %u", base, base + count,
                p->tiles_t);
  const uint64_t tiles = (uint64_t)p->nr_groups * p->tiles_d * count;
  if (tiles == 0) return DD_OK;
  P.ttile_base = base;
  P.ttile_count = count;
  p->launched = true;
  p->kinfo->launch(P, (unsigned)tiles, p->smem, stream);
  DD_CUDA(cudaGetLastError(), "launch dedispersion kernel");
  return DD_OK;
}

// Time tiles, samples per time tile and the largest delay of a built plan.
dd_status plan_time_tiles(const dd_plan *p, uint32_t *tiles_t, uint32_t *tile_t,
                          uint32_t *max_delay) {
  if (dd_status st = ensure_built(p)) return st;
  if (!p->ready) return fail(DD_ERR_INVALID_ARGUMENT, "plan tables are invalid: %s", p->invalid.c_str());
  *tiles_t = p->tiles_t;
  *tile_t = (uint32_t)p->kinfo->tile_t;
  *max_delay = p->max_delay;
  return DD_OK;
}

// The kernel arguments of one run of `p` on the given device buffers; also
// the rows each group sums (the cost of one of its tiles).
dd_status plan_problem(const dd_plan *p, const void *d_input, float *d_output,
                       ProblemDesc *out, uint64_t *rows_per_group) {
  if (dd_status st = ensure_built(p)) return st;
  if (!p->ready)
    return fail(DD_ERR_INVALID_ARGUMENT, p->have_shifts ? "plan tables are invalid: %s"
                                                        : "plan has no shift table%s",
                p->have_shifts ? p->invalid.c_str() : "");
  const uint64_t tiles = (uint64_t)p->nr_groups * p->tiles_d * p->tiles_t;
  if (tiles && (!d_input || !d_output)) return fail(DD_ERR_INVALID_ARGUMENT, "NULL data pointer");
  if (tiles > 0x7fffffffull)
    return fail(DD_ERR_UNSUPPORTED, "problem has %llu tiles", (unsigned long long)tiles);
  const Dims &d = p->dims;
  ProblemDesc P{};
  P.in = static_cast<const uint8_t *>(d_input);
  P.out = d_output;
  P.groups = p->d_groups;
  P.entries = p->d_entries;
  P.status = p->d_status;
  P.row_bytes = d.row_bytes;
  P.out_dm_stride = p->out_dm_stride;
  P.nr_groups = p->nr_groups;
  P.nr_dms = d.nr_dms;
  P.nr_samples = d.nr_samples;
  P.bits = p->mode == DD_STEP_TWO ? 32 : p->bits;
  P.first_dm = d.first_dm;
  P.dm_step = d.dm_step;
  P.win_samples = p->win;
  P.tiles_t = p->tiles_t;
  P.tiles_d = p->tiles_d;
  P.tma = (d.row_bytes % 16 == 0 && reinterpret_cast<uintptr_t>(d_input) % 16 == 0) ? 1u : 0u;
  P.out_vec4 = (d.out_row % 4 == 0 && reinterpret_cast<uintptr_t>(d_output) % 16 == 0) ? 1u : 0u;
  P.mul_hi8 = 1u << 24;
  P.wait_ns = p->wait_ns;
  if (p->use_delay_tables) {
    P.delay_rows = (uint32_t)p->delay_shift.size();
    P.delay_rel = p->d_delay_rel;
  }
  if (p->kinfo->family == kFamilyTmem32) {
    P.delay_rows = (uint32_t)p->delay_shift.size();
    P.tmem_tab = reinterpret_cast<const uint4 *>(p->d_tmem_tab);
  }
  if (p->packed) {
    const uint32_t D1 = p->obs.nr_dms_subbanding;
    P.packed = 1;
    P.pair_groups = (D1 + 1) / 2;
    P.pair_d1 = D1;
    P.flush_rows = p->flush_rows;
    P.pair_stride = (uint64_t)d.nr_dms * d.out_row;
  }
  if (p->kinfo->family == kFamilyShared8) {
    P.stage_rows = p->d_stage_rows;
    P.stage_count = (uint32_t)p->shared.stages.size();
    P.tile_stage = p->d_tile_stage;
    P.pool = p->d_pool;
    P.cw = p->shared.cw;
    P.psw = p->shared.psw;
    P.slots = p->shared.slots;
    P.table_bytes = p->shared.table_bytes;
  }
  *out = P;
  if (rows_per_group)
    *rows_per_group = p->nr_groups ? p->entries.size() / p->nr_groups : 0;
  return DD_OK;
}
}  // namespace dd

extern "C" {

const char *dd_last_error(void) { return g_error.c_str(); }

int dd_version(void) { return DD_ABI_VERSION; }

dd_status dd_device_count(int *count) {
  if (!count) return fail(DD_ERR_INVALID_ARGUMENT, "count is NULL");
  *count = 0;
  cudaError_t e = cudaGetDeviceCount(count);
  if (e != cudaSuccess) {
    (void)cudaGetLastError();
    *count = 0;
  }
  return DD_OK;
}

uint64_t dd_pad(uint64_t value, uint64_t padding) { return pad(value, padding); }

float dd_max_freq(const dd_observation *o) { return o ? max_freq(o) : 0.0f; }
float dd_subband_min_freq(const dd_observation *o) {
  return (o && o->nr_subbands) ? subband_min_freq(o) : 0.0f;
}
float dd_subband_max_freq(const dd_observation *o) {
  return (o && o->nr_subbands) ? subband_max_freq(o) : 0.0f;
}
float dd_subband_bandwidth(const dd_observation *o) {
  return (o && o->nr_subbands) ? subband_bandwidth(o) : 0.0f;
}

dd_status dd_get_shifts(const dd_observation *o, uint32_t padding, float *shifts,
                        size_t capacity) {
  if (!o || !shifts) return fail(DD_ERR_INVALID_ARGUMENT, "NULL argument");
  if (o->nr_channels == 0) return fail(DD_ERR_INVALID_ARGUMENT, "nr_channels is 0");
  if (o->downsampling == 0) return fail(DD_ERR_INVALID_ARGUMENT, "downsampling is 0");
  size_t n = pad(o->nr_channels, padding / sizeof(float));
  if (capacity < n) return fail(DD_ERR_INVALID_ARGUMENT, "shift table needs %zu floats", n);
  std::fill(shifts, shifts + n, 0.0f);
  shift_table(o, o->min_freq, o->channel_bandwidth, max_freq(o), o->nr_channels, shifts);
  return DD_OK;
}

dd_status dd_get_shifts_step_two(const dd_observation *o, uint32_t padding, float *shifts,
                                 size_t capacity) {
  if (!o || !shifts) return fail(DD_ERR_INVALID_ARGUMENT, "NULL argument");
  if (o->nr_subbands == 0 || o->nr_subbands > o->nr_channels)
    return fail(DD_ERR_INVALID_ARGUMENT, "nr_subbands must be in 1..nr_channels");
  if (o->downsampling == 0) return fail(DD_ERR_INVALID_ARGUMENT, "downsampling is 0");
  size_t n = pad(o->nr_subbands, padding / sizeof(float));
  if (capacity < n) return fail(DD_ERR_INVALID_ARGUMENT, "shift table needs %zu floats", n);
  std::fill(shifts, shifts + n, 0.0f);
  shift_table(o, subband_min_freq(o), subband_bandwidth(o), subband_max_freq(o),
              o->nr_subbands, shifts);
  return DD_OK;
}

dd_status dd_get_layout(const dd_observation *o, dd_mode mode, uint32_t input_bits,
                        uint32_t padding, const float *shifts, dd_layout *layout) {
  dd_status st = check_obs(o, mode);
  if (st) return st;
  if (!layout) return fail(DD_ERR_INVALID_ARGUMENT, "layout is NULL");
  if (mode == DD_STEP_TWO) input_bits = 32;
  if (!bits_ok(input_bits)) return fail(DD_ERR_UNSUPPORTED, "input_bits %u not supported", input_bits);
  Dims d = dims_of(o, mode, input_bits, padding);
  layout->input_row_bytes = d.row_bytes;
  layout->input_bytes = d.input_bytes;
  layout->output_row_elems = d.out_row;
  layout->output_bytes = d.output_rows * d.out_row * sizeof(float);
  layout->mapping_row_elems = d.mapping_row;
  layout->zapped_elems = d.zapped_elems;
  layout->shifts_elems = d.shift_elems;
  layout->max_delay = 0;
  if (shifts && d.nr_dms) {
    uint32_t n = mode == DD_STEP_TWO ? o->nr_subbands : o->nr_channels;
    for (uint32_t c = 0; c < n; c++) {
      float sh = shifts[c];
      if (mode == DD_STEP_ONE) {
        uint32_t cps = o->nr_channels / o->nr_subbands;
        if (c >= cps * o->nr_subbands) break;
        volatile float rel = shifts[c] - shifts[(c / cps + 1) * cps - 1];
        sh = rel;
      }
      layout->max_delay = std::max(layout->max_delay, dd::host_delay(d.first_dm, d.dm_step, d.nr_dms - 1, sh));
    }
  }
  layout->required_dispersed_samples = d.nr_samples + layout->max_delay;
  return DD_OK;
}

dd_status dd_default_conf(const dd_observation *o, dd_mode mode, uint32_t input_bits,
                          dd_conf *conf) {
  (void)o;
  if (!conf) return fail(DD_ERR_INVALID_ARGUMENT, "conf is NULL");
  if (mode == DD_STEP_TWO) input_bits = 32;
  if (!bits_ok(input_bits)) return fail(DD_ERR_UNSUPPORTED, "input_bits %u not supported", input_bits);
  const dd::KernelInfo *k = default_kernel(mode, input_bits, true);
  if (!k) return fail(DD_ERR_UNSUPPORTED, "no kernel for %u-bit input", input_bits);
  *conf = conf_of(*k);
  return DD_OK;
}

dd_status dd_conf_print(const dd_conf *c, char *text, size_t capacity) {
  if (!c || !text || capacity == 0) return fail(DD_ERR_INVALID_ARGUMENT, "NULL argument");
  int n = snprintf(text, capacity, "%u %u %u %u %u %u %u %u %u", c->split_batches ? 1u : 0u,
                   c->local_mem ? 1u : 0u, c->unroll, c->threads_d0, c->threads_d1, c->threads_d2,
                   c->items_d0, c->items_d1, c->items_d2);
  if (n < 0 || (size_t)n >= capacity) return fail(DD_ERR_INVALID_ARGUMENT, "buffer too small");
  return DD_OK;
}

dd_status dd_read_tuned_conf(const char *path, const char *device, uint32_t nr_dms,
                             dd_conf *conf) {
  if (!path || !device || !conf) return fail(DD_ERR_INVALID_ARGUMENT, "NULL argument");
  std::ifstream in(path);
  if (!in) return fail(DD_ERR_FILE, "Impossible to open %s", path);
  std::string line;
  unsigned lineno = 0;
  while (std::getline(in, line)) {
    lineno++;
    if (line.empty() || !std::isalpha(static_cast<unsigned char>(line[0]))) continue;
    std::istringstream ls(line);
    std::string dev;
    unsigned long v[10];
    ls >> dev;
    bool good = true;
    for (int i = 0; i < 10 && good; i++) good = static_cast<bool>(ls >> v[i]);
    if (!good)
      return fail(DD_ERR_FILE, "%s:%u: expected 'device nrDMs split local unroll tD0 tD1 tD2 "
                  "iD0 iD1 iD2'", path, lineno);
    if (dev != device || v[0] != nr_dms) continue;
    conf->split_batches = v[1] != 0; conf->local_mem = v[2] != 0; conf->unroll = (uint32_t)v[3];
    conf->threads_d0 = (uint32_t)v[4]; conf->threads_d1 = (uint32_t)v[5];
    conf->threads_d2 = (uint32_t)v[6]; conf->items_d0 = (uint32_t)v[7];
    conf->items_d1 = (uint32_t)v[8]; conf->items_d2 = (uint32_t)v[9];
    return DD_OK;  // the first line for (device, nrDMs) wins, as std::map::insert keeps it
  }
  return fail(DD_ERR_NOT_FOUND, "no entry for device '%s' and %u DMs in %s", device, nr_dms, path);
}

dd_status dd_write_tuned_conf(const char *path, const char *device, uint32_t nr_dms,
                              const dd_conf *conf) {
  if (!path || !device || !conf) return fail(DD_ERR_INVALID_ARGUMENT, "NULL argument");
  if (!*device || !std::isalpha(static_cast<unsigned char>(device[0])) || strchr(device, ' '))
    return fail(DD_ERR_INVALID_ARGUMENT, "device name must start with a letter and hold no spaces");
  char text[256];
  dd_status st = dd_conf_print(conf, text, sizeof(text));
  if (st) return st;
  std::ofstream out(path, std::ios::app);
  if (!out) return fail(DD_ERR_FILE, "Impossible to open %s", path);
  out << device << " " << nr_dms << " " << text << "\n";
  return out ? DD_OK : fail(DD_ERR_FILE, "write to %s failed", path);
}

dd_status dd_plan_create(dd_plan **plan, const dd_observation *o, dd_mode mode,
                         uint32_t input_bits, uint32_t padding, const dd_conf *conf,
                         int device) {
  if (!plan) return fail(DD_ERR_INVALID_ARGUMENT, "plan is NULL");
  *plan = nullptr;
  dd_status st = check_obs(o, mode);
  if (st) return st;
  if (mode == DD_STEP_TWO) input_bits = 32;
  if (!bits_ok(input_bits)) return fail(DD_ERR_UNSUPPORTED, "input_bits %u not supported", input_bits);
  st = device_ok();
  if (st) return st;
  int ndev = 0;
  cudaGetDeviceCount(&ndev);
  if (device < 0 || device >= ndev)
    return fail(DD_ERR_INVALID_ARGUMENT, "device %d out of range (0..%d)", device, ndev - 1);
  dd_conf c{};
  if (conf) c = *conf;
  else dd_default_conf(o, mode, input_bits, &c);
  if (c.split_batches) return fail(DD_ERR_UNSUPPORTED, "split_batches is not implemented by the reference either");
  if (!c.local_mem) return fail(DD_ERR_UNSUPPORTED, "only local_mem=1 (staged rows) configurations are compiled");
  const dd::KernelInfo *k = find_kernel(mode, input_bits, c);
  if (!k) {
    char text[128];
    dd_conf_print(&c, text, sizeof(text));
    return fail(DD_ERR_UNSUPPORTED, "no compiled kernel for configuration '%s' (%u-bit input)", text,
                input_bits);
  }
  dd_plan *p = new dd_plan();
  p->device = device; p->obs = *o; p->mode = mode; p->bits = input_bits; p->padding = padding;
  p->kinfo = k;
  p->auto_kernel = conf == nullptr;
  p->dims = dims_of(o, mode, input_bits, padding);
  {
    DeviceGuard g(device);
    cudaError_t e = cudaMalloc(&p->d_status, sizeof(uint32_t));
    if (e == cudaSuccess) e = cudaMemset(p->d_status, 0, sizeof(uint32_t));
    if (e != cudaSuccess) {
      delete p;
      return cuda_fail(e, "allocate status word");
    }
  }
  *plan = p;
  return DD_OK;
}

int dd_kernel_count(void) {
  int n = 0;
  dd::kernel_registry(&n);
  return n;
}

dd_status dd_kernel_info(int index, char *name, size_t capacity, uint32_t *elem_bits,
                         dd_conf *conf) {
  int n = 0;
  const dd::KernelInfo *reg = dd::kernel_registry(&n);
  if (index < 0 || index >= n) return fail(DD_ERR_INVALID_ARGUMENT, "kernel index %d out of range", index);
  if (name && capacity) {
    std::strncpy(name, reg[index].name, capacity);
    name[capacity - 1] = 0;
  }
  if (elem_bits) *elem_bits = (uint32_t)reg[index].elem_bits;
  if (conf) *conf = conf_of(reg[index]);
  return DD_OK;
}

dd_status dd_plan_create_with_kernel(dd_plan **plan, const dd_observation *o, dd_mode mode,
                                     uint32_t input_bits, uint32_t padding, int kernel_index,
                                     int device) {
  int n = 0;
  const dd::KernelInfo *reg = dd::kernel_registry(&n);
  if (kernel_index < 0 || kernel_index >= n)
    return fail(DD_ERR_INVALID_ARGUMENT, "kernel index %d out of range", kernel_index);
  const uint32_t bits = mode == DD_STEP_TWO ? 32 : input_bits;
  if (!bits_ok(bits)) return fail(DD_ERR_UNSUPPORTED, "input_bits %u not supported", bits);
  if ((uint32_t)reg[kernel_index].elem_bits != family_bits(mode, bits))
    return fail(DD_ERR_UNSUPPORTED, "kernel %s does not take %u-bit input", reg[kernel_index].name,
                bits);
  dd_conf c = conf_of(reg[kernel_index]);
  dd_status st = dd_plan_create(plan, o, mode, input_bits, padding, &c, device);
  if (st) return st;
  (*plan)->kinfo = &reg[kernel_index];
  return DD_OK;
}

namespace {
// Rebuild after a table change.  Tables set one at a time can be
// inconsistent in between (delays checked before the zapped mask arrives):
// such errors are kept and reported by the next run; device errors return.
dd_status rebuild_deferred(dd_plan *p) {
  dd_status st = rebuild_auto(p);
  if (st == DD_ERR_INVALID_ARGUMENT || st == DD_ERR_UNSUPPORTED) {
    p->invalid = g_error;
    return DD_OK;
  }
  if (!st) p->invalid.clear();
  return st;
}
}  // namespace

dd_status dd_plan_set_shifts(dd_plan *p, const float *shifts, size_t n) {
  if (!p || !shifts) return fail(DD_ERR_INVALID_ARGUMENT, "NULL argument");
  size_t need = p->mode == DD_STEP_TWO ? p->obs.nr_subbands : p->obs.nr_channels;
  if (n < need) return fail(DD_ERR_INVALID_ARGUMENT, "shift table has %zu entries, needs %zu", n, need);
  p->shifts.assign(shifts, shifts + need);
  p->have_shifts = true;
  p->dirty = true;
  p->ready = false;
  return DD_OK;
}

dd_status dd_plan_set_zapped(dd_plan *p, const uint32_t *zapped, size_t n) {
  if (!p || !zapped) return fail(DD_ERR_INVALID_ARGUMENT, "NULL argument");
  if (p->mode == DD_STEP_TWO) return fail(DD_ERR_INVALID_ARGUMENT, "step two has no zapped mask");
  if (n < p->obs.nr_channels)
    return fail(DD_ERR_INVALID_ARGUMENT, "zapped mask has %zu entries, needs %u", n, p->obs.nr_channels);
  p->zapped.assign(zapped, zapped + p->obs.nr_channels);
  p->dirty = true;
  p->ready = false;
  return DD_OK;
}

dd_status dd_plan_set_beam_mapping(dd_plan *p, const uint32_t *mapping, size_t n) {
  if (!p || !mapping) return fail(DD_ERR_INVALID_ARGUMENT, "NULL argument");
  if (p->mode == DD_STEP_ONE) return fail(DD_ERR_INVALID_ARGUMENT, "step one has no beam mapping");
  size_t need = (size_t)p->obs.nr_synthesized_beams * p->dims.mapping_row;
  if (n < need) return fail(DD_ERR_INVALID_ARGUMENT, "beam mapping has %zu entries, needs %zu", n, need);
  p->mapping.assign(mapping, mapping + need);
  p->dirty = true;
  p->ready = false;
  return DD_OK;
}

dd_status dd_plan_run(dd_plan *p, const void *d_input, float *d_output, void *stream) {
  if (!p) return fail(DD_ERR_INVALID_ARGUMENT, "plan is NULL");
  dd::ProblemDesc P{};
  dd_status st = dd::plan_problem(p, d_input, d_output, &P, nullptr);
  if (st) return st;
  const uint64_t tiles = (uint64_t)p->nr_groups * p->tiles_d * p->tiles_t;
  if (tiles == 0) return DD_OK;
  DeviceGuard g(p->device);
  if (!g.ok) return fail(DD_ERR_CUDA, "cannot select device %d", p->device);
  p->launched = true;
  // The shared, swar8 and pair tiles take part (the scalar and TMEM-window
  // tiles launch as usual; the latter holds all of an SM's TMEM per CTA).
  if (p->overlap && p->kinfo->family != dd::kFamilyScalar &&
      p->kinfo->family != dd::kFamilyTmem32) {
    // A programmatic dependent of the stream's previous kernel: its tiles
    // start on SMs the previous launch's last wave leaves idle.
    P.overlap = 1;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)tiles);
    cfg.blockDim = dim3((unsigned)p->kinfo->threads);
    cfg.dynamicSmemBytes = p->smem;
    cfg.stream = static_cast<cudaStream_t>(stream);
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    void *args[] = {&P};
    DD_CUDA(cudaLaunchKernelExC(&cfg, p->kinfo->func, args), "launch dedispersion kernel");
    return DD_OK;
  }
  p->kinfo->launch(P, (unsigned)tiles, p->smem, static_cast<cudaStream_t>(stream));
  DD_CUDA(cudaGetLastError(), "launch dedispersion kernel");
  return DD_OK;
}

dd_status dd_plan_set_wait_limit(dd_plan *p, uint32_t ns) {
  if (!p) return fail(DD_ERR_INVALID_ARGUMENT, "plan is NULL");
  p->wait_ns = ns;
  return DD_OK;
}

dd_status dd_plan_set_overlap(dd_plan *p, int enable) {
  if (!p) return fail(DD_ERR_INVALID_ARGUMENT, "plan is NULL");
  p->overlap = enable != 0;
  return DD_OK;
}

dd_status dd_plan_run_stats(dd_plan *p, const void *d_input, float *d_output,
                            dd_dm_accum *d_accum, void *stream) {
  if (!p || !d_accum) return fail(DD_ERR_INVALID_ARGUMENT, "NULL argument");
  if (p->mode != DD_SINGLE_STEP || p->bits > 16)
    return fail(DD_ERR_UNSUPPORTED,
                "detection statistics are computed for single-step input of 1-16 bits");
  dd::ProblemDesc P{};
  dd_status st = dd::plan_problem(p, d_input, d_output, &P, nullptr);
  if (st) return st;
  const uint64_t tiles = (uint64_t)p->nr_groups * p->tiles_d * p->tiles_t;
  const uint64_t rows = (uint64_t)p->nr_groups * p->dims.nr_dms;
  DeviceGuard g(p->device);
  if (!g.ok) return fail(DD_ERR_CUDA, "cannot select device %d", p->device);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  DD_CUDA(cudaMemsetAsync(d_accum, 0, rows * sizeof(dd_dm_accum), s), "clear statistics");
  if (tiles == 0) return DD_OK;
  const bool fused = p->kinfo->family == dd::kFamilyShared8;
  if (fused) P.accum = reinterpret_cast<unsigned long long *>(d_accum);
  p->launched = true;
  p->kinfo->launch(P, (unsigned)tiles, p->smem, s);
  DD_CUDA(cudaGetLastError(), "launch dedispersion kernel");
  if (!fused)
    DD_CUDA(dd::launch_row_stats(P, reinterpret_cast<unsigned long long *>(d_accum),
                                 (uint32_t)rows, s),
            "launch statistics kernel");
  return DD_OK;
}

dd_status dd_plan_check(dd_plan *p, void *stream) {
  if (!p) return fail(DD_ERR_INVALID_ARGUMENT, "plan is NULL");
  DeviceGuard g(p->device);
  DD_CUDA(cudaStreamSynchronize(static_cast<cudaStream_t>(stream)), "synchronize stream");
  uint32_t status = 0;
  DD_CUDA(cudaMemcpy(&status, p->d_status, sizeof(status), cudaMemcpyDeviceToHost), "read status");
  if (status) {
    DD_CUDA(cudaMemset(p->d_status, 0, sizeof(uint32_t)), "reset status");
    if (status & dd::kStatusTimeout)
      return fail(DD_ERR_TIMEOUT, "a bounded wait for a staged row ran out on the device");
    return fail(DD_ERR_CUDA, "device status 0x%x", status);
  }
  return DD_OK;
}

dd_status dd_plan_time(dd_plan *p, const void *d_input, float *d_output, uint32_t warmup,
                       uint32_t iterations, float *mean_ms, float *std_ms) {
  if (!p || !mean_ms || iterations == 0) return fail(DD_ERR_INVALID_ARGUMENT, "bad argument");
  DeviceGuard g(p->device);
  cudaStream_t s = nullptr;
  DD_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking), "create stream");
  std::vector<cudaEvent_t> ev(iterations + 1, nullptr);
  dd_status st = DD_OK;
  for (auto &e : ev)
    if (cudaEventCreate(&e) != cudaSuccess) st = cuda_fail(cudaGetLastError(), "create event");
  for (uint32_t i = 0; i < warmup && !st; i++) st = dd_plan_run(p, d_input, d_output, s);
  if (!st && cudaEventRecord(ev[0], s) != cudaSuccess) st = cuda_fail(cudaGetLastError(), "record");
  for (uint32_t i = 0; i < iterations && !st; i++) {
    st = dd_plan_run(p, d_input, d_output, s);
    if (!st && cudaEventRecord(ev[i + 1], s) != cudaSuccess)
      st = cuda_fail(cudaGetLastError(), "record");
  }
  if (!st) st = dd_plan_check(p, s);
  if (!st) {
    double sum = 0, sq = 0;
    for (uint32_t i = 0; i < iterations; i++) {
      float ms = 0;
      cudaEventElapsedTime(&ms, ev[i], ev[i + 1]);
      sum += ms;
      sq += (double)ms * ms;
    }
    const double mean = sum / iterations;
    *mean_ms = (float)mean;
    if (std_ms) *std_ms = (float)std::sqrt(std::max(0.0, sq / iterations - mean * mean));
  }
  for (auto &e : ev)
    if (e) cudaEventDestroy(e);
  cudaStreamDestroy(s);
  return st;
}

dd_status dd_plan_launches(const dd_plan *p, uint32_t *launches) {
  if (!p || !launches) return fail(DD_ERR_INVALID_ARGUMENT, "NULL argument");
  *launches = ((uint64_t)p->nr_groups * p->tiles_d * p->tiles_t) ? 1u : 0u;
  return DD_OK;
}

dd_status dd_plan_get_conf(const dd_plan *p, dd_conf *conf) {
  if (p) {
    dd_status st = ensure_built(p);
    if (st) return st;
  }
  if (!p || !conf) return fail(DD_ERR_INVALID_ARGUMENT, "NULL argument");
  *conf = conf_of(*p->kinfo);
  return DD_OK;
}

dd_status dd_plan_adds(const dd_plan *p, uint64_t *adds) {
  if (!p || !adds) return fail(DD_ERR_INVALID_ARGUMENT, "NULL argument");
  if (dd_status st = ensure_built(p)) return st;
  if (!p->ready)
    return fail(DD_ERR_INVALID_ARGUMENT, p->have_shifts ? "plan tables are invalid: %s"
                                                        : "plan has no shift table%s",
                p->have_shifts ? p->invalid.c_str() : "");
  const dd::KernelInfo &k = *p->kinfo;
  const uint64_t per_tile = k.family == dd::kFamilyShared8
                                ? p->shared.adds_partial + p->shared.adds_series
                                : (p->nr_groups ? p->entries.size() / p->nr_groups : 0) *
                                      (uint64_t)k.tile_d * k.tile_t * p->tiles_d;
  *adds = per_tile * p->nr_groups * p->tiles_t;
  return DD_OK;
}

dd_status dd_plan_destroy(dd_plan *p) {
  if (!p) return DD_OK;
  {
    DeviceGuard g(p->device);
    if (p->d_groups) cudaFree(p->d_groups);
    if (p->d_entries) cudaFree(p->d_entries);
    if (p->d_status) cudaFree(p->d_status);
    if (p->d_delay_rel) cudaFree(p->d_delay_rel);
    if (p->d_tmem_tab) cudaFree(p->d_tmem_tab);
    if (p->d_stage_rows) cudaFree(p->d_stage_rows);
    if (p->d_tile_stage) cudaFree(p->d_tile_stage);
    if (p->d_pool) cudaFree(p->d_pool);
  }
  delete p;
  return DD_OK;
}

}  // extern "C"

// ---- synchronous host-buffer calls ----------------------------------------

namespace {

// Per-thread cache of the last plan and device buffers of the synchronous
// calls, so that repeated calls on one geometry only copy and launch.
// Chunked host-buffer runs (run_sync): launches per call and the smallest
// problem (in tiles) that is split.  At 1536 channels x 2048 DMs x 24576
// samples a call takes 4.19 ms in one chunk and 3.27 / 3.13 / 3.08 / 3.06 /
// 3.06 / 3.24 ms in 4 / 8 / 12 / 16 / 24 / 32 (one GB300, pinned host
// buffers; the kernel alone takes 2.87 ms).
constexpr uint32_t kChunks = 16;
constexpr uint64_t kChunkMinTiles = 2048;

// The device address under which the kernels can write `bytes` of host
// memory at `host` directly (NVLink-C2C on a Grace host), or NULL.  Both ends
// of the range must be pinned (page-locked, mapped) memory whose device
// addresses are `bytes - 1` apart, and the device must reach host memory
// through the host's page tables (pageable memory access), so that every
// address of a valid buffer is reachable even between two pinned
// allocations.  The kernels' output stores then need no device buffer and no
// copy back: at 1536 x 2048 x 24576 a launch writing its 201 MB to pinned
// host memory took 2.78 ms against 2.75 ms into device memory.
void *host_output_device_address(void *host, size_t bytes, int dev) {
  if (!host || bytes == 0) return nullptr;
  // The device attribute, read once per thread (run_sync's cache is per
  // thread too; it always runs on device 0).
  thread_local int pageable = -1;
  if (pageable < 0) {
    if (cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccess, dev) != cudaSuccess) {
      (void)cudaGetLastError();
      pageable = 0;
    }
  }
  if (!pageable) return nullptr;
  cudaPointerAttributes a{}, b{};
  if (cudaPointerGetAttributes(&a, host) != cudaSuccess ||
      cudaPointerGetAttributes(&b, static_cast<char *>(host) + bytes - 1) != cudaSuccess) {
    (void)cudaGetLastError();
    return nullptr;
  }
  if (a.type != cudaMemoryTypeHost || b.type != cudaMemoryTypeHost || !a.devicePointer ||
      !b.devicePointer)
    return nullptr;
  if (static_cast<char *>(b.devicePointer) - static_cast<char *>(a.devicePointer) !=
      static_cast<ptrdiff_t>(bytes - 1))
    return nullptr;
  return a.devicePointer;
}

struct SyncCache {
  dd_plan *plan = nullptr;
  dd_observation obs{};
  dd_mode mode = DD_SINGLE_STEP;
  uint32_t bits = 0, padding = 0;
  std::vector<float> shifts;
  std::vector<uint32_t> zapped, mapping;
  void *d_in = nullptr;
  float *d_out = nullptr;
  size_t cap_in = 0, cap_out = 0;
  cudaStream_t stream = nullptr;
  // Chunked runs: a second compute stream, the output and input copy
  // streams, and events [input of chunk 0 .. kChunks - 1, chunk 0 ..
  // kChunks - 1 done, copies done, side done].
  cudaStream_t side = nullptr, copy = nullptr, copy_in = nullptr;
  std::vector<cudaEvent_t> events;
  ~SyncCache() {
    if (plan) dd_plan_destroy(plan);
    if (d_in) cudaFree(d_in);
    if (d_out) cudaFree(d_out);
    if (stream) cudaStreamDestroy(stream);
    if (side) cudaStreamDestroy(side);
    if (copy) cudaStreamDestroy(copy);
    if (copy_in) cudaStreamDestroy(copy_in);
    for (cudaEvent_t e : events) cudaEventDestroy(e);
  }
};

thread_local SyncCache g_sync;

dd_status run_sync(const dd_observation *o, dd_mode mode, const uint32_t *zapped,
                   const uint32_t *mapping, const void *input, float *output,
                   const float *shifts, uint32_t padding, uint32_t bits) {
  dd_status st = check_obs(o, mode);
  if (st) return st;
  if (!input || !output || !shifts) return fail(DD_ERR_INVALID_ARGUMENT, "NULL data pointer");
  if (mode != DD_STEP_TWO && !zapped) return fail(DD_ERR_INVALID_ARGUMENT, "zapped mask is NULL");
  if (mode != DD_STEP_ONE && !mapping) return fail(DD_ERR_INVALID_ARGUMENT, "beam mapping is NULL");
  if (mode == DD_STEP_TWO) bits = 32;
  st = device_ok();
  if (st) return st;
  SyncCache &c = g_sync;
  const bool same_geom = c.plan && c.mode == mode && c.bits == bits && c.padding == padding &&
                         std::memcmp(&c.obs, o, sizeof(*o)) == 0;
  if (!same_geom) {
    if (c.plan) dd_plan_destroy(c.plan);
    c.plan = nullptr;
    c.shifts.clear(); c.zapped.clear(); c.mapping.clear();
    st = dd_plan_create(&c.plan, o, mode, bits, padding, nullptr, 0);
    if (st) return st;
    c.obs = *o; c.mode = mode; c.bits = bits; c.padding = padding;
  }
  const Dims &d = c.plan->dims;
  const size_t nsh = mode == DD_STEP_TWO ? o->nr_subbands : o->nr_channels;
  bool dirty = false;
  if (c.shifts.size() != nsh || std::memcmp(c.shifts.data(), shifts, nsh * 4)) {
    c.shifts.assign(shifts, shifts + nsh);
    c.plan->shifts = c.shifts;
    c.plan->have_shifts = true;
    dirty = true;
  }
  if (mode != DD_STEP_TWO &&
      (c.zapped.size() != o->nr_channels || std::memcmp(c.zapped.data(), zapped, o->nr_channels * 4))) {
    c.zapped.assign(zapped, zapped + o->nr_channels);
    c.plan->zapped = c.zapped;
    dirty = true;
  }
  if (mode != DD_STEP_ONE) {
    size_t nm = (size_t)o->nr_synthesized_beams * d.mapping_row;
    if (c.mapping.size() != nm || std::memcmp(c.mapping.data(), mapping, nm * 4)) {
      c.mapping.assign(mapping, mapping + nm);
      c.plan->mapping = c.mapping;
      dirty = true;
    }
  }
  if (dirty) {
    st = rebuild_auto(c.plan);
    if (st) {
      c.shifts.clear();
      return st;
    }
  }
  DeviceGuard g(0);
  if (!c.stream) DD_CUDA(cudaStreamCreateWithFlags(&c.stream, cudaStreamNonBlocking), "create stream");
  const size_t in_bytes = d.input_bytes;
  const size_t out_bytes = d.output_rows * d.out_row * sizeof(float);
  if (in_bytes > c.cap_in) {
    if (c.d_in) cudaFree(c.d_in);
    c.d_in = nullptr; c.cap_in = 0;
    DD_CUDA(cudaMalloc(&c.d_in, in_bytes), "allocate device input");
    c.cap_in = in_bytes;
  }
  // Pinned host output on a Grace host: the kernels write it directly, and
  // no device output buffer is needed.
  float *direct = static_cast<float *>(host_output_device_address(output, out_bytes, 0));
  if (!direct && out_bytes > c.cap_out) {
    if (c.d_out) cudaFree(c.d_out);
    c.d_out = nullptr; c.cap_out = 0;
    DD_CUDA(cudaMalloc(&c.d_out, out_bytes), "allocate device output");
    c.cap_out = out_bytes;
  }
  const dd_plan *p = c.plan;
  const uint64_t tt_total = p->tiles_t;
  const uint64_t tiles = (uint64_t)p->nr_groups * p->tiles_d * tt_total;
  float *kout = direct ? direct : c.d_out;
  if (tiles < kChunkMinTiles || tt_total < 2 || !d.nr_samples || !d.output_rows) {
    // Small problems: one copy in, one launch, one copy out.
    if (in_bytes)
      DD_CUDA(cudaMemcpyAsync(c.d_in, input, in_bytes, cudaMemcpyHostToDevice, c.stream),
              "copy input");
    st = dd_plan_run(c.plan, c.d_in, kout, c.stream);
    if (st) return st;
    if (!direct && d.output_rows && d.nr_samples)
      DD_CUDA(cudaMemcpy2DAsync(output, d.out_row * sizeof(float), c.d_out,
                                d.out_row * sizeof(float), (size_t)d.nr_samples * sizeof(float),
                                d.output_rows, cudaMemcpyDeviceToHost, c.stream),
              "copy output");
    return dd_plan_check(c.plan, c.stream);
  }
  // Chunked over time tiles: chunk k computes every (group, DM tile) over
  // its time tiles, so it needs input samples below its last tile's end +
  // the largest delay.  The input comes in pieces on a copy stream, each
  // before the first chunk that reads it; chunks alternate between two
  // compute streams (a chunk's last partial wave overlaps the next one); each
  // chunk's output columns go back on a third stream while later chunks
  // compute.
  for (cudaStream_t *x : {&c.side, &c.copy, &c.copy_in})
    if (!*x) DD_CUDA(cudaStreamCreateWithFlags(x, cudaStreamNonBlocking), "create stream");
  while (c.events.size() < 2 * kChunks + 2) {
    cudaEvent_t e;
    DD_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming), "create event");
    c.events.push_back(e);
  }
  dd::ProblemDesc P{};
  st = dd::plan_problem(p, c.d_in, kout, &P, nullptr);
  if (st) return st;
  const uint32_t K = (uint32_t)std::min<uint64_t>(kChunks, tt_total);
  const uint64_t T = (uint64_t)p->kinfo->tile_t;
  const uint64_t in_rows = d.input_bytes / d.row_bytes;
  const uint64_t elem_bits = mode == DD_STEP_TWO ? 32 : bits;
  // Bytes of each input row that hold samples below `samples`, with slack
  // for the staged windows' alignment.
  auto row_bytes_below = [&](uint64_t samples) {
    const uint64_t bytes = (samples * elem_bits + 7) / 8 + 128;
    return std::min<uint64_t>((bytes + 15) / 16 * 16, d.row_bytes);
  };
  const uint8_t *in8 = static_cast<const uint8_t *>(input);
  uint8_t *din8 = static_cast<uint8_t *>(c.d_in);
  uint64_t copied = 0;
  for (uint32_t k = 0; k < K; k++) {
    const uint64_t a = tt_total * k / K, b = tt_total * (k + 1) / K;
    const uint64_t need = k + 1 == K ? d.row_bytes : row_bytes_below(b * T + p->max_delay);
    if (need > copied) {
      DD_CUDA(cudaMemcpy2DAsync(din8 + copied, d.row_bytes, in8 + copied, d.row_bytes,
                                need - copied, in_rows, cudaMemcpyHostToDevice, c.copy_in),
              "copy input");
      copied = need;
    }
    DD_CUDA(cudaEventRecord(c.events[k], c.copy_in), "record input");
    cudaStream_t sk = (k & 1u) ? c.side : c.stream;
    DD_CUDA(cudaStreamWaitEvent(sk, c.events[k], 0), "wait input");
    P.ttile_base = (uint32_t)a;
    P.ttile_count = (uint32_t)(b - a);
    p->kinfo->launch(P, (unsigned)((uint64_t)p->nr_groups * p->tiles_d * (b - a)), p->smem, sk);
    DD_CUDA(cudaGetLastError(), "launch dedispersion kernel");
    DD_CUDA(cudaEventRecord(c.events[kChunks + k], sk), "record chunk");
  }
  // The copies out after every launch: a copy to pageable host memory blocks
  // this thread, and the later chunks must already be queued.  Output the
  // kernels wrote straight into host memory needs none: the copy stream only
  // waits for the chunks.
  for (uint32_t k = 0; k < K; k++) {
    if (direct) {
      DD_CUDA(cudaStreamWaitEvent(c.copy, c.events[kChunks + k], 0), "wait chunk");
      continue;
    }
    const uint64_t a = tt_total * k / K, b = tt_total * (k + 1) / K;
    const uint64_t t0 = a * T, t1 = std::min<uint64_t>(b * T, d.nr_samples);
    DD_CUDA(cudaStreamWaitEvent(c.copy, c.events[kChunks + k], 0), "wait chunk");
    if (t1 > t0)
      DD_CUDA(cudaMemcpy2DAsync(output + t0, d.out_row * sizeof(float), c.d_out + t0,
                                d.out_row * sizeof(float), (t1 - t0) * sizeof(float),
                                d.output_rows, cudaMemcpyDeviceToHost, c.copy),
              "copy output");
  }
  DD_CUDA(cudaEventRecord(c.events[2 * kChunks], c.copy), "record copies");
  DD_CUDA(cudaEventRecord(c.events[2 * kChunks + 1], c.side), "record side");
  DD_CUDA(cudaStreamWaitEvent(c.stream, c.events[2 * kChunks], 0), "join copies");
  DD_CUDA(cudaStreamWaitEvent(c.stream, c.events[2 * kChunks + 1], 0), "join side");
  return dd_plan_check(c.plan, c.stream);
}

}  // namespace

extern "C" {

dd_status dd_dedispersion(const dd_observation *o, const uint32_t *zapped,
                          const uint32_t *beam_mapping, const void *input, float *output,
                          const float *shifts, uint32_t padding, uint32_t input_bits) {
  return run_sync(o, DD_SINGLE_STEP, zapped, beam_mapping, input, output, shifts, padding,
                  input_bits);
}

dd_status dd_subband_dedispersion_step_one(const dd_observation *o, const uint32_t *zapped,
                                           const void *input, float *output, const float *shifts,
                                           uint32_t padding, uint32_t input_bits) {
  return run_sync(o, DD_STEP_ONE, zapped, nullptr, input, output, shifts, padding, input_bits);
}

dd_status dd_subband_dedispersion_step_two(const dd_observation *o, const uint32_t *beam_mapping,
                                           const float *input, float *output, const float *shifts,
                                           uint32_t padding) {
  return run_sync(o, DD_STEP_TWO, nullptr, beam_mapping, input, output, shifts, padding, 32);
}

}  // extern "C"
