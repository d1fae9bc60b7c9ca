// dd_internal.h -- descriptors shared by the host library and the kernels.
//
// A dedispersion problem is a set of output groups.  Each group sums a list
// of input rows (its live channels, or its subbands in step two), each with
// its own delay per unit DM, into a [DM][sample] block of the output:
//
//   out[g.out_offset + dm * out_dm_stride + t] =
//       sum_k in_row(g, k)[t + (uint)((first_dm + dm * dm_step) * shift_k)]
//
// Single step (include/Dedispersion.hpp:70-109): group = synthesized beam,
//   rows = non-zapped channels of the mapped beam.
// Step one (include/Dedispersion.hpp:111-153): group = (beam, subband),
//   rows = non-zapped channels of the subband, shift relative to the
//   subband's last channel.
// Step two (include/Dedispersion.hpp:155-176): group = (synthesized beam,
//   step-one DM), rows = the subbands of the step-one output.
#pragma once

#include <cstddef>
#include <cstdint>

#include <cuda_runtime.h>

namespace dd {

// One output group.
struct GroupDesc {
  uint32_t entry_begin;  // first entry of this group in the entry table
  uint32_t entry_count;  // rows summed (0: the group's output is all zero)
  uint64_t out_offset;   // float offset of (dm 0, sample 0) of the group
};

// One input row of a group.
struct EntryDesc {
  uint64_t row_offset;  // byte offset of the row from the input base
  float shift;          // delay in samples per unit DM
  uint32_t delay_row;   // row of the precomputed delay tables (when present)
};

// One pipeline stage of the shared-partial-sum family (kFamilyShared8), for
// one DM tile: up to 4 subgroups of up to kSharedRows consecutive rows of a
// group (32 rows).  For every DM d of the tile a subgroup's delays are
// base(d) + rel(row, d), base(d) = the least delay of its rows.  DMs whose
// relative-delay vectors are equal share one partial-sum series
//   P_v[u] = sum_rows in_row[t0 + bmin + u + rel_v(row)],
// and DM d adds P_{v(d)}[t + base(d) - bmin]: the same integer sum as the
// direct form with fewer adds.  The stage table (in `pool`, laid out as
// dd_shared.cuh describes) holds the subgroups' series programs and each
// DM's series offsets.
struct SharedStage {
  uint32_t pool;         // u16 index of the stage table in the pool (x8)
  uint32_t row_first;    // first row of the stage within its group
  uint16_t nrows;        // rows in the stage (<= 32)
  uint16_t nsub;         // subgroups (<= 4)
  uint16_t table_bytes;  // bytes of the stage table (multiple of 16)
  uint16_t nitems;       // phase-A work items
  uint32_t bmin[4];      // window start of each subgroup relative to t0 (x4)
  uint8_t row_sub[32];   // subgroup of each row
};
static_assert(sizeof(SharedStage) == 64, "stage descriptor layout");
constexpr int kSharedRows = 8;

// Device status word bits, set with atomicOr by a kernel.
enum : uint32_t {
  kStatusTimeout = 1u,  // a bounded wait on a bulk copy ran out
};

// Everything a kernel needs to compute one problem.
struct ProblemDesc {
  const uint8_t *in;
  float *out;
  const GroupDesc *groups;
  const EntryDesc *entries;
  uint32_t *status;
  uint64_t row_bytes;      // input row pitch in bytes (also the clamp)
  uint64_t out_dm_stride;  // floats between consecutive DM rows of a group
  uint32_t nr_groups;
  uint32_t nr_dms;
  uint32_t nr_samples;     // output samples per DM row
  uint32_t bits;           // 1, 2, 4, 8, 16 or 32 (float)
  float first_dm;
  float dm_step;
  uint32_t win_samples;    // samples staged per row and tile (kFamilyTmem32: rows
                           // per group the shared memory holds)
  uint32_t tiles_t;        // time tiles per group
  uint32_t tiles_d;        // DM tiles per group
  uint32_t tma;            // 1: rows staged by bulk async copies
  uint32_t out_vec4;       // 1: float4 stores are aligned
  uint32_t mul_hi8;        // always 1 << 24 (w >> 8 as a high-half multiply)
  uint32_t delay_rows;     // rows of the delay table below
  // Optional precomputed delays (NULL: computed on the device).  For DM
  // tile t (first DM d0), delay row r and j < tile_d:
  //   delay_rel[(t * delay_rows + r) * tile_d + j]
  //       = delay(r, min(d0 + j, nr_dms - 1)) - delay(r, d0)
  const uint16_t *delay_rel;
  // Shared-partial-sum family only (NULL otherwise).
  const uint4 *stage_rows;      // [group][stage][32] row slots (dd_shared.cuh)
  uint32_t stage_count;         // stages of one group (all DM tiles)
  const uint32_t *tile_stage;   // [tiles_d + 1]: first stage of each DM tile
  const uint16_t *pool;         // stage tables
  uint32_t cw;                  // words per shifted copy of a staged row (even)
  uint32_t psw;                 // words per copy of one partial-sum series
  uint32_t slots;               // partial-sum series slots per stage
  uint32_t table_bytes;         // largest stage table (multiple of 16)
  // Detection statistics of the output rows (NULL: not requested): per row
  // {sum, sum of squares, peak << 32 | (0xffffffff - sample)}, accumulated
  // with atomics by the shared-partial-sum kernel.
  unsigned long long *accum;
  // Packed subband intermediate (0: float rows).  Step one with packed = 1
  // writes, per pair of coarse DMs (2p, 2p + 1), one 32-bit word per sample:
  // the exact sum of DM 2p in the low 16 bits, of DM 2p + 1 in the high 16
  // (0 where 2p + 1 is past the last coarse DM); row (beam, p, subband) at
  // ((beam * pairs + p) * subbands + subband) * out_row words.  The pair
  // kernel (step two) reads those rows: group (synthesized beam, p) writes
  // DM rows d of coarse DM 2p at out_offset + d * out_dm_stride and of coarse
  // DM 2p + 1 pair_stride floats further on.
  // Tiles of a launch.  With ttile_count = 0 a launch of G CTAs computes
  // tiles [tile_base, tile_base + G) of the problem's (group, DM tile, time
  // tile) order.  With ttile_count > 0 it computes, for every (group, DM
  // tile), the time tiles [ttile_base, ttile_base + ttile_count).
  uint32_t tile_base;
  uint32_t ttile_base, ttile_count;
  // 1: launched as a programmatic dependent of the stream's previous kernel
  // (dd_plan_set_overlap): the kernel lets the next launch start early and
  // waits for the previous one before its first global write.
  uint32_t overlap;
  uint32_t packed;
  uint32_t pair_groups;   // pairs of coarse DMs (groups per synthesized beam)
  uint32_t pair_d1;       // coarse DMs
  uint32_t flush_rows;    // rows summed in 16-bit lanes before widening
  uint64_t pair_stride;   // floats from a coarse DM 2p row to its 2p + 1 row
  // Limit of each bounded wait for a staged copy, in ns (0: the default of
  // 2 s; below 1000: give up as soon as the first test of the barrier finds
  // the copy not landed).  The test of the timeout path sets it
  // (dd_plan_set_wait_limit).  The drain after a timeout keeps its own
  // limit, so every copy in flight lands before a CTA exits.
  uint32_t wait_ns;
  // kFamilyTmem32: the offsets of every (DM tile, delay row), 20 words each
  // (dd_tmem.cuh, tmem_tables); rows are entries' delay_row.
  const uint4 *tmem_tab;
};

// One entry of the kernel registry: a compiled tile configuration.
struct KernelInfo {
  const char *name;
  int family;       // kFamilySwar8, kFamilyScalar, kFamilyShared8, kFamilyPair16, kFamilyTmem32
  int elem_bits;    // swar8: 8 (covers 1/2/4/8); scalar: 16 or 32
  int items_t;      // samples per thread
  int items_d;      // DMs per thread
  int warps_d;      // warps along the DM axis
  int channels;     // rows per pipeline stage
  int threads;
  int tile_t;       // samples per tile
  int tile_d;       // DMs per tile
  int variant;      // swar8 inner loop (kUnpackMaskHigh / kUnpackPermute)
  const void *func;
  void (*launch)(const ProblemDesc &, unsigned grid, size_t smem,
                 cudaStream_t stream);
  int max_rows;     // rows a group may have (0: any)
};

enum { kFamilySwar8 = 0, kFamilyScalar = 1, kFamilyShared8 = 2, kFamilyPair16 = 3, kFamilyTmem32 = 4 };

// Registry of compiled configurations (dd_kernels.cu).
const KernelInfo *kernel_registry(int *count);
// Dynamic shared memory bytes of a configuration for a window size.
size_t kernel_smem_bytes(const KernelInfo &k, uint32_t win_samples,
                         uint32_t bits);
// Samples a window must hold beyond the tile for row alignment.
uint32_t window_alignment_samples(uint32_t bits);

// Delay of a row for one DM, in the reference's float order
// ((firstDM + dm * dmStep) * shift, truncated; include/Dedispersion.hpp:81).
// Host version; the device version is in dd_device.cuh.
inline uint32_t host_delay(float first_dm, float dm_step, uint32_t dm,
                           float shift) {
  volatile float step_dm = static_cast<float>(dm) * dm_step;
  volatile float dm_value = first_dm + step_dm;
  volatile float product = dm_value * shift;
  return static_cast<uint32_t>(product);
}

}  // namespace dd
