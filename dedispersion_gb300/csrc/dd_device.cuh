// dd_device.cuh -- sm_103a device code of the dedispersion tile kernels.
//
// One CTA computes one tile: TILE_D DMs x TILE_T output samples of one output
// group (dd_internal.h).  For every input row of the group (a live channel,
// or a subband in step two) the CTA needs the row window
//
//   [t0 + delay(row, d0), t0 + TILE_T + delay(row, d0 + TILE_D - 1))
//
// It stages CH rows per pipeline stage into shared memory with bulk async
// copies (cp.async.bulk, the 1-D TMA path; no multicast), completion tracked
// by an mbarrier per staging slot, three slots in flight.  The device twin of
// the reference's local-memory kernel (include/Dedispersion.hpp:225-309),
// which copies each channel's window into __local memory.
//
// Three tile families:
//
// * swar8 (input of 1, 2, 4 or 8 bits).  Rows are expanded to one byte per
//   sample while staged and kept as four copies shifted by 0..3 bytes, so a
//   window read at any sample offset is one aligned 32-bit load.  A loaded
//   word holds four consecutive samples; two byte permutes spread them over
//   two registers of two 16-bit lanes, and integer adds accumulate two
//   samples per lane pair (SWAR).  16-bit lanes are flushed into 32-bit
//   totals every 256 rows (256 * 255 < 2^16), so sums are exact integers.
//
// * scalar (16-bit or float input, and step two).  Element loads at any
//   offset; 16-bit input accumulates in uint32, float input in float32 in row
//   order, the reference's own order (include/Dedispersion.hpp:79-104), so
//   float results are identical to the reference's.
//
// * pair (step two over the packed subband intermediate, ProblemDesc::
//   packed).  A 32-bit word holds the 16-bit step-one sums of two coarse
//   DMs; one load and one add serve both.
//
// Every wait on a bulk copy is bounded (kWaitNs); when one runs out the CTA
// sets kStatusTimeout in the problem's status word, waits a bounded time for
// its other copies, and returns.
#pragma once

#include <cstdint>

#include "dd_internal.h"

namespace dd {

constexpr int kNRaw = 3;                            // staging slots
constexpr unsigned long long kWaitNs = 2000000000ull;  // 2 s per bulk copy
constexpr unsigned long long kDrainNs = 50000000ull;   // 50 ms when aborting

__host__ __device__ inline uint32_t round_up(uint32_t v, uint32_t m) {
  return (v + m - 1) / m * m;
}

// Samples per 16 bytes of a row: the alignment of a staged window's start.
__host__ __device__ inline uint32_t align_samples(uint32_t bits) {
  return bits <= 8 ? 16u * (8u / bits) : 16u / (bits / 8u);
}

// Shared memory layout of one CTA (byte offsets from the dynamic base).
struct SmemLayout {
  uint32_t raw_bytes;   // bytes fetched per staged row
  uint32_t raw_stride;  // bytes between raw slots (>= raw_bytes)
  uint32_t copy_words;  // words of one shifted copy (swar8)
  uint32_t area_words;  // words between copy areas (>= CH * 4 * copy_words)
  uint32_t off_bar, off_wstart, off_table, off_raw, off_copy, total;
};

__host__ __device__ inline SmemLayout make_layout(int family, uint32_t win,
                                                  uint32_t bits, int ch,
                                                  int tile_d) {
  SmemLayout L;
  const uint32_t a = align_samples(bits);
  if (family == kFamilySwar8) {
    L.raw_bytes = round_up((win + a) * bits / 8u, 16u);
    L.copy_words = win / 4u;
  } else {
    L.raw_bytes = round_up(win * (bits / 8u), 16u);
    L.copy_words = 0;
  }
  L.off_bar = 0;
  L.off_wstart = 64;
  L.off_table = round_up(L.off_wstart + 2u * kNRaw * ch * 4u, 128u);
  L.off_raw = round_up(L.off_table + 2u * ch * tile_d * 4u, 128u);
  L.raw_stride = L.raw_bytes;
  L.area_words = ch * 4u * L.copy_words;
  L.off_copy = round_up(L.off_raw + kNRaw * ch * L.raw_stride, 128u);
  L.total = L.off_copy + 2u * L.area_words * 4u;
  return L;
}

// ---- PTX wrappers ---------------------------------------------------------

__device__ __forceinline__ uint32_t smem_addr(const void *p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)),
               "r"(count)
               : "memory");
}

__device__ __forceinline__ void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t *bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_addr(bar))
               : "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar,
                                                      uint32_t bytes) {
  asm volatile(
      "mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(
          smem_addr(bar)),
      "r"(bytes)
      : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_addr(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// Programmatic dependent launch: let the stream's next grid begin launching
// (once every CTA of this grid has issued this or exited), and wait until
// the previous grid has completed and its writes are visible.
__device__ __forceinline__ void allow_dependents() {
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}
__device__ __forceinline__ void wait_prerequisites() {
  asm volatile("griddepcontrol.wait;" ::: "memory");
}

__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Non-blocking test of the phase with `parity`.
__device__ __forceinline__ bool mbar_test_wait(uint64_t *bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_addr(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// Bounded wait for the phase with `parity` to complete.  `test_ns` is the
// problem's override of the limit (ProblemDesc::wait_ns, 0: `limit_ns`),
// read only once the first try has failed so that the common path stays
// as short as it was; an override below a microsecond gives up right after
// that first try.
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity,
                                          unsigned long long limit_ns,
                                          uint32_t test_ns = 0) {
  if (mbar_try_wait(bar, parity)) return true;
  if (test_ns) {
    if (test_ns < 1000u) return false;
    limit_ns = test_ns;
  }
  const unsigned long long start = global_ns();
  for (;;) {
#pragma unroll 1
    for (int i = 0; i < 32; ++i)
      if (mbar_try_wait(bar, parity)) return true;
    if (global_ns() - start > limit_ns) return false;
  }
}

// 1-D bulk copy global -> shared, completing `bytes` on `bar`.  Both
// addresses 16-byte aligned, bytes a multiple of 16.
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src,
                                         uint32_t bytes, uint64_t *bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes "
      "[%0], [%1], %2, [%3];" ::"r"(smem_addr(dst)),
      "l"(src), "r"(bytes), "r"(smem_addr(bar))
      : "memory");
}

// The reference's per-row delay, (uint)((firstDM + dm * dmStep) * shift),
// with every operation rounded as the CPU rounds it (no contraction).
__device__ __forceinline__ uint32_t dev_delay(float first, float step,
                                              uint32_t dm, float shift) {
  const float v = __fadd_rn(first, __fmul_rn(__uint2float_rn(dm), step));
  return __float2uint_rz(__fmul_rn(v, shift));
}

// Samples 4k..4k+3 of a packed sub-byte row, one per byte, zero-extended.
// Sample n lives in byte n / (8 / bits) at bit (n % (8 / bits)) * bits.
__device__ __forceinline__ uint32_t expand_word(const uint8_t *row, uint32_t k,
                                                uint32_t bits) {
  if (bits == 4) {
    // [s1 s0][s3 s2] -> bytes (b0, b0, b1, b1), then the low nibble of
    // bytes 0 and 2 and the high nibble of bytes 1 and 3.
    const uint32_t t = __byte_perm(reinterpret_cast<const uint16_t *>(row)[k], 0, 0x1100);
    return (t & 0x000F000Fu) | ((t >> 4) & 0x0F000F00u);
  }
  if (bits == 2) {
    // Samples 0 and 2 (bits 0-1, 4-5) and 1 and 3 (bits 2-3, 6-7) are moved
    // into place by two multiplies of disjoint shifted copies (no carries).
    const uint32_t v = row[k];
    return (((v & 0x33u) * 0x1001u) & 0x00030003u) | (((v & 0xCCu) * 0x40040u) & 0x03000300u);
  }
  const uint32_t v = (row[k >> 1] >> ((k & 1u) * 4u)) & 0xFu;
  uint32_t out = 0;
#pragma unroll
  for (int s = 0; s < 4; ++s) out |= ((v >> s) & 1u) << (8 * s);
  return out;
}

// ---- staging shared by both families --------------------------------------

struct StageCtx {
  uint64_t *bars;
  uint32_t *wstart;  // first staged sample of each row of a slot
  uint32_t *wmod;    // t0 + delay(row, first DM of the tile) - wstart
  uint8_t *raw;
  uint32_t raw_bytes;   // fetched per row
  uint32_t raw_stride;  // between slots
};

// Issue stage `s` (global stage index gs) of group G: lanes 0..CH-1 of the
// calling warp each stage one row.  Every lane < CH arrives once.
template <int CH>
__device__ __forceinline__ void issue_stage(const ProblemDesc &P,
                                            const GroupDesc &G,
                                            const StageCtx &S, uint32_t s,
                                            uint32_t gs, uint32_t t0,
                                            uint32_t d0, uint32_t dtile,
                                            int lane) {
  if (lane >= CH) return;
  const uint32_t slot = gs % kNRaw;
  uint64_t *bar = S.bars + slot;
  const uint32_t e = s * CH + lane;
  if (e >= G.entry_count) {
    mbar_arrive(bar);
    return;
  }
  const EntryDesc E = P.entries[G.entry_begin + e];
  const uint32_t a = align_samples(P.bits);
  // One delay per row and stage: computed here rather than loaded, keeping
  // global latency off the issuing warp (equal to the host's delay_base).
  (void)dtile;
  const uint32_t base = dev_delay(P.first_dm, P.dm_step, d0, E.shift);
  const uint32_t ws = (t0 + base) / a * a;
  S.wstart[slot * CH + lane] = ws;
  S.wmod[slot * CH + lane] = t0 + base - ws;
  if (P.tma) {
    const uint64_t boff = P.bits <= 8 ? (uint64_t)ws * P.bits / 8u
                                      : (uint64_t)ws * (P.bits / 8u);
    const uint64_t avail = P.row_bytes - boff;
    const uint32_t bytes =
        avail < S.raw_bytes ? static_cast<uint32_t>(avail) : S.raw_bytes;
    mbar_arrive_expect_tx(bar, bytes);
    bulk_g2s(S.raw + (slot * CH + lane) * S.raw_stride,
             P.in + E.row_offset + boff, bytes, bar);
  } else {
    mbar_arrive(bar);
  }
}

// Start of the precomputed relative delays of stage s (NULL if absent).
__device__ __forceinline__ const uint16_t *stage_rel(const ProblemDesc &P,
                                                     const GroupDesc &G,
                                                     uint32_t s, int CH,
                                                     uint32_t dtile, int tile_d) {
  if (!P.delay_rel) return nullptr;
  const uint32_t row0 = P.entries[G.entry_begin + s * CH].delay_row;
  return P.delay_rel + ((size_t)dtile * P.delay_rows + row0) * tile_d;
}

// The (row, DM) table entries of one stage that a thread fills, and the
// precomputed delays for them, loaded one stage ahead so that their global
// latency hides behind the current stage's sums.  Entry idx = tid + r * THREADS.
template <int CH, int TILE_D, int THREADS>
struct StageDelays {
  static constexpr int R = (CH * TILE_D + THREADS - 1) / THREADS;
  uint32_t v[R];

  __device__ __forceinline__ void load(const ProblemDesc &P, const GroupDesc &G, uint32_t s,
                                       uint32_t dtile, uint32_t cnt) {
    const uint16_t *rel = stage_rel(P, G, s, CH, dtile, TILE_D);
    if (!rel) return;
#pragma unroll
    for (int r = 0; r < R; ++r) {
      const uint32_t idx = threadIdx.x + r * THREADS;
      v[r] = idx < cnt * TILE_D ? rel[idx] : 0u;
    }
  }

  // Sample offset of entry r from the start of its row's staged window.
  __device__ __forceinline__ uint32_t offset(const ProblemDesc &P, const GroupDesc &G,
                                             const StageCtx &S, int r, uint32_t s,
                                             uint32_t slot, uint32_t t0, uint32_t d0) const {
    const uint32_t idx = threadIdx.x + r * THREADS;
    const uint32_t ch = idx / TILE_D, j = idx % TILE_D;
    if (P.delay_rel) return v[r] + S.wmod[slot * CH + ch];
    const uint32_t d = (d0 + j) < P.nr_dms ? (d0 + j) : (P.nr_dms - 1);
    const float sh = P.entries[G.entry_begin + s * CH + ch].shift;
    return t0 + dev_delay(P.first_dm, P.dm_step, d, sh) - S.wstart[slot * CH + ch];
  }
};

__device__ __forceinline__ uint32_t lds_u32(uint32_t addr) {
  uint32_t v;
  asm volatile("ld.shared.b32 %0, [%1];" : "=r"(v) : "r"(addr));
  return v;
}

// Without bulk copies (unaligned rows): the CTA copies the windows of one
// stage byte by byte; bytes past the row end read as zero.
template <int CH, int TY>
__device__ __forceinline__ void copy_stage_plain(const ProblemDesc &P,
                                                 const GroupDesc &G,
                                                 const StageCtx &S, uint32_t s,
                                                 uint32_t slot, uint32_t cnt) {
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
  for (uint32_t ch = ty; ch < cnt; ch += TY) {
    const EntryDesc E = P.entries[G.entry_begin + s * CH + ch];
    const uint32_t ws = S.wstart[slot * CH + ch];
    const uint64_t boff = P.bits <= 8 ? (uint64_t)ws * P.bits / 8u
                                      : (uint64_t)ws * (P.bits / 8u);
    const uint8_t *src = P.in + E.row_offset;
    uint8_t *dst = S.raw + (slot * CH + ch) * S.raw_stride;
    for (uint32_t b = tx; b < S.raw_bytes; b += 32)
      dst[b] = (boff + b < P.row_bytes) ? src[boff + b] : 0;
  }
}

// Abort path: wait a bounded time for stages [from, to) still in flight.
__device__ __forceinline__ void drain_stages(const StageCtx &S, uint32_t sc,
                                             uint32_t from, uint32_t to) {
  for (uint32_t s = from; s < to; ++s) {
    const uint32_t gs = sc + s;
    (void)mbar_wait(S.bars + gs % kNRaw, (gs / kNRaw) & 1u, kDrainNs);
  }
}

// Test hook of the timeout path (ProblemDesc::wait_ns of 1..999 ns), right
// after the prologue has issued stages [0, pro): one non-blocking test of
// stage 0's barrier.  A copy that has not landed yet -- the common case this
// early -- sends the CTA down the path a wait that runs out takes: the status
// bit, a bounded drain of the stages in flight, an early return (true).  It
// sits outside the stage loop, so the loop's code is the same with or
// without it.
__device__ __forceinline__ bool timeout_test_hook(const ProblemDesc &P, const StageCtx &S,
                                                  uint32_t sc, uint32_t pro) {
  const bool ok = mbar_test_wait(S.bars + sc % kNRaw, (sc / kNRaw) & 1u);
  if (!__syncthreads_or(!ok)) return false;
  if (threadIdx.x == 0) atomicOr(P.status, kStatusTimeout);
  drain_stages(S, sc, 0, pro);
  return true;
}

// Whether a problem asks for the timeout test hook.
__device__ __forceinline__ bool timeout_test(const ProblemDesc &P) {
  return P.wait_ns - 1u < 999u;
}

// ---- swar8 tile -----------------------------------------------------------

// Inner-loop variants of the swar8 family.  Both keep sums exact.
//
// kUnpackPermute: two byte permutes spread a word's samples (b0 b1 b2 b3)
//   into two registers of 16-bit lanes, (b0, b1) and (b2, b3), and integer
//   adds accumulate them (all on the integer ALU pipe).
// kUnpackMaskHigh: one AND keeps the even samples, E += w & 0x00FF00FF
//   (lanes b0, b2), and one high-half multiply-add on the FMA pipe adds
//   w >> 8 = b1 + 2^8 b2 + 2^16 b3 to a plain 32-bit sum A.  After at most
//   256 rows A = S1 + 2^8 S2 + 2^16 S3 < 2^32 exactly; S2 is E's high lane, so
//   A - (S2 << 8) = S1 + 2^16 S3 with S1 < 2^16 splits into S1 and S3.
// kUnpackPermuteMad: the permutes of kUnpackPermute, with both accumulations
//   issued as multiply-adds by one on the FMA pipe.
// kUnpackPermuteHalf: the (b0, b1) accumulation as integer adds, the
//   (b2, b3) one as multiply-adds, splitting the adds over both pipes.
enum {
  kUnpackPermute = 0,
  kUnpackMaskHigh = 1,
  kUnpackPermuteMad = 2,
  kUnpackPermuteHalf = 3
};

__device__ __forceinline__ uint32_t mad_hi(uint32_t a, uint32_t b, uint32_t c) {
  uint32_t d;
  asm("mad.hi.u32 %0, %1, %2, %3;" : "=r"(d) : "r"(a), "r"(b), "r"(c));
  return d;
}

// a * b + c on the FMA pipe; with b = 1 (a run-time value, so that the
// compiler cannot turn it back into an add) it is an add off the ALU pipe.
__device__ __forceinline__ uint32_t mad_lo(uint32_t a, uint32_t b, uint32_t c) {
  uint32_t d;
  asm("mad.lo.u32 %0, %1, %2, %3;" : "=r"(d) : "r"(a), "r"(b), "r"(c));
  return d;
}

// Computes one tile; returns false if the CTA must stop (timeout).  `sc`
// counts the CTA's stages across tiles (mbarrier phase bookkeeping).
// SHORT: every group has at most 257 rows (the host checks), so the 16-bit
// lanes never pass 2^16 - 1 (257 * 255 = 65535) and need no 32-bit totals:
// the registers those would take hold more samples per thread instead.
template <int NW, int NDT, int TY, int CH, int VAR, bool SHORT = false>
__device__ __forceinline__ bool swar8_tile(const ProblemDesc &P,
                                           const GroupDesc &G, uint32_t dtile,
                                           uint32_t ttile, uint8_t *smem,
                                           const SmemLayout &L, uint32_t &sc) {
  constexpr int kTileT = 32 * NW * 4;
  constexpr int kTileD = TY * NDT;
  constexpr int kThreads = 32 * TY;
  static_assert(CH <= 32 && CH % 2 == 0, "CH rows per stage, even, <= 32");
  static_assert(!SHORT || VAR != kUnpackMaskHigh, "short groups read lanes (b0, b1), (b2, b3)");
  const int tid = threadIdx.x, tx = tid & 31, ty = tid >> 5;
  const uint32_t t0 = ttile * kTileT, d0 = dtile * kTileD;
  const uint32_t K = G.entry_count;
  const uint32_t nst = (K + CH - 1) / CH;
  const uint32_t cw = L.copy_words;
  const uint32_t mul = P.mul_hi8;
  const uint32_t one = P.mul_hi8 >> 24;  // 1, unknown to the compiler
  StageCtx S;
  S.bars = reinterpret_cast<uint64_t *>(smem + L.off_bar);
  S.wstart = reinterpret_cast<uint32_t *>(smem + L.off_wstart);
  S.wmod = S.wstart + kNRaw * CH;
  S.raw = smem + L.off_raw;
  S.raw_bytes = L.raw_bytes;
  S.raw_stride = L.raw_stride;
  uint32_t *table = reinterpret_cast<uint32_t *>(smem + L.off_table);
  uint32_t *copies = reinterpret_cast<uint32_t *>(smem + L.off_copy);

  if (ty == 0) {
    const uint32_t pro = nst < (uint32_t)kNRaw ? nst : (uint32_t)kNRaw;
    for (uint32_t s = 0; s < pro; ++s)
      issue_stage<CH>(P, G, S, s, sc + s, t0, d0, dtile, tx);
  }
  if (timeout_test(P) && nst &&
      timeout_test_hook(P, S, sc, nst < (uint32_t)kNRaw ? nst : (uint32_t)kNRaw))
    return false;

  // kUnpackPermute: lo = (b0, b1) lanes, hi = (b2, b3) lanes.
  // kUnpackMaskHigh: lo = E (b0, b2 lanes), hi = A (w >> 8 sum).
  constexpr int TJ = SHORT ? 1 : NDT, TI = SHORT ? 1 : NW;
  uint32_t lo[NDT][NW], hi[NDT][NW], tot[TJ][TI][4];
#pragma unroll
  for (int j = 0; j < NDT; ++j)
#pragma unroll
    for (int i = 0; i < NW; ++i) lo[j][i] = hi[j][i] = 0;
#pragma unroll
  for (int j = 0; j < TJ; ++j)
#pragma unroll
    for (int i = 0; i < TI; ++i)
      tot[j][i][0] = tot[j][i][1] = tot[j][i][2] = tot[j][i][3] = 0;
  // Sample k (0..3) of word i of DM j: from the totals, or for short groups
  // straight from the 16-bit lanes.
  auto lane = [&](int j, int i, int k) -> uint32_t {
    if constexpr (SHORT) {
      const uint32_t v = k < 2 ? lo[j][i] : hi[j][i];
      return (k & 1) ? v >> 16 : v & 0xFFFFu;
    } else {
      return tot[j][i][k];
    }
  };
  uint32_t since = 0;
  using Delays = StageDelays<CH, kTileD, kThreads>;
  Delays delays;
  if (nst) delays.load(P, G, 0, dtile, K < (uint32_t)CH ? K : CH);

  auto flush = [&]() {
    if constexpr (!SHORT) {
#pragma unroll
      for (int j = 0; j < NDT; ++j)
#pragma unroll
        for (int i = 0; i < NW; ++i) {
          if (VAR != kUnpackMaskHigh) {
            tot[j][i][0] += lo[j][i] & 0xFFFFu;
            tot[j][i][1] += lo[j][i] >> 16;
            tot[j][i][2] += hi[j][i] & 0xFFFFu;
            tot[j][i][3] += hi[j][i] >> 16;
          } else {
            const uint32_t s2 = lo[j][i] >> 16;
            const uint32_t x = hi[j][i] - (s2 << 8);
            tot[j][i][0] += lo[j][i] & 0xFFFFu;
            tot[j][i][1] += x & 0xFFFFu;
            tot[j][i][2] += s2;
            tot[j][i][3] += x >> 16;
          }
          lo[j][i] = hi[j][i] = 0;
        }
    }
  };

  for (uint32_t s = 0; s < nst; ++s) {
    const uint32_t gs = sc + s, slot = gs % kNRaw, area = gs & 1u;
    const uint32_t cnt = (K - s * CH) < (uint32_t)CH ? (K - s * CH) : CH;
    const bool ok = mbar_wait(S.bars + slot, (gs / kNRaw) & 1u, kWaitNs, P.wait_ns);
    if (!P.tma) {
      copy_stage_plain<CH, TY>(P, G, S, s, slot, cnt);
      __syncthreads();
    }
    // Expand to bytes and write the four shifted copies of each row, two
    // words per thread and step (copy m word k = samples 4k+m .. 4k+m+3).
    uint32_t *ac = copies + area * L.area_words;
    for (uint32_t ch = ty; ch < cnt; ch += TY) {
      const uint8_t *r = S.raw + (slot * CH + ch) * S.raw_stride;
      uint32_t *dst = ac + ch * 4u * cw;
      for (uint32_t k = 2 * tx; k < cw; k += 64) {
        uint32_t w0, w1, w2;
        if (P.bits == 8) {
          const uint2 v = *reinterpret_cast<const uint2 *>(r + 4 * k);
          w0 = v.x;
          w1 = v.y;
          w2 = reinterpret_cast<const uint32_t *>(r)[k + 2];
        } else {
          w0 = expand_word(r, k, P.bits);
          w1 = expand_word(r, k + 1, P.bits);
          w2 = expand_word(r, k + 2, P.bits);
        }
        *reinterpret_cast<uint2 *>(dst + k) = make_uint2(w0, w1);
        *reinterpret_cast<uint2 *>(dst + cw + k) =
            make_uint2(__funnelshift_r(w0, w1, 8), __funnelshift_r(w1, w2, 8));
        *reinterpret_cast<uint2 *>(dst + 2 * cw + k) =
            make_uint2(__funnelshift_r(w0, w1, 16), __funnelshift_r(w1, w2, 16));
        *reinterpret_cast<uint2 *>(dst + 3 * cw + k) =
            make_uint2(__funnelshift_r(w0, w1, 24), __funnelshift_r(w1, w2, 24));
      }
    }
    // Byte offset of (row, DM) in the copy area: copy (o & 3), word (o >> 2).
    uint32_t *tb = table + area * (CH * kTileD);
#pragma unroll
    for (int r = 0; r < Delays::R; ++r) {
      const uint32_t idx = tid + r * kThreads;
      if (idx < cnt * kTileD) {
        const uint32_t ch = idx / kTileD;
        const uint32_t o = delays.offset(P, G, S, r, s, slot, t0, d0);
        tb[idx] = 4u * (ch * 4u * cw + (o & 3u) * cw + (o >> 2));
      }
    }
    if (__syncthreads_or(!ok)) {
      if (tid == 0) atomicOr(P.status, kStatusTimeout);
      const uint32_t last = (s + kNRaw) < nst ? (s + kNRaw) : nst;
      drain_stages(S, sc, s, last);
      return false;
    }
    if (ty == 0 && s + kNRaw < nst)
      issue_stage<CH>(P, G, S, s + kNRaw, gs + kNRaw, t0, d0, dtile, tx);
    if (s + 1 < nst)
      delays.load(P, G, s + 1, dtile, (K - (s + 1) * CH) < (uint32_t)CH ? (K - (s + 1) * CH) : CH);

    if (since + cnt > 256u) {
      flush();
      since = 0;
    }
    since += cnt;

    // 32-bit shared addresses: one add per (row, DM), immediates per word.
    const uint32_t *tbt = tb + ty * NDT;
    const uint32_t acs = smem_addr(ac) + 4u * tx;
    uint32_t ch = 0;
    for (; ch + 1 < cnt; ch += 2) {
      uint32_t p1[NDT], p2[NDT];
#pragma unroll
      for (int j = 0; j < NDT; ++j) {
        p1[j] = acs + tbt[ch * kTileD + j];
        p2[j] = acs + tbt[(ch + 1) * kTileD + j];
      }
#pragma unroll
      for (int j = 0; j < NDT; ++j)
#pragma unroll
        for (int i = 0; i < NW; ++i) {
          const uint32_t w1 = lds_u32(p1[j] + 128u * i);
          const uint32_t w2 = lds_u32(p2[j] + 128u * i);
          if (VAR == kUnpackPermute) {
            lo[j][i] += __byte_perm(w1, 0, 0x4140) + __byte_perm(w2, 0, 0x4140);
            hi[j][i] += __byte_perm(w1, 0, 0x4342) + __byte_perm(w2, 0, 0x4342);
          } else if (VAR == kUnpackMaskHigh) {
            lo[j][i] += (w1 & 0x00FF00FFu) + (w2 & 0x00FF00FFu);
            hi[j][i] = mad_hi(w2, mul, mad_hi(w1, mul, hi[j][i]));
          } else if (VAR == kUnpackPermuteMad) {
            lo[j][i] = mad_lo(__byte_perm(w2, 0, 0x4140), one,
                              mad_lo(__byte_perm(w1, 0, 0x4140), one, lo[j][i]));
            hi[j][i] = mad_lo(__byte_perm(w2, 0, 0x4342), one,
                              mad_lo(__byte_perm(w1, 0, 0x4342), one, hi[j][i]));
          } else {
            lo[j][i] += __byte_perm(w1, 0, 0x4140) + __byte_perm(w2, 0, 0x4140);
            hi[j][i] = mad_lo(__byte_perm(w2, 0, 0x4342), one,
                              mad_lo(__byte_perm(w1, 0, 0x4342), one, hi[j][i]));
          }
        }
    }
    if (ch < cnt) {
#pragma unroll
      for (int j = 0; j < NDT; ++j) {
        const uint32_t p = acs + tbt[ch * kTileD + j];
#pragma unroll
        for (int i = 0; i < NW; ++i) {
          const uint32_t w = lds_u32(p + 128u * i);
          if (VAR == kUnpackMaskHigh) {
            lo[j][i] += w & 0x00FF00FFu;
            hi[j][i] = mad_hi(w, mul, hi[j][i]);
          } else {
            lo[j][i] += __byte_perm(w, 0, 0x4140);
            hi[j][i] += __byte_perm(w, 0, 0x4342);
          }
        }
      }
    }
  }
  sc += nst;
  flush();
  // An overlapped launch writes only after the previous grid completed.
  if (P.overlap) wait_prerequisites();

  if (P.packed) {
    // Pairs (2p, 2p + 1) of the thread's DMs (d0 and NDT even): exact sums
    // below 2^16, the host checked.
    static_assert(NDT % 2 == 0, "DM pairs per thread");
#pragma unroll
    for (int j = 0; j < NDT; j += 2) {
      const uint32_t d = d0 + ty * NDT + j;
      if (d >= P.nr_dms) continue;
      const bool hi_ok = d + 1u < P.nr_dms;
      uint32_t *orow = reinterpret_cast<uint32_t *>(P.out) + G.out_offset +
                       (uint64_t)(d >> 1) * P.out_dm_stride;
#pragma unroll
      for (int i = 0; i < NW; ++i) {
        const uint32_t t = t0 + 4u * (tx + 32u * i);
        uint32_t w[4];
#pragma unroll
        for (int k = 0; k < 4; ++k)
          w[k] = t + k < P.nr_samples
                     ? (lane(j, i, k) | (hi_ok ? lane(j + 1, i, k) << 16 : 0u)) : 0u;
        if (P.out_vec4 && t + 3u < P.nr_samples) {
          *reinterpret_cast<uint4 *>(orow + t) = make_uint4(w[0], w[1], w[2], w[3]);
        } else {
#pragma unroll
          for (int k = 0; k < 4; ++k)
            if (t + k < P.nr_samples) orow[t + k] = w[k];
        }
      }
    }
    return true;
  }

#pragma unroll
  for (int j = 0; j < NDT; ++j) {
    const uint32_t d = d0 + ty * NDT + j;
    if (d >= P.nr_dms) continue;
    float *orow = P.out + G.out_offset + (uint64_t)d * P.out_dm_stride;
#pragma unroll
    for (int i = 0; i < NW; ++i) {
      const uint32_t v0 = lane(j, i, 0), v1 = lane(j, i, 1);
      const uint32_t v2 = lane(j, i, 2), v3 = lane(j, i, 3);
      const uint32_t t = t0 + 4u * (tx + 32u * i);
      if (P.out_vec4 && t + 3u < P.nr_samples) {
        *reinterpret_cast<float4 *>(orow + t) =
            make_float4((float)v0, (float)v1, (float)v2, (float)v3);
      } else {
        if (t < P.nr_samples) orow[t] = (float)v0;
        if (t + 1u < P.nr_samples) orow[t + 1] = (float)v1;
        if (t + 2u < P.nr_samples) orow[t + 2] = (float)v2;
        if (t + 3u < P.nr_samples) orow[t + 3] = (float)v3;
      }
    }
  }
  return true;
}

// ---- scalar tile ----------------------------------------------------------

template <typename T>
struct ScalarAcc;
template <>
struct ScalarAcc<uint16_t> {
  using type = uint32_t;
};
template <>
struct ScalarAcc<float> {
  using type = float;
};

// Element load from a 32-bit shared address, widened to the accumulator.
template <typename T>
__device__ __forceinline__ typename ScalarAcc<T>::type lds_elem(uint32_t addr);
template <>
__device__ __forceinline__ uint32_t lds_elem<uint16_t>(uint32_t addr) {
  uint32_t v;
  asm volatile("ld.shared.u16 %0, [%1];" : "=r"(v) : "r"(addr));
  return v;
}
template <>
__device__ __forceinline__ float lds_elem<float>(uint32_t addr) {
  float v;
  asm volatile("ld.shared.f32 %0, [%1];" : "=f"(v) : "r"(addr));
  return v;
}

template <typename T, int NS, int NDT, int TY, int CH>
__device__ __forceinline__ bool scalar_tile(const ProblemDesc &P,
                                            const GroupDesc &G, uint32_t dtile,
                                            uint32_t ttile, uint8_t *smem,
                                            const SmemLayout &L, uint32_t &sc) {
  using Acc = typename ScalarAcc<T>::type;
  constexpr int kTileT = 32 * NS;
  constexpr int kTileD = TY * NDT;
  constexpr int kThreads = 32 * TY;
  constexpr int kAhead = kNRaw - 1;  // raw slots are read by compute
  static_assert(CH <= 32, "CH rows per stage <= 32");
  const int tid = threadIdx.x, tx = tid & 31, ty = tid >> 5;
  const uint32_t t0 = ttile * kTileT, d0 = dtile * kTileD;
  const uint32_t K = G.entry_count;
  const uint32_t nst = (K + CH - 1) / CH;
  StageCtx S;
  S.bars = reinterpret_cast<uint64_t *>(smem + L.off_bar);
  S.wstart = reinterpret_cast<uint32_t *>(smem + L.off_wstart);
  S.wmod = S.wstart + kNRaw * CH;
  S.raw = smem + L.off_raw;
  S.raw_bytes = L.raw_bytes;
  S.raw_stride = L.raw_stride;
  uint32_t *table = reinterpret_cast<uint32_t *>(smem + L.off_table);
  const uint32_t raws = smem_addr(S.raw) + (uint32_t)sizeof(T) * tx;

  if (ty == 0) {
    const uint32_t pro = nst < (uint32_t)kAhead ? nst : (uint32_t)kAhead;
    for (uint32_t s = 0; s < pro; ++s)
      issue_stage<CH>(P, G, S, s, sc + s, t0, d0, dtile, tx);
  }
  if (timeout_test(P) && nst &&
      timeout_test_hook(P, S, sc, nst < (uint32_t)kAhead ? nst : (uint32_t)kAhead))
    return false;

  Acc acc[NDT][NS];
#pragma unroll
  for (int j = 0; j < NDT; ++j)
#pragma unroll
    for (int i = 0; i < NS; ++i) acc[j][i] = Acc(0);
  using Delays = StageDelays<CH, kTileD, kThreads>;
  Delays delays;
  if (nst) delays.load(P, G, 0, dtile, K < (uint32_t)CH ? K : CH);

  for (uint32_t s = 0; s < nst; ++s) {
    const uint32_t gs = sc + s, slot = gs % kNRaw, area = gs & 1u;
    const uint32_t cnt = (K - s * CH) < (uint32_t)CH ? (K - s * CH) : CH;
    const bool ok = mbar_wait(S.bars + slot, (gs / kNRaw) & 1u, kWaitNs, P.wait_ns);
    if (!P.tma) {
      copy_stage_plain<CH, TY>(P, G, S, s, slot, cnt);
      __syncthreads();
    }
    // Byte offset of (row, DM) from the start of the raw slots.
    uint32_t *tb = table + area * (CH * kTileD);
#pragma unroll
    for (int r = 0; r < Delays::R; ++r) {
      const uint32_t idx = tid + r * kThreads;
      if (idx < cnt * kTileD) {
        const uint32_t ch = idx / kTileD;
        const uint32_t o = delays.offset(P, G, S, r, s, slot, t0, d0);
        tb[idx] = (slot * CH + ch) * L.raw_stride + (uint32_t)sizeof(T) * o;
      }
    }
    if (s + 1 < nst)
      delays.load(P, G, s + 1, dtile, (K - (s + 1) * CH) < (uint32_t)CH ? (K - (s + 1) * CH) : CH);
    if (__syncthreads_or(!ok)) {
      if (tid == 0) atomicOr(P.status, kStatusTimeout);
      const uint32_t last = (s + kAhead) < nst ? (s + kAhead) : nst;
      drain_stages(S, sc, s, last);
      return false;
    }
    if (ty == 0 && s + kAhead < nst)
      issue_stage<CH>(P, G, S, s + kAhead, gs + kAhead, t0, d0, dtile, tx);

    const uint32_t *tbt = tb + ty * NDT;
    for (uint32_t ch = 0; ch < cnt; ++ch) {
      uint32_t b[NDT];
#pragma unroll
      for (int j = 0; j < NDT; ++j) b[j] = raws + tbt[ch * kTileD + j];
#pragma unroll
      for (int j = 0; j < NDT; ++j)
#pragma unroll
        for (int i = 0; i < NS; ++i)
          acc[j][i] += lds_elem<T>(b[j] + (uint32_t)(32 * sizeof(T)) * i);
    }
  }
  sc += nst;

#pragma unroll
  for (int j = 0; j < NDT; ++j) {
    const uint32_t d = d0 + ty * NDT + j;
    if (d >= P.nr_dms) continue;
    float *orow = P.out + G.out_offset + (uint64_t)d * P.out_dm_stride;
#pragma unroll
    for (int i = 0; i < NS; ++i) {
      const uint32_t t = t0 + tx + 32u * i;
      if (t < P.nr_samples) orow[t] = (float)acc[j][i];
    }
  }
  return true;
}

// ---- pair tile (step two over a packed intermediate) ----------------------

// Step two of the subband method over the packed step-one rows (words of two
// coarse DMs' 16-bit sums, ProblemDesc::packed): every 32-bit shared load
// feeds one add of two 16-bit lanes, i.e. two of the reference's float adds
// (include/Dedispersion.hpp:166-170), exact because the sums are integers.
// Lanes widen into 32-bit totals every P.flush_rows rows, before they can
// overflow.  Staging, delays and the pipeline are the scalar tile's.
template <int NS, int NDT, int TY, int CH>
__device__ __forceinline__ bool pair_tile(const ProblemDesc &P, uint32_t g,
                                          const GroupDesc &G, uint32_t dtile,
                                          uint32_t ttile, uint8_t *smem,
                                          const SmemLayout &L, uint32_t &sc) {
  constexpr int kTileT = 32 * NS;
  constexpr int kTileD = TY * NDT;
  constexpr int kThreads = 32 * TY;
  constexpr int kAhead = kNRaw - 1;
  static_assert(CH <= 32, "CH rows per stage <= 32");
  const int tid = threadIdx.x, tx = tid & 31, ty = tid >> 5;
  const uint32_t t0 = ttile * kTileT, d0 = dtile * kTileD;
  const uint32_t K = G.entry_count;
  const uint32_t nst = (K + CH - 1) / CH;
  StageCtx S;
  S.bars = reinterpret_cast<uint64_t *>(smem + L.off_bar);
  S.wstart = reinterpret_cast<uint32_t *>(smem + L.off_wstart);
  S.wmod = S.wstart + kNRaw * CH;
  S.raw = smem + L.off_raw;
  S.raw_bytes = L.raw_bytes;
  S.raw_stride = L.raw_stride;
  uint32_t *table = reinterpret_cast<uint32_t *>(smem + L.off_table);
  const uint32_t raws = smem_addr(S.raw) + 4u * tx;

  if (ty == 0) {
    const uint32_t pro = nst < (uint32_t)kAhead ? nst : (uint32_t)kAhead;
    for (uint32_t s = 0; s < pro; ++s)
      issue_stage<CH>(P, G, S, s, sc + s, t0, d0, dtile, tx);
  }
  if (timeout_test(P) && nst &&
      timeout_test_hook(P, S, sc, nst < (uint32_t)kAhead ? nst : (uint32_t)kAhead))
    return false;

  uint32_t acc[NDT][NS], tlo[NDT][NS], thi[NDT][NS];
#pragma unroll
  for (int j = 0; j < NDT; ++j)
#pragma unroll
    for (int i = 0; i < NS; ++i) acc[j][i] = tlo[j][i] = thi[j][i] = 0;
  auto widen = [&]() {
#pragma unroll
    for (int j = 0; j < NDT; ++j)
#pragma unroll
      for (int i = 0; i < NS; ++i) {
        tlo[j][i] += acc[j][i] & 0xFFFFu;
        thi[j][i] += acc[j][i] >> 16;
        acc[j][i] = 0;
      }
  };
  uint32_t since = 0;
  using Delays = StageDelays<CH, kTileD, kThreads>;
  Delays delays;
  if (nst) delays.load(P, G, 0, dtile, K < (uint32_t)CH ? K : CH);

  for (uint32_t s = 0; s < nst; ++s) {
    const uint32_t gs = sc + s, slot = gs % kNRaw, area = gs & 1u;
    const uint32_t cnt = (K - s * CH) < (uint32_t)CH ? (K - s * CH) : CH;
    const bool ok = mbar_wait(S.bars + slot, (gs / kNRaw) & 1u, kWaitNs, P.wait_ns);
    if (!P.tma) {
      copy_stage_plain<CH, TY>(P, G, S, s, slot, cnt);
      __syncthreads();
    }
    uint32_t *tb = table + area * (CH * kTileD);
#pragma unroll
    for (int r = 0; r < Delays::R; ++r) {
      const uint32_t idx = tid + r * kThreads;
      if (idx < cnt * kTileD) {
        const uint32_t ch = idx / kTileD;
        const uint32_t o = delays.offset(P, G, S, r, s, slot, t0, d0);
        tb[idx] = (slot * CH + ch) * L.raw_stride + 4u * o;
      }
    }
    if (s + 1 < nst)
      delays.load(P, G, s + 1, dtile, (K - (s + 1) * CH) < (uint32_t)CH ? (K - (s + 1) * CH) : CH);
    if (__syncthreads_or(!ok)) {
      if (tid == 0) atomicOr(P.status, kStatusTimeout);
      const uint32_t last = (s + kAhead) < nst ? (s + kAhead) : nst;
      drain_stages(S, sc, s, last);
      return false;
    }
    if (ty == 0 && s + kAhead < nst)
      issue_stage<CH>(P, G, S, s + kAhead, gs + kAhead, t0, d0, dtile, tx);

    const uint32_t *tbt = tb + ty * NDT;
    for (uint32_t ch = 0; ch < cnt; ++ch) {
      uint32_t b[NDT];
#pragma unroll
      for (int j = 0; j < NDT; ++j) b[j] = raws + tbt[ch * kTileD + j];
#pragma unroll
      for (int j = 0; j < NDT; ++j)
#pragma unroll
        for (int i = 0; i < NS; ++i) acc[j][i] += lds_u32(b[j] + 128u * i);
      if (++since == P.flush_rows) {
        widen();
        since = 0;
      }
    }
  }
  sc += nst;
  widen();
  if (P.overlap) wait_prerequisites();

  const bool hi_ok = (g % P.pair_groups) * 2u + 1u < P.pair_d1;
#pragma unroll
  for (int j = 0; j < NDT; ++j) {
    const uint32_t d = d0 + ty * NDT + j;
    if (d >= P.nr_dms) continue;
    float *orow = P.out + G.out_offset + (uint64_t)d * P.out_dm_stride;
#pragma unroll
    for (int i = 0; i < NS; ++i) {
      const uint32_t t = t0 + tx + 32u * i;
      if (t < P.nr_samples) {
        orow[t] = (float)tlo[j][i];
        if (hi_ok) orow[P.pair_stride + t] = (float)thi[j][i];
      }
    }
  }
  return true;
}

// Split a linear tile index (offset by P.tile_base) into (group, DM tile,
// time tile); time fastest, over P.ttile_count time tiles from P.ttile_base
// when ttile_count is set.
__device__ __forceinline__ void decode_tile(const ProblemDesc &P,
                                            uint32_t tile, uint32_t &g,
                                            uint32_t &dtile, uint32_t &ttile) {
  tile += P.tile_base;
  const uint32_t nt = P.ttile_count ? P.ttile_count : P.tiles_t;
  ttile = tile % nt + P.ttile_base;
  const uint32_t rest = tile / nt;
  dtile = rest % P.tiles_d;
  g = rest / P.tiles_d;
}

__device__ __forceinline__ void init_barriers(uint8_t *smem,
                                              const SmemLayout &L, int ch) {
  if (threadIdx.x == 0) {
    uint64_t *bars = reinterpret_cast<uint64_t *>(smem + L.off_bar);
    for (int r = 0; r < kNRaw; ++r) mbar_init(bars + r, ch);
    fence_mbar_init();
  }
  __syncthreads();
}

}  // namespace dd
