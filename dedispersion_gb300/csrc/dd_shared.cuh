// dd_shared.cuh -- the shared-partial-sum tile family (kFamilyShared8), for
// input of 1, 2, 4 or 8 bits in single-step form.
//
// The direct form adds every live row into every DM of a tile.  Here the
// rows of a group are cut into subgroups of up to kSharedRows consecutive
// rows (chosen per DM tile on the host).  Within a subgroup, DM d's delays
// are base(d) + rel(row, d); many DMs of a tile share the vector rel(., d)
// (high-frequency rows barely move between DMs), so the tile computes each
// distinct vector's partial sum once,
//
//   P_v[u] = sum_rows in_row[t0 + bmin + u + rel_v(row)]       (phase A)
//
// and every DM adds one series per subgroup at its own offset,
//
//   out[d][t] += P_{v(d)}[t + base(d) - bmin]                  (phase B).
//
// Phase A walks each subgroup's vectors in a chain chosen on the host so
// that consecutive vectors differ in few rows: the first is summed over its
// rows, each next one is the previous minus the rows that moved plus their
// new samples.  The chain is cut in two halves that a lane runs side by
// side (two independent dependency chains per lane).  Integer addition is exact and every intermediate value is a
// sum of samples (non-negative), so the result equals the direct form's bit
// for bit (8-bit rows: P <= 8 * 255, output < 2^24).  On the 1536-channel,
// 2048-DM table the adds per DM-sample drop from 1459 to about 320.
//
// A pipeline stage holds up to kSubMax subgroups (kStageRows rows).  Per
// stage: the rows and the stage table arrive by 16-byte asynchronous copies
// (the last four warps issue them, every thread's arrival counted on the
// slot's mbarrier)
// in one of kSharedSlots slots; the CTA expands them into four byte-shifted copies
// (any window read is one aligned 32-bit load); warps run the chains of
// (subgroup, 31-group chunk) work items, writing each series in two copies
// shifted by one sample (a read at any offset is aligned loads of two 16-bit
// samples); then every thread adds kSubMax series into the 16-bit lanes of
// its DMs (three-input adds; absent subgroups read a zero series), flushed
// into 32-bit totals before a lane could pass 2^16.  Every wait is bounded
// as in the direct families.
#pragma once

#include <cstdint>

#include "dd_device.cuh"

namespace dd {

constexpr int kSubMax = 4;                              // subgroups per stage
constexpr int kSharedSlots = 3;                         // stages staged at once
constexpr int kStageRows = kSubMax * kSharedRows;       // rows per stage
constexpr uint32_t kLaneSeries = 32;                    // series per 16-bit lane (32 * 2040 < 2^16)
constexpr uint32_t kItemsMax = 32;                      // phase-A items per stage
// Stage table (in shared memory; u16 units unless noted):
//   [0] nsub [1] nrows [2] nitems [3 + k] copy words of subgroup k's rows
//   (even, <= cw) [7] 0
//   [8 + 4k] bmin_k lo, [+1] bmin_k hi, [+2] first row of k, [+3] program of k
//   [kTabItems ..)     items: subgroup << 8 | chunk
//   [kTabSeries ..)    u32: per DM of the tile, kSubMax series byte offsets
//                      (from the partial-sum area)
//   programs (u32, 16-byte aligned): n | ng << 16, nA | nB << 16, dst of
//   chain A's first vector, dst of chain B's (~0: no chain B), 8 copy-area
//   byte offsets of A's first vector's rows, 8 of B's, then nA and nB
//   micro-ops of 4 u32: (old byte offset, new byte offset, dst, real); dst is
//   where the series stands after the micro-op, real = 1 when the vector is
//   complete (else dst is the dummy series and nothing is stored); nA == nB
//   whenever chain B exists
constexpr uint32_t kTabItems = 8 + 4 * kSubMax;
constexpr uint32_t kTabSeries = kTabItems + kItemsMax;
static_assert(kTabSeries % 8 == 0, "series offsets 16-byte aligned");

struct SharedLayout {
  uint32_t raw_bytes;  // bytes staged per row
  uint32_t off_table, off_raw, off_copy, zero_copy, off_part, zero_word, dummy_word, total;
};

// Shared memory of one CTA: mbarriers, kSharedSlots stage tables and x
// kStageRows raw rows, the shifted copies of one stage's rows (and one zero
// row, which rows past a subgroup's end and no-op micro-ops read), `slots`
// partial-sum series (two copies each), one zero series (read for absent
// subgroups) and one dummy series (written by incomplete vectors).  Host and device
// use this one formula.
__host__ __device__ inline SharedLayout make_shared_layout(uint32_t cw, uint32_t psw,
                                                           uint32_t slots,
                                                           uint32_t table_bytes,
                                                           uint32_t bits) {
  SharedLayout L;
  const uint32_t win = 4u * cw + 8u + align_samples(bits);  // samples per row
  L.raw_bytes = round_up(win * bits / 8u, 16u);
  L.off_table = 128;
  L.off_raw = round_up(L.off_table + kSharedSlots * table_bytes, 128u);
  L.off_copy = round_up(L.off_raw + kSharedSlots * kStageRows * L.raw_bytes, 128u);
  L.zero_copy = kStageRows * 4u * cw;  // cw zero words after the copies
  L.off_part = round_up(L.off_copy + (kStageRows * 4u + 1u) * cw * 4u, 128u);
  L.zero_word = 2u * slots * psw;
  L.dummy_word = L.zero_word + psw;
  L.total = L.off_part + (2u * slots + 3u) * psw * 4u;
  return L;
}

__device__ __forceinline__ void sts_v2(uint32_t addr, uint32_t a, uint32_t b) {
  asm volatile("st.shared.v2.b32 [%0], {%1, %2};" ::"r"(addr), "r"(a), "r"(b)
               : "memory");
}

// Predicated store (no branch): writes only where `on` is non-zero.
__device__ __forceinline__ void sts_v2_if(uint32_t on, uint32_t addr, uint32_t a, uint32_t b) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.u32 p, %3, 0;\n\t"
      "@p st.shared.v2.b32 [%0], {%1, %2};\n\t}" ::"r"(addr),
      "r"(a), "r"(b), "r"(on)
      : "memory");
}

__device__ __forceinline__ uint2 lds_v2(uint32_t addr) {
  uint2 v;
  asm volatile("ld.shared.v2.b32 {%0, %1}, [%2];" : "=r"(v.x), "=r"(v.y) : "r"(addr));
  return v;
}

__device__ __forceinline__ void cp_async16(uint32_t dst, const void *src, uint32_t src_bytes) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(dst), "l"(src),
               "r"(src_bytes)
               : "memory");
}

// Arrive on `bar` once every cp.async this thread issued before has landed.
__device__ __forceinline__ void cp_async_arrive(uint64_t *bar) {
  asm volatile("cp.async.mbarrier.arrive.noinc.shared::cta.b64 [%0];" ::"r"(smem_addr(bar))
               : "memory");
}

// Row slot r of a stage (host-built, per group): x, y = byte offset of the
// row in the input, z = its subgroup's window start | kRowPresent, w = u16
// index of the stage table in the pool.
constexpr uint32_t kRowPresent = 0x80000000u;

__device__ __forceinline__ uint4 shared_row_info(const ProblemDesc &P, uint32_t g,
                                                 uint32_t stage, uint32_t r) {
  return __ldg(P.stage_rows + ((size_t)g * P.stage_count + stage) * kStageRows + r);
}

// The last kCopyThreads threads of the CTA (four warps) stage the rows and
// tables; the others go straight on to their partial sums.  Issuing a stage's
// ~1100 asynchronous copies stalls the issuing warps for about a thousand
// cycles (outstanding global requests), and the last warps of a stage have
// the fewest phase-A items.
constexpr int kCopyThreads = 128;
constexpr uint32_t kCopyPerRow = kCopyThreads / kStageRows;  // threads per row slot

// Copies one stage into `slot` with 16-byte asynchronous copies (the
// vectorised staging path; one bulk copy per ~500-byte row costs more):
// copy thread `ctid` (0 .. kCopyThreads - 1, negative for the other threads)
// copies a share of row slot ctid / kCopyPerRow and of the stage table, then
// every thread arrives on the slot's mbarrier when its copies land.  `info`
// is the copy thread's row slot.
__device__ __forceinline__ void shared_copy(const ProblemDesc &P, const uint4 &info,
                                            uint32_t slot, uint32_t t0, const SharedLayout &L,
                                            uint8_t *smem, int ctid) {
  if (ctid >= 0) {
    const uint32_t r = (uint32_t)ctid / kCopyPerRow, c0 = (uint32_t)ctid % kCopyPerRow;
    if ((info.z & kRowPresent) && P.tma) {
      const uint32_t a = align_samples(P.bits);
      const uint32_t ws = (t0 + (info.z & ~kRowPresent)) & ~(a - 1u);
      const uint64_t boff = (uint64_t)ws * P.bits / 8u;
      const uint64_t avail = P.row_bytes - boff;
      const uint8_t *src = P.in + (((uint64_t)info.y << 32) | info.x) + boff;
      const uint32_t dst = smem_addr(smem + L.off_raw + (slot * kStageRows + r) * L.raw_bytes);
      for (uint32_t b = 16u * c0; b < L.raw_bytes; b += 16u * kCopyPerRow) {
        const uint32_t n = avail > b ? (avail - b < 16u ? (uint32_t)(avail - b) : 16u) : 0u;
        cp_async16(dst + b, n ? src + b : src, n);
      }
    }
    const uint32_t tdst = smem_addr(smem + L.off_table + slot * P.table_bytes);
    for (uint32_t b = 16u * (uint32_t)ctid; b < P.table_bytes; b += 16u * kCopyThreads)
      cp_async16(tdst + b, P.pool + info.w + b / 2u, 16u);
  }
  cp_async_arrive(reinterpret_cast<uint64_t *>(smem) + slot);
}

// Computes one tile (TY * ND DMs x 64 * NW samples); returns false if the CTA
// must stop (timeout).  `sc` counts the CTA's stages (mbarrier phases).
template <int NW, int ND, int TY>
__device__ __forceinline__ bool shared8_tile(const ProblemDesc &P, uint32_t g_index,
                                             const GroupDesc &G, uint32_t dtile, uint32_t ttile,
                                             uint8_t *smem, const SharedLayout &L, uint32_t &sc) {
  static_assert(32 * TY >= kCopyThreads && kCopyThreads % kStageRows == 0,
                "copy threads: whole warps, equal shares of the row slots");
  constexpr int kTileT = 64 * NW;
  constexpr int kTileD = TY * ND;
  constexpr uint32_t kAhead = kSharedSlots - 1;
  // Row expansion: warps per row and rows per pass.
  constexpr int kRowWarps = TY >= kStageRows ? TY / kStageRows : 1;
  constexpr int kRowStep = TY >= kStageRows ? kStageRows : TY;
  const int tid = threadIdx.x, tx = tid & 31, ty = tid >> 5;
  const uint32_t t0 = ttile * kTileT;
  const uint32_t sbeg = P.tile_stage[dtile];
  const uint32_t nst = P.tile_stage[dtile + 1] - sbeg;
  const uint32_t one = P.mul_hi8 >> 24;  // 1, unknown to the compiler
  const uint32_t cw = P.cw, psw = P.psw;
  uint64_t *bars = reinterpret_cast<uint64_t *>(smem);
  uint32_t *copy = reinterpret_cast<uint32_t *>(smem + L.off_copy);
  const uint32_t copy_s = smem_addr(copy);
  const uint32_t part_s = smem_addr(smem + L.off_part);
  const uint32_t sbase = smem_addr(smem);
  // Phase B reads the series with plain loads (the compiler schedules them
  // more freely than volatile ones; measured 2 % faster).
  auto ldc = [&](uint32_t x) { return *reinterpret_cast<const uint32_t *>(smem + (x - sbase)); };

  // The copy threads stage every stage; `next` is a copy thread's row slot of
  // the next stage to copy, loaded one stage ahead.
  const int ctid = tid - (32 * TY - kCopyThreads);
  const uint32_t myrow = ctid >= 0 ? (uint32_t)ctid / kCopyPerRow : 0u;
  {
    const uint32_t pro = nst < kAhead ? nst : kAhead;
    for (uint32_t s = 0; s < pro; ++s)
      shared_copy(P, ctid >= 0 ? shared_row_info(P, g_index, sbeg + s, myrow) : uint4{},
                  (sc + s) % kSharedSlots, t0, L, smem, ctid);
  }
  uint4 next = make_uint4(0, 0, 0, 0);
  if (ctid >= 0 && kAhead < nst) next = shared_row_info(P, g_index, sbeg + kAhead, myrow);

  uint32_t acc[ND][NW], tot[ND][NW][2];
#pragma unroll
  for (int j = 0; j < ND; ++j)
#pragma unroll
    for (int i = 0; i < NW; ++i) acc[j][i] = tot[j][i][0] = tot[j][i][1] = 0;
  uint32_t since = 0;

  auto flush = [&]() {
#pragma unroll
    for (int j = 0; j < ND; ++j)
#pragma unroll
      for (int i = 0; i < NW; ++i) {
        tot[j][i][0] += acc[j][i] & 0xFFFFu;
        tot[j][i][1] += acc[j][i] >> 16;
        acc[j][i] = 0;
      }
  };
  auto abort = [&](uint32_t s) {
    if (tid == 0) atomicOr(P.status, kStatusTimeout);
    for (uint32_t u = s; u < nst && u < s + kAhead; ++u)
      (void)mbar_wait(bars + (sc + u) % kSharedSlots, ((sc + u) / kSharedSlots) & 1u, kDrainNs);
    return false;
  };
  // Test hook of the timeout path (timeout_test_hook in dd_device.cuh).
  if (timeout_test(P) && nst &&
      __syncthreads_or(!mbar_test_wait(bars + sc % kSharedSlots, (sc / kSharedSlots) & 1u)))
    return abort(0);

  for (uint32_t s = 0; s < nst; ++s) {
    const uint32_t gs = sc + s, slot = gs % kSharedSlots;
    const bool ok = mbar_wait(bars + slot, (gs / kSharedSlots) & 1u, kWaitNs, P.wait_ns);
    const uint16_t *tb =
        reinterpret_cast<const uint16_t *>(smem + L.off_table + slot * P.table_bytes);
    uint8_t *rs = smem + L.off_raw + slot * kStageRows * L.raw_bytes;
    const uint32_t a = align_samples(P.bits);
    if (!P.tma) {
      // Rows not 16-byte aligned: the CTA copies them (the table came by
      // asynchronous copies and is valid once every thread saw its wait
      // succeed).
      if (__syncthreads_or(!ok)) return abort(s);
      for (uint32_t r = ty; r < tb[1]; r += TY) {
        const uint4 info = shared_row_info(P, g_index, sbeg + s, r);
        const uint32_t bm = info.z & ~kRowPresent;
        const uint64_t boff = (uint64_t)((t0 + bm) & ~(a - 1u)) * P.bits / 8u;
        const uint8_t *src = P.in + (((uint64_t)info.y << 32) | info.x);
        uint8_t *dst = rs + r * L.raw_bytes;
        for (uint32_t b = tx; b < L.raw_bytes; b += 32)
          dst[b] = (boff + b < P.row_bytes) ? src[boff + b] : 0;
      }
      __syncthreads();
    }
    {
      // Expand the rows to bytes in four copies: copy m word k of row r =
      // window samples 4k + m .. 4k + m + 3 from its subgroup's series
      // origin t0 + bmin.  Values read before the CTA agrees that the wait
      // succeeded are clamped so that no access leaves its buffer.
      const uint32_t nrows = tb[1] < (uint32_t)kStageRows ? tb[1] : (uint32_t)kStageRows;
      for (uint32_t r = (TY >= kStageRows ? ty % kStageRows : ty); r < nrows; r += kRowStep) {
        const uint32_t k = (r >= tb[8 + 4 + 2]) + (r >= tb[8 + 8 + 2]) + (r >= tb[8 + 12 + 2]);
        const uint32_t bm = tb[8 + 4 * k] | ((uint32_t)tb[8 + 4 * k + 1] << 16);
        const uint32_t xw = ((t0 + bm) & (a - 1u)) >> 2;
        const uint32_t cwk = tb[3 + k] < cw ? tb[3 + k] : cw;  // words phase A reads
        const uint8_t *row = rs + r * L.raw_bytes;
        uint32_t *dst = copy + r * 4u * cw;
        auto put = [&](uint32_t kk, uint32_t w0, uint32_t w1, uint32_t w2) {
          *reinterpret_cast<uint2 *>(dst + kk) = make_uint2(w0, w1);
          *reinterpret_cast<uint2 *>(dst + cw + kk) =
              make_uint2(__funnelshift_r(w0, w1, 8), __funnelshift_r(w1, w2, 8));
          *reinterpret_cast<uint2 *>(dst + 2 * cw + kk) =
              make_uint2(__funnelshift_r(w0, w1, 16), __funnelshift_r(w1, w2, 16));
          *reinterpret_cast<uint2 *>(dst + 3 * cw + kk) =
              make_uint2(__funnelshift_r(w0, w1, 24), __funnelshift_r(w1, w2, 24));
        };
        const uint32_t wr = TY >= kStageRows ? ty / kStageRows : 0;
        if (P.bits == 8) {
          for (uint32_t kk = 2u * (tx + 32u * wr); kk < cwk; kk += 64u * kRowWarps) {
            const uint32_t *r32 = reinterpret_cast<const uint32_t *>(row) + xw + kk;
            put(kk, r32[0], r32[1], r32[2]);
          }
        } else {
          for (uint32_t kk = 2u * (tx + 32u * wr); kk < cwk; kk += 64u * kRowWarps)
            put(kk, expand_word(row, xw + kk, P.bits), expand_word(row, xw + kk + 1, P.bits),
                expand_word(row, xw + kk + 2, P.bits));
        }
      }
    }
    if (__syncthreads_or(!ok)) return abort(s);
    // Every thread is past the previous stage: its slot takes stage s + kAhead.
    if (s + kAhead < nst) {
      shared_copy(P, next, (gs + kAhead) % kSharedSlots, t0, L, smem, ctid);
      if (ctid >= 0 && s + kAhead + 1 < nst)
        next = shared_row_info(P, g_index, sbeg + s + kAhead + 1, myrow);
    }

    // Phase A: item = (subgroup, chunk of 31 groups of 4 samples); lane 31
    // computes the next chunk's first group for lane 30's shifted copy.  Each
    // lane runs the subgroup's two half-chains A and B side by side (two
    // independent dependency chains), one micro-op (one moved row) of each
    // per step.
    const uint32_t nitems = tb[2];
    for (uint32_t it = ty; it < nitems; it += TY) {
      const uint32_t item = tb[kTabItems + it];
      const uint32_t *prog = reinterpret_cast<const uint32_t *>(tb + tb[8 + 4 * (item >> 8) + 3]);
      const uint4 hdr = *reinterpret_cast<const uint4 *>(prog);
      const uint32_t n = hdr.x & 0xFFFFu, ng = hdr.x >> 16;
      const uint32_t nA = hdr.y & 0xFFFFu;
      const bool hasB = hdr.w != 0xFFFFFFFFu;
      const uint32_t g = (item & 0xFFu) * 31u + tx;
      // Lanes past the series compute its last group again and store nothing.
      const uint32_t gb = copy_s + 4u * (g < ng ? g : ng - 1u);
      // Lane 31 and lanes past the series store nothing (predicated stores);
      // neither does a micro-op whose vector is not complete yet (dst = the
      // dummy series).
      const uint32_t keep = (tx < 31 && g < ng) ? 1u : 0u;
      const uint32_t pg = part_s + 8u * g;
      // lo = (P[4g], P[4g+1]), hi = (P[4g+2], P[4g+3]) as 16-bit lanes.
      uint32_t loA = 0, hiA = 0, loB = 0, hiB = 0;
      auto rows = [&](const uint32_t *offs, uint32_t &lo, uint32_t &hi) {
        const uint4 o0 = *reinterpret_cast<const uint4 *>(offs);
        const uint4 o1 = *reinterpret_cast<const uint4 *>(offs + 4);
        const uint32_t off[kSharedRows] = {o0.x, o0.y, o0.z, o0.w, o1.x, o1.y, o1.z, o1.w};
#pragma unroll
        for (int e = 0; e < kSharedRows; ++e) {  // rows past n read the zero row
          const uint32_t w = lds_u32(gb + off[e]);
          lo = mad_lo(__byte_perm(w, 0, 0x4140), one, lo);
          hi = mad_lo(__byte_perm(w, 0, 0x4342), one, hi);
        }
      };
      // `real` = 0 for micro-ops whose vector is not complete yet (their dst
      // is the dummy series; the host sets the flag in the micro-op).
      auto store = [&](uint32_t dst, uint32_t real, uint32_t lo, uint32_t hi) {
        const uint32_t nlo = __shfl_down_sync(0xffffffffu, lo, 1);
        const uint32_t on = keep & real;
        sts_v2_if(on, pg + dst, lo, hi);
        sts_v2_if(on, pg + dst + 4u * psw, __byte_perm(lo, hi, 0x5432),
                  __byte_perm(hi, nlo, 0x5432));
      };
      rows(prog + 4, loA, hiA);
      if (hasB) rows(prog + 12, loB, hiB);
      store(hdr.z, 1u, loA, hiA);
      if (hasB) store(hdr.w, 1u, loB, hiB);
      // Chain B exists whenever there are micro-ops; the host pads the two
      // halves to the same length with no-op micro-ops.
      const uint4 *ua = reinterpret_cast<const uint4 *>(prog + 20);
      const uint4 *ub = ua + nA;
      auto apply = [&](uint32_t wo, uint32_t wn, uint32_t &lo, uint32_t &hi) {
        lo = lo - __byte_perm(wo, 0, 0x4140) + __byte_perm(wn, 0, 0x4140);
        hi = hi - __byte_perm(wo, 0, 0x4342) + __byte_perm(wn, 0, 0x4342);
      };
      if (nA) {
        // Software pipeline: the row words of step i + 1 and the micro-ops of
        // step i + 2 are loaded before step i's stores (the shared-memory
        // accesses are volatile: they issue in source order).  Row addresses
        // are formed by IMAD, on the FMA pipe, leaving the integer ALU pipe
        // to the unpacking and the adds.
        uint4 a = ua[0], b = ub[0];
        uint32_t oa = lds_u32(mad_lo(a.x, one, gb)), na = lds_u32(mad_lo(a.y, one, gb));
        uint32_t ob = lds_u32(mad_lo(b.x, one, gb)), nb = lds_u32(mad_lo(b.y, one, gb));
        uint4 an = ua[nA > 1 ? 1 : 0], bn = ub[nA > 1 ? 1 : 0];
        for (uint32_t i = 0; i < nA; ++i) {
          const uint32_t oa1 = lds_u32(mad_lo(an.x, one, gb)), na1 = lds_u32(mad_lo(an.y, one, gb));
          const uint32_t ob1 = lds_u32(mad_lo(bn.x, one, gb)), nb1 = lds_u32(mad_lo(bn.y, one, gb));
          const uint32_t i2 = i + 2 < nA ? i + 2 : nA - 1;
          const uint4 an2 = ua[i2], bn2 = ub[i2];
          apply(oa, na, loA, hiA);
          apply(ob, nb, loB, hiB);
          store(a.z, a.w, loA, hiA);
          store(b.z, b.w, loB, hiB);
          a = an; b = bn; an = an2; bn = bn2;
          oa = oa1; na = na1; ob = ob1; nb = nb1;
        }
      }
    }
    __syncthreads();

    // Phase B: each DM adds kSubMax series (copy base & 1, word base >> 1).
    if (since + (uint32_t)kSubMax > kLaneSeries) {
      flush();
      since = 0;
    }
    since += kSubMax;
    const uint4 *offb = reinterpret_cast<const uint4 *>(tb + kTabSeries) + ty * ND;
    const uint32_t pb = part_s + 4u * tx;
#pragma unroll
    for (int j = 0; j < ND; ++j) {
      const uint4 oo = offb[j];
      const uint32_t a0 = pb + oo.x, a1 = pb + oo.y, a2 = pb + oo.z, a3 = pb + oo.w;
#pragma unroll
      for (int i = 0; i < NW; ++i) {
        acc[j][i] += ldc(a0 + 128u * i) + ldc(a1 + 128u * i);
        acc[j][i] += ldc(a2 + 128u * i) + ldc(a3 + 128u * i);
      }
    }
  }
  sc += nst;
  flush();
  // An overlapped launch writes only after the previous grid on the stream
  // completed (it may still be writing the same output).
  if (P.overlap) wait_prerequisites();

#pragma unroll
  for (int j = 0; j < ND; ++j) {
    const uint32_t d = dtile * kTileD + ty * ND + j;
    if (d >= P.nr_dms) continue;
    float *orow = P.out + G.out_offset + (uint64_t)d * P.out_dm_stride;
#pragma unroll
    for (int i = 0; i < NW; ++i) {
      const uint32_t t = t0 + 2u * (tx + 32u * i);
      const float v0 = (float)tot[j][i][0], v1 = (float)tot[j][i][1];
      if (P.out_vec4 && t + 1u < P.nr_samples) {
        *reinterpret_cast<float2 *>(orow + t) = make_float2(v0, v1);
      } else {
        if (t < P.nr_samples) orow[t] = v0;
        if (t + 1u < P.nr_samples) orow[t + 1] = v1;
      }
    }
  }
  if (P.accum) {
    // Detection statistics from the totals still in registers: a warp holds
    // every sample of its DMs in this tile; one set of atomics per DM.
#pragma unroll
    for (int j = 0; j < ND; ++j) {
      const uint32_t d = dtile * kTileD + ty * ND + j;
      if (d >= P.nr_dms) continue;  // uniform over the warp
      unsigned long long s1 = 0, s2 = 0, best = 0;
#pragma unroll
      for (int i = 0; i < NW; ++i)
#pragma unroll
        for (int h = 0; h < 2; ++h) {
          const uint32_t t = t0 + 2u * (tx + 32u * i) + h, v = tot[j][i][h];
          if (t < P.nr_samples) {
            s1 += v;
            s2 += (unsigned long long)v * v;
            const unsigned long long key = ((unsigned long long)v << 32) | (0xFFFFFFFFu - t);
            best = key > best ? key : best;
          }
        }
#pragma unroll
      for (int o = 16; o; o >>= 1) {
        s1 += __shfl_xor_sync(0xffffffffu, s1, o);
        s2 += __shfl_xor_sync(0xffffffffu, s2, o);
        const unsigned long long ob = __shfl_xor_sync(0xffffffffu, best, o);
        best = ob > best ? ob : best;
      }
      if (tx == 0) {
        unsigned long long *a = P.accum + 3ull * ((uint64_t)g_index * P.nr_dms + d);
        atomicAdd(a, s1);
        atomicAdd(a + 1, s2);
        atomicMax(a + 2, best);
      }
    }
  }
  return true;
}

}  // namespace dd
