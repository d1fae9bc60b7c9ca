// dd_kernels_tmem.cu -- the TMEM-window tile for float32 single-step input
// (dd_tmem.cuh describes it) and its registry entry.
#include "dd_kernels.cuh"
#include "dd_tmem.cuh"

namespace dd {

// 16 columns of this warp's 32 lanes from registers (tcgen05.st, shape
// 32x32b: thread i writes lane i, register j to column taddr + j).
__device__ __forceinline__ void tm_st8(uint32_t taddr, const uint32_t (&v)[16]) {
  asm volatile(
      "tcgen05.st.sync.aligned.32x32b.x8.b32 [%0], {%1, %2, %3, %4, %5, %6, %7, %8};"
      :: "r"(taddr), "r"(v[0]), "r"(v[1]), "r"(v[2]), "r"(v[3]), "r"(v[4]), "r"(v[5]),
         "r"(v[6]), "r"(v[7])
      : "memory");
}

__device__ __forceinline__ void tm_st16(uint32_t taddr, const uint32_t (&v)[16]) {
  asm volatile(
      "tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], {%1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, %16};"
      :: "r"(taddr), "r"(v[0]), "r"(v[1]), "r"(v[2]), "r"(v[3]), "r"(v[4]), "r"(v[5]), "r"(v[6]), "r"(v[7]), "r"(v[8]), "r"(v[9]), "r"(v[10]), "r"(v[11]), "r"(v[12]), "r"(v[13]), "r"(v[14]), "r"(v[15])
      : "memory");
}

// Two 16-column loads (tcgen05.ld, shape 32x32b) and the wait for both in
// one statement, so that no use of the registers can be scheduled before
// the data has arrived.
__device__ __forceinline__ void tm_ld16x2(uint32_t ta, uint32_t tb, uint32_t (&a)[16],
                                          uint32_t (&b)[16]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, [%32];\n\t"
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%33];\n\t"
      "tcgen05.wait::ld.sync.aligned;"
      : "=r"(a[0]), "=r"(a[1]), "=r"(a[2]), "=r"(a[3]), "=r"(a[4]), "=r"(a[5]), "=r"(a[6]), "=r"(a[7]), "=r"(a[8]), "=r"(a[9]), "=r"(a[10]), "=r"(a[11]), "=r"(a[12]), "=r"(a[13]), "=r"(a[14]), "=r"(a[15]),
        "=r"(b[0]), "=r"(b[1]), "=r"(b[2]), "=r"(b[3]), "=r"(b[4]), "=r"(b[5]), "=r"(b[6]), "=r"(b[7]), "=r"(b[8]), "=r"(b[9]), "=r"(b[10]), "=r"(b[11]), "=r"(b[12]), "=r"(b[13]), "=r"(b[14]), "=r"(b[15])
      : "r"(ta), "r"(tb)
      : "memory");
}

__device__ __forceinline__ void cp_async16_tm(uint32_t dst, const void *src, uint32_t n) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(dst), "l"(src), "r"(n)
               : "memory");
}

__device__ __forceinline__ void cp_async_arrive_tm(uint64_t *bar) {
  asm volatile("cp.async.mbarrier.arrive.noinc.shared::cta.b64 [%0];" ::"r"(smem_addr(bar))
               : "memory");
}

__device__ __forceinline__ uint4 lds128_tm(uint32_t a) {
  uint4 v;
  asm volatile("ld.shared.v4.b32 {%0, %1, %2, %3}, [%4];"
               : "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w)
               : "r"(a));
  return v;
}

__device__ __forceinline__ void tm_fence_before() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tm_fence_after() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

// Byte offset of window chunk g in a staged row (one pad chunk per 8).
__device__ __forceinline__ uint32_t tm_chunk(uint32_t g) { return 16u * (g + (g >> 3)); }

__global__ void __launch_bounds__(kTmThreads, 1) tmem32_kernel(const ProblemDesc P) {
  extern __shared__ __align__(128) uint8_t smem[];
  __shared__ uint64_t bars[kTmSlots];
  __shared__ uint32_t tbase_s;
  // Offsets of each slot's rows (tmem_tables), fetched with the rows.
  __shared__ __align__(16) uint32_t tab[kTmSlots][kTmRows][kTmTabWords];
  const int tid = threadIdx.x, w = tid >> 5, tx = tid & 31, q = w & 3, k = w >> 2;
  uint32_t g, dtile, ttile;
  decode_tile(P, blockIdx.x, g, dtile, ttile);
  const GroupDesc G = P.groups[g];
  const uint32_t t0 = ttile * kTmTileT, d0 = dtile * kTmTileD;
  const uint32_t nrows = G.entry_count;  // <= P.win_samples (the host checks)
  const uint32_t nst = (nrows + kTmRows - 1) / kTmRows;
  const uint32_t base = smem_addr(smem);
  float *shift_s = reinterpret_cast<float *>(smem + kTmSlots * kTmSlotBytes);
  uint32_t *chunk_s = reinterpret_cast<uint32_t *>(shift_s + P.win_samples);
  uint32_t *drow_s = chunk_s + P.win_samples;

  if (w == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 512;" ::"r"(
                     smem_addr(&tbase_s))
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (tid == 0) {
    for (uint32_t s = 0; s < kTmSlots; ++s) mbar_init(bars + s, kTmThreads);
    fence_mbar_init();
  }
  for (uint32_t r = tid; r < nrows; r += kTmThreads) {
    const EntryDesc E = P.entries[G.entry_begin + r];
    shift_s[r] = E.shift;
    chunk_s[r] = static_cast<uint32_t>(E.row_offset >> 4);  // 16-byte rows when P.tma
    drow_s[r] = E.delay_row;
  }
  tm_fence_before();
  __syncthreads();
  tm_fence_after();
  const uint32_t tbase = tbase_s;
  const uint32_t tmem = tbase + ((uint32_t)(32 * q) << 16);

  // Copies of step u into slot u % 3: thread tid copies chunks
  // (tid & 127) + 128 i of row tid >> 7 (the window from
  // W_0 = t0 + B), threads 0..19 also the rows' offset entries, then every
  // thread arrives once on the slot.
  const uint32_t crow = tid >> 7, cc = tid & 127;
  auto copy = [&](uint32_t u) {
    const uint32_t slot = u % kTmSlots;
    const uint32_t r = u * kTmRows + crow;
    if (tid < kTmRows * kTmTabChunks) {
      const uint32_t rr = tid / kTmTabChunks, c = tid % kTmTabChunks;
      const uint32_t rt = u * kTmRows + rr;
      if (rt < nrows && P.tma)
        cp_async16_tm(smem_addr(&tab[slot][rr][4 * c]),
                      P.tmem_tab + ((size_t)dtile * P.delay_rows + drow_s[rt]) * kTmTabChunks + c,
                      16u);
      else if (rt < nrows)
        *reinterpret_cast<uint4 *>(&tab[slot][rr][4 * c]) =
            P.tmem_tab[((size_t)dtile * P.delay_rows + drow_s[rt]) * kTmTabChunks + c];
    }
    if (r < nrows) {
      const uint32_t rel = (t0 + (dev_delay(P.first_dm, P.dm_step, d0, shift_s[r]) & ~3u)) * 4u;
      const uint32_t dst = base + slot * kTmSlotBytes + crow * kTmRowBytes;
      if (P.tma) {
        const uint8_t *src = P.in + (uint64_t)chunk_s[r] * 16u + rel;
        if ((uint64_t)rel + 16u * kTmChunks <= P.row_bytes) {
          // The whole window lies inside the row.
#pragma unroll
          for (int i = 0; i < 2; ++i) {
            const uint32_t c = cc + 128u * i;
            if (c < kTmChunks) cp_async16_tm(dst + tm_chunk(c), src + 16u * c, 16u);
          }
        } else {
#pragma unroll
          for (int i = 0; i < 2; ++i) {
            const uint32_t c = cc + 128u * i;
            if (c < kTmChunks) {
              const uint64_t off = (uint64_t)rel + 16u * c;
              const uint32_t n = P.row_bytes > off
                                     ? (P.row_bytes - off < 16u ? (uint32_t)(P.row_bytes - off) : 16u)
                                     : 0u;
              cp_async16_tm(dst + tm_chunk(c), n ? src + 16u * c : P.in, n);
            }
          }
        }
      } else {
        // Rows not 16-byte aligned: byte loads, zero past the row end.
        const uint8_t *src = P.in + P.entries[G.entry_begin + r].row_offset;
        for (uint32_t c = cc; c < kTmChunks; c += 128) {
          uint32_t v[4];
#pragma unroll
          for (int x = 0; x < 4; ++x) {
            v[x] = 0;
#pragma unroll
            for (int y = 0; y < 4; ++y) {
              const uint64_t off = (uint64_t)rel + 16u * c + 4u * x + y;
              const uint32_t b = off < P.row_bytes ? src[off] : 0u;
              v[x] |= b << (8 * y);
            }
          }
          asm volatile("st.shared.v4.b32 [%0], {%1, %2, %3, %4};" ::"r"(dst + tm_chunk(c)),
                       "r"(v[0]), "r"(v[1]), "r"(v[2]), "r"(v[3])
                       : "memory");
        }
      }
    }
    if (P.tma)
      cp_async_arrive_tm(bars + slot);
    else
      mbar_arrive(bars + slot);
  };

  if (nst > 0) copy(0);
  if (nst > 1) copy(1);

  float acc[kTmDPW][kTmT];
#pragma unroll
  for (int j = 0; j < kTmDPW; ++j)
#pragma unroll
    for (int i = 0; i < kTmT; ++i) acc[j][i] = 0.f;

  bool ok = true;
  if (timeout_test(P) && nst && __syncthreads_or(!mbar_test_wait(bars, 0u))) ok = false;
  for (uint32_t s = 0; ok && s < nst; ++s) {
    const uint32_t slot = s % kTmSlots, buf = s & 1u;
    const uint32_t nr = min(nrows - s * kTmRows, (uint32_t)kTmRows);
    const bool landed = mbar_wait(bars + slot, (s / kTmSlots) & 1u, kWaitNs, P.wait_ns);
    if (landed) {
      // Warp k copies columns 16k .. 16k + 15 of its quarter's windows, or
      // the first 8 of them where the row's DMs reach no further.
      const uint32_t sb = base + slot * kTmSlotBytes;
      for (uint32_t r = 0; r < nr; ++r) {
        const uint32_t *e = tab[slot][r];
        const uint32_t cols = (e[2] >> (8 * q)) & 0xFFu;
        if (16u * k >= cols) continue;  // warp-uniform: no DM reaches these columns
        const bool half = 16u * k + 8u >= cols;
        const uint32_t g0 = ((e[1] >> (8 * q)) & 0xFFu) + 4u * tx + 4u * k;
        uint32_t v[16];
#pragma unroll
        for (int m = 0; m < 4; ++m) {
          if (m >= 2 && half) break;
          const uint4 x = lds128_tm(sb + r * kTmRowBytes + tm_chunk(g0 + m));
          v[4 * m] = x.x;
          v[4 * m + 1] = x.y;
          v[4 * m + 2] = x.z;
          v[4 * m + 3] = x.w;
        }
        if (half)
          tm_st8(tmem + buf * 256u + r * kTmCols + 16u * k, v);
        else
          tm_st16(tmem + buf * 256u + r * kTmCols + 16u * k, v);
      }
      asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
    }
    tm_fence_before();
    if (__syncthreads_or(!landed)) {
      ok = false;
      break;
    }
    tm_fence_after();
    if (s + 2 < nst) copy(s + 2);
    for (uint32_t r = 0; r < nr; ++r) {
      const uint32_t ow = tab[slot][r][4 + 4 * q + k];
      const uint32_t col = tmem + buf * 256u + r * kTmCols;
#pragma unroll
      for (int j = 0; j < kTmDPW; j += 2) {
        uint32_t x0[16], x1[16];
        tm_ld16x2(col + ((ow >> (8 * j)) & 0xFFu), col + ((ow >> (8 * j + 8)) & 0xFFu), x0, x1);
#pragma unroll
        for (int i = 0; i < kTmT; ++i) acc[j][i] += __uint_as_float(x0[i]);
#pragma unroll
        for (int i = 0; i < kTmT; ++i) acc[j + 1][i] += __uint_as_float(x1[i]);
      }
    }
  }
  if (!ok) {
    // A wait ran out: report it, let every copy in flight land, write nothing.
    if (tid == 0) atomicOr(P.status, kStatusTimeout);
    asm volatile("cp.async.wait_all;" ::: "memory");
  } else {
    const uint32_t t = t0 + kTmT * tx;
#pragma unroll
    for (int j = 0; j < kTmDPW; ++j) {
      const uint32_t d = d0 + 16u * q + kTmDPW * k + j;
      if (d >= P.nr_dms) continue;
      float *o = P.out + G.out_offset + (uint64_t)d * P.out_dm_stride + t;
      if (P.out_vec4 && t + kTmT <= P.nr_samples) {
#pragma unroll
        for (int i = 0; i < kTmT; i += 4)
          *reinterpret_cast<float4 *>(o + i) =
              make_float4(acc[j][i], acc[j][i + 1], acc[j][i + 2], acc[j][i + 3]);
      } else {
#pragma unroll
        for (int i = 0; i < kTmT; ++i)
          if (t + i < P.nr_samples) o[i] = acc[j][i];
      }
    }
  }
  tm_fence_before();
  __syncthreads();
  if (w == 0) {
    tm_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 512;" ::"r"(tbase) : "memory");
  }
}

void launch_tmem32(const ProblemDesc &P, unsigned grid, size_t smem, cudaStream_t stream) {
  tmem32_kernel<<<grid, kTmThreads, smem, stream>>>(P);
}


static const KernelInfo kPart[] = {
    // items_t = samples per lane, items_d = DMs per warp, warps_d = warps,
    // channels = rows per step.
    {"tmem32_t16_d64", kFamilyTmem32, 32, kTmT, kTmDPW, kTmThreads / 32, kTmRows, kTmThreads,
     kTmTileT, kTmTileD, 0, reinterpret_cast<const void *>(&tmem32_kernel), &launch_tmem32},
};

const KernelInfo *kernels_tmem(int *count) {
  *count = static_cast<int>(sizeof(kPart) / sizeof(kPart[0]));
  return kPart;
}

}  // namespace dd
