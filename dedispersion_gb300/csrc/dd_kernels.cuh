// dd_kernels.cuh -- kernel templates, launchers and registry-entry macros of
// the compiled tile configurations (instantiated in dd_kernels_*.cu).
#pragma once

#include <cuda_runtime.h>

#include "dd_device.cuh"
#include "dd_shared.cuh"

namespace dd {


// Grid-mapped kernel: one CTA per tile.
template <int NW, int NDT, int TY, int CH, int VAR, bool SHORT = false>
__global__ void __launch_bounds__(32 * TY, (TY >= 16 ? 1 : (TY >= 8 ? 2 : 4)))
    swar8_kernel(const ProblemDesc P) {
  extern __shared__ __align__(128) uint8_t smem[];
  if (P.overlap) allow_dependents();
  const SmemLayout L = make_layout(kFamilySwar8, P.win_samples, P.bits, CH, TY * NDT);
  init_barriers(smem, L, CH);
  uint32_t g, dtile, ttile, sc = 0;
  decode_tile(P, blockIdx.x, g, dtile, ttile);
  (void)swar8_tile<NW, NDT, TY, CH, VAR, SHORT>(P, P.groups[g], dtile, ttile, smem, L, sc);
}

template <typename T, int NS, int NDT, int TY, int CH>
__global__ void __launch_bounds__(32 * TY, (TY >= 8 ? 2 : 4))
    scalar_kernel(const ProblemDesc P) {
  extern __shared__ __align__(128) uint8_t smem[];
  const SmemLayout L = make_layout(kFamilyScalar, P.win_samples, P.bits, CH, TY * NDT);
  init_barriers(smem, L, CH);
  uint32_t g, dtile, ttile, sc = 0;
  decode_tile(P, blockIdx.x, g, dtile, ttile);
  (void)scalar_tile<T, NS, NDT, TY, CH>(P, P.groups[g], dtile, ttile, smem, L, sc);
}

template <int NS, int NDT, int TY, int CH, int MINB>
__global__ void __launch_bounds__(32 * TY, MINB)
    pair_kernel(const ProblemDesc P) {
  extern __shared__ __align__(128) uint8_t smem[];
  if (P.overlap) allow_dependents();
  const SmemLayout L = make_layout(kFamilyPair16, P.win_samples, 32, CH, TY * NDT);
  init_barriers(smem, L, CH);
  uint32_t g, dtile, ttile, sc = 0;
  decode_tile(P, blockIdx.x, g, dtile, ttile);
  (void)pair_tile<NS, NDT, TY, CH>(P, g, P.groups[g], dtile, ttile, smem, L, sc);
}

template <int NW, int ND, int TY>
__global__ void __launch_bounds__(32 * TY, (TY >= 16 ? 1 : 2))
    shared8_kernel(const ProblemDesc P) {
  extern __shared__ __align__(128) uint8_t smem[];
  if (P.overlap) allow_dependents();
  const SharedLayout L = make_shared_layout(P.cw, P.psw, P.slots, P.table_bytes, P.bits);
  if (threadIdx.x == 0) {
    uint64_t *bars = reinterpret_cast<uint64_t *>(smem);
    for (int r = 0; r < kSharedSlots; ++r) mbar_init(bars + r, blockDim.x);
    fence_mbar_init();
  }
  // The zero series that absent subgroups of a stage read, and the zero row.
  uint32_t *zero = reinterpret_cast<uint32_t *>(smem + L.off_part) + L.zero_word;
  for (uint32_t w = threadIdx.x; w < P.psw; w += blockDim.x) zero[w] = 0;
  uint32_t *zrow = reinterpret_cast<uint32_t *>(smem + L.off_copy) + L.zero_copy;
  for (uint32_t w = threadIdx.x; w < P.cw; w += blockDim.x) zrow[w] = 0;
  __syncthreads();
  uint32_t g, dtile, ttile, sc = 0;
  decode_tile(P, blockIdx.x, g, dtile, ttile);
  (void)shared8_tile<NW, ND, TY>(P, g, P.groups[g], dtile, ttile, smem, L, sc);
}

template <int NW, int NDT, int TY, int CH, int VAR, bool SHORT = false>
void launch_swar8(const ProblemDesc &P, unsigned grid, size_t smem,
                  cudaStream_t stream) {
  swar8_kernel<NW, NDT, TY, CH, VAR, SHORT><<<grid, 32 * TY, smem, stream>>>(P);
}

template <typename T, int NS, int NDT, int TY, int CH>
void launch_scalar(const ProblemDesc &P, unsigned grid, size_t smem,
                   cudaStream_t stream) {
  scalar_kernel<T, NS, NDT, TY, CH><<<grid, 32 * TY, smem, stream>>>(P);
}

template <int NS, int NDT, int TY, int CH, int MINB>
void launch_pair(const ProblemDesc &P, unsigned grid, size_t smem, cudaStream_t stream) {
  pair_kernel<NS, NDT, TY, CH, MINB><<<grid, 32 * TY, smem, stream>>>(P);
}

template <int NW, int ND, int TY>
void launch_shared8(const ProblemDesc &P, unsigned grid, size_t smem,
                    cudaStream_t stream) {
  shared8_kernel<NW, ND, TY><<<grid, 32 * TY, smem, stream>>>(P);
}

#define DD_SWAR8(NW, NDT, TY, CH, VAR)                                        \
  {"swar8_i" #NW "_d" #NDT "_w" #TY "_c" #CH "_v" #VAR, kFamilySwar8, 8,     \
   4 * NW, NDT, TY, CH, 32 * TY, 128 * NW, TY * NDT, VAR,                    \
   reinterpret_cast<const void *>(&swar8_kernel<NW, NDT, TY, CH, VAR>),      \
   &launch_swar8<NW, NDT, TY, CH, VAR>}

// Short-group swar8 tiles: groups of at most 257 rows only (max_rows; step
// one's subbands), 16-bit lanes without 32-bit totals (257 * 255 < 2^16).
#define DD_SWAR8_SHORT(NW, NDT, TY, CH, VAR)                                  \
  {"swar8s_i" #NW "_d" #NDT "_w" #TY "_c" #CH "_v" #VAR, kFamilySwar8, 8,    \
   4 * NW, NDT, TY, CH, 32 * TY, 128 * NW, TY * NDT, VAR,                    \
   reinterpret_cast<const void *>(&swar8_kernel<NW, NDT, TY, CH, VAR, true>), \
   &launch_swar8<NW, NDT, TY, CH, VAR, true>, 257}

#define DD_SCALAR(T, BITS, NS, NDT, TY, CH)                                   \
  {"scalar" #BITS "_i" #NS "_d" #NDT "_w" #TY "_c" #CH, kFamilyScalar, BITS, \
   NS, NDT, TY, CH, 32 * TY, 32 * NS, TY * NDT, 0,                            \
   reinterpret_cast<const void *>(&scalar_kernel<T, NS, NDT, TY, CH>),       \
   &launch_scalar<T, NS, NDT, TY, CH>}


// Shared partial sums: items_t = samples per thread and DM (2 per word),
// channels = rows per subgroup.
#define DD_SHARED8(NW, ND, TY)                                                \
  {"shared8_i" #NW "_d" #ND "_w" #TY, kFamilyShared8, 8, 2 * NW, ND, TY,      \
   kSharedRows, 32 * TY, 64 * NW, TY * ND, 0,                                 \
   reinterpret_cast<const void *>(&shared8_kernel<NW, ND, TY>),              \
   &launch_shared8<NW, ND, TY>}

// Pair tiles (packed subband step two): items_t = samples per thread, items_d
// = DMs per thread, MINB = CTAs per SM the registers are budgeted for.  Not
// in the registry: they read only the packed intermediate that a subband
// pipeline's own step one writes.
#define DD_PAIR(NS, NDT, TY, CH, MINB)                                        \
  {"pair16_i" #NS "_d" #NDT "_w" #TY "_c" #CH "_b" #MINB, kFamilyPair16, 32, \
   NS, NDT, TY, CH, 32 * TY, 32 * NS, TY * NDT, 0,                            \
   reinterpret_cast<const void *>(&pair_kernel<NS, NDT, TY, CH, MINB>),      \
   &launch_pair<NS, NDT, TY, CH, MINB>}

const KernelInfo *pair_kernels(int *count);

// Parts of the registry, one per translation unit (compiled in parallel).
const KernelInfo *kernels_swar8_a(int *count);
const KernelInfo *kernels_swar8_b(int *count);
const KernelInfo *kernels_swar8_c(int *count);
const KernelInfo *kernels_scalar(int *count);
const KernelInfo *kernels_shared8(int *count);
const KernelInfo *kernels_tmem(int *count);
const KernelInfo *kernels_swar8_s(int *count);

}  // namespace dd
