// dd_kernels.cu -- compiled tile configurations and their launchers.
//
// Each configuration is one template instantiation; the registry lists them
// with their DedispersionConf meaning (threads/items per dimension, rows per
// stage) so that plans and the tuner can pick one at run time.  The reference
// compiles one OpenCL kernel per configuration at run time instead
// (src/DedispersionTest.cpp:339-354); here every configuration is compiled
// ahead of time for sm_103a.
#include <cuda_runtime.h>

#include "dd_device.cuh"

namespace dd {

// Grid-mapped kernel: one CTA per tile.
template <int NW, int NDT, int TY, int CH, int VAR>
__global__ void __launch_bounds__(32 * TY, (TY >= 16 ? 1 : (TY >= 8 ? 2 : 4)))
    swar8_kernel(const ProblemDesc P) {
  extern __shared__ __align__(128) uint8_t smem[];
  const SmemLayout L = make_layout(kFamilySwar8, P.win_samples, P.bits, CH, TY * NDT);
  init_barriers(smem, L, CH);
  uint32_t g, dtile, ttile, sc = 0;
  decode_tile(P, blockIdx.x, g, dtile, ttile);
  (void)swar8_tile<NW, NDT, TY, CH, VAR>(P, P.groups[g], dtile, ttile, smem, L, sc);
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

template <int NW, int NDT, int TY, int CH, int VAR>
void launch_swar8(const ProblemDesc &P, unsigned grid, size_t smem,
                  cudaStream_t stream) {
  swar8_kernel<NW, NDT, TY, CH, VAR><<<grid, 32 * TY, smem, stream>>>(P);
}

template <typename T, int NS, int NDT, int TY, int CH>
void launch_scalar(const ProblemDesc &P, unsigned grid, size_t smem,
                   cudaStream_t stream) {
  scalar_kernel<T, NS, NDT, TY, CH><<<grid, 32 * TY, smem, stream>>>(P);
}

#define DD_SWAR8(NW, NDT, TY, CH, VAR)                                        \
  {"swar8_i" #NW "_d" #NDT "_w" #TY "_c" #CH "_v" #VAR, kFamilySwar8, 8,     \
   4 * NW, NDT, TY, CH, 32 * TY, 128 * NW, TY * NDT, VAR,                    \
   reinterpret_cast<const void *>(&swar8_kernel<NW, NDT, TY, CH, VAR>),      \
   &launch_swar8<NW, NDT, TY, CH, VAR>}

#define DD_SCALAR(T, BITS, NS, NDT, TY, CH)                                   \
  {"scalar" #BITS "_i" #NS "_d" #NDT "_w" #TY "_c" #CH, kFamilyScalar, BITS, \
   NS, NDT, TY, CH, 32 * TY, 32 * NS, TY * NDT, 0,                            \
   reinterpret_cast<const void *>(&scalar_kernel<T, NS, NDT, TY, CH>),       \
   &launch_scalar<T, NS, NDT, TY, CH>}

static const KernelInfo kRegistry[] = {
    // swar8: items_t = 4 * NW samples per thread, NDT DMs per thread,
    // last argument the inner-loop variant (kUnpackMaskHigh, kUnpackPermute).
    DD_SWAR8(4, 4, 8, 16, kUnpackPermuteMad),  // default: 512 samples x 32 DMs
    DD_SWAR8(2, 8, 8, 16, kUnpackPermuteMad),
    DD_SWAR8(4, 4, 16, 16, kUnpackPermuteMad),
    DD_SWAR8(4, 4, 8, 16, kUnpackPermute),
    DD_SWAR8(4, 4, 8, 8, kUnpackPermute),
    DD_SWAR8(2, 8, 8, 16, kUnpackPermute),
    DD_SWAR8(2, 4, 8, 16, kUnpackPermute),
    DD_SWAR8(4, 2, 8, 16, kUnpackPermute),
    DD_SWAR8(4, 4, 8, 16, kUnpackPermuteHalf),
    DD_SWAR8(2, 8, 8, 16, kUnpackPermuteHalf),
    DD_SWAR8(4, 4, 8, 16, kUnpackMaskHigh),
    // scalar float (float input, step two) and 16-bit.
    DD_SCALAR(float, 32, 8, 4, 8, 8),
    DD_SCALAR(float, 32, 4, 4, 8, 8),
    DD_SCALAR(float, 32, 8, 2, 8, 8),
    DD_SCALAR(float, 32, 4, 8, 4, 8),
    DD_SCALAR(uint16_t, 16, 8, 4, 8, 8),
    DD_SCALAR(uint16_t, 16, 4, 4, 8, 8),
};

const KernelInfo *kernel_registry(int *count) {
  *count = static_cast<int>(sizeof(kRegistry) / sizeof(kRegistry[0]));
  return kRegistry;
}

size_t kernel_smem_bytes(const KernelInfo &k, uint32_t win_samples,
                         uint32_t bits) {
  return make_layout(k.family, win_samples, bits, k.channels, k.tile_d).total;
}

uint32_t window_alignment_samples(uint32_t bits) { return align_samples(bits); }

}  // namespace dd
