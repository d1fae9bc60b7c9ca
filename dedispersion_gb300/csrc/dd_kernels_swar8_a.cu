// dd_kernels_swar8_a.cu -- 1/2/4/8-bit tile configurations, 16 samples per thread.
#include "dd_kernels.cuh"

namespace dd {

static const KernelInfo kPart[] = {
    // The default: 512 samples x 32 DMs per tile, 256 threads, 16 rows per stage.
    DD_SWAR8(4, 4, 8, 16, kUnpackPermuteMad),
    DD_SWAR8(2, 8, 8, 16, kUnpackPermuteMad),
    DD_SWAR8(4, 4, 16, 16, kUnpackPermuteMad),
    DD_SWAR8(4, 4, 8, 8, kUnpackPermuteMad),
    DD_SWAR8(4, 4, 4, 16, kUnpackPermuteMad),
    DD_SWAR8(4, 4, 4, 8, kUnpackPermuteMad),
    DD_SWAR8(4, 2, 8, 16, kUnpackPermuteMad),
    DD_SWAR8(4, 2, 8, 8, kUnpackPermuteMad),
    DD_SWAR8(4, 2, 16, 16, kUnpackPermuteMad),
    DD_SWAR8(4, 2, 4, 16, kUnpackPermuteMad),
    DD_SWAR8(4, 4, 8, 16, kUnpackPermute),
    DD_SWAR8(4, 4, 8, 8, kUnpackPermute),
    DD_SWAR8(4, 4, 8, 16, kUnpackPermuteHalf),
    DD_SWAR8(4, 4, 8, 16, kUnpackMaskHigh),
};

const KernelInfo *kernels_swar8_a(int *count) {
  *count = static_cast<int>(sizeof(kPart) / sizeof(kPart[0]));
  return kPart;
}

}  // namespace dd
