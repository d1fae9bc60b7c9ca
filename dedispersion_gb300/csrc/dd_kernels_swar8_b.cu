// dd_kernels_swar8_b.cu -- 1/2/4/8-bit tile configurations, 8 samples per thread.
#include "dd_kernels.cuh"

namespace dd {

static const KernelInfo kPart[] = {
    DD_SWAR8(2, 8, 8, 8, kUnpackPermuteMad),
    DD_SWAR8(2, 8, 16, 16, kUnpackPermuteMad),
    DD_SWAR8(2, 8, 4, 16, kUnpackPermuteMad),
    DD_SWAR8(2, 4, 8, 16, kUnpackPermuteMad),
    DD_SWAR8(2, 4, 8, 8, kUnpackPermuteMad),
    DD_SWAR8(2, 4, 16, 16, kUnpackPermuteMad),
    DD_SWAR8(2, 4, 4, 16, kUnpackPermuteMad),
    DD_SWAR8(2, 2, 8, 16, kUnpackPermuteMad),
    DD_SWAR8(2, 2, 16, 16, kUnpackPermuteMad),
    DD_SWAR8(2, 2, 4, 8, kUnpackPermuteMad),
    DD_SWAR8(2, 8, 8, 16, kUnpackPermute),
    DD_SWAR8(2, 8, 8, 16, kUnpackPermuteHalf),
};

const KernelInfo *kernels_swar8_b(int *count) {
  *count = static_cast<int>(sizeof(kPart) / sizeof(kPart[0]));
  return kPart;
}

}  // namespace dd
