// dd_kernels_swar8_c.cu -- 1/2/4/8-bit tile configurations, 4 samples per thread.
#include "dd_kernels.cuh"

namespace dd {

static const KernelInfo kPart[] = {
    DD_SWAR8(1, 8, 8, 16, kUnpackPermuteMad),
    DD_SWAR8(1, 8, 8, 8, kUnpackPermuteMad),
    DD_SWAR8(1, 8, 16, 16, kUnpackPermuteMad),
    DD_SWAR8(1, 8, 4, 16, kUnpackPermuteMad),
    DD_SWAR8(1, 4, 8, 16, kUnpackPermuteMad),
    DD_SWAR8(1, 4, 16, 16, kUnpackPermuteMad),
    DD_SWAR8(1, 4, 4, 8, kUnpackPermuteMad),
    DD_SWAR8(2, 4, 4, 8, kUnpackPermuteMad),
    DD_SWAR8(4, 4, 16, 8, kUnpackPermuteMad),
    DD_SWAR8(2, 8, 16, 8, kUnpackPermuteMad),
};

const KernelInfo *kernels_swar8_c(int *count) {
  *count = static_cast<int>(sizeof(kPart) / sizeof(kPart[0]));
  return kPart;
}

}  // namespace dd
