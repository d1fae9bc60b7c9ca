// dd_kernels_scalar.cu -- 16-bit and float tile configurations (also step two).
#include "dd_kernels.cuh"

namespace dd {

static const KernelInfo kPart[] = {
    // float input and step two, then 16-bit input; the default of each width
    // first (fastest of a sweep at 1536 channels x 2048 DMs x 24576 samples:
    // float 8.34 ms, 16-bit 8.43 ms).
    DD_SCALAR(float, 32, 8, 8, 4, 16),
    DD_SCALAR(float, 32, 8, 4, 8, 8),
    DD_SCALAR(float, 32, 4, 4, 8, 8),
    DD_SCALAR(float, 32, 8, 2, 8, 8),
    DD_SCALAR(float, 32, 4, 8, 4, 8),
    DD_SCALAR(float, 32, 8, 4, 8, 16),
    DD_SCALAR(float, 32, 4, 4, 4, 16),
    DD_SCALAR(float, 32, 8, 2, 4, 8),
    DD_SCALAR(uint16_t, 16, 8, 4, 8, 16),
    DD_SCALAR(uint16_t, 16, 8, 4, 8, 8),
    DD_SCALAR(uint16_t, 16, 4, 4, 8, 8),
    DD_SCALAR(uint16_t, 16, 8, 2, 4, 8),
};

const KernelInfo *kernels_scalar(int *count) {
  *count = static_cast<int>(sizeof(kPart) / sizeof(kPart[0]));
  return kPart;
}

}  // namespace dd
