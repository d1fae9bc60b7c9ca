// dd_kernels_swar8_s.cu -- short-group swar8 tiles: groups of at most 256
// rows (step one's subbands), whose 16-bit lanes need no 32-bit totals.
#include "dd_kernels.cuh"

namespace dd {

static const KernelInfo kPart[] = {
    // The subband step-one default: 512 samples x 64 coarse DMs, 8 rows per
    // stage (0.170 ms at 1536 channels in 32 subbands, 64 coarse DMs, against
    // 0.186 ms for the fastest tile with 32-bit totals).
    DD_SWAR8_SHORT(4, 8, 8, 8, kUnpackPermuteMad),
    DD_SWAR8_SHORT(2, 8, 8, 16, kUnpackPermuteMad),
    DD_SWAR8_SHORT(4, 8, 8, 16, kUnpackPermuteMad),
    DD_SWAR8_SHORT(4, 4, 16, 16, kUnpackPermuteMad),
};

const KernelInfo *kernels_swar8_s(int *count) {
  *count = static_cast<int>(sizeof(kPart) / sizeof(kPart[0]));
  return kPart;
}

}  // namespace dd
