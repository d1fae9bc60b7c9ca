// dd_kernels_pair.cu -- pair tile configurations (packed subband step two):
// samples per thread, DMs per thread, warps, rows per stage, CTAs per SM.
// The first is the default.
#include "dd_kernels.cuh"

namespace dd {

static const KernelInfo kPairs[] = {
    DD_PAIR(8, 4, 8, 16, 2),
    DD_PAIR(4, 4, 8, 16, 2),
    DD_PAIR(4, 8, 4, 16, 4),
    DD_PAIR(4, 4, 8, 8, 2),
    DD_PAIR(8, 2, 8, 16, 2),
    DD_PAIR(2, 8, 8, 16, 2),
    DD_PAIR(4, 4, 8, 16, 3),
    DD_PAIR(4, 2, 8, 16, 4),
    DD_PAIR(2, 4, 8, 16, 4),
    DD_PAIR(8, 2, 8, 16, 3),
    DD_PAIR(8, 4, 4, 16, 4),
};

const KernelInfo *pair_kernels(int *count) {
  *count = static_cast<int>(sizeof(kPairs) / sizeof(kPairs[0]));
  return kPairs;
}

}  // namespace dd
