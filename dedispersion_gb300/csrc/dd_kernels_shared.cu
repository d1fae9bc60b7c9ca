// dd_kernels_shared.cu -- shared-partial-sum tile configurations (1/2/4/8-bit
// single step).  DedispersionConf meaning: threads_d1 = warps along DMs,
// items_d0 = samples per thread and DM, items_d1 = DMs per thread, unroll =
// rows per subgroup, items_d2 = rows per subgroup (marks the family).  Every
// configuration runs 16 warps, one CTA per SM.
#include "dd_kernels.cuh"

namespace dd {

static const KernelInfo kPart[] = {
    DD_SHARED8(4, 4, 16),  // 256 samples x 64 DMs
    DD_SHARED8(8, 2, 16),  // 512 samples x 32 DMs
    DD_SHARED8(2, 4, 16),  // 128 samples x 64 DMs
    DD_SHARED8(4, 2, 16),  // 256 samples x 32 DMs
};

const KernelInfo *kernels_shared8(int *count) {
  *count = static_cast<int>(sizeof(kPart) / sizeof(kPart[0]));
  return kPart;
}

}  // namespace dd
