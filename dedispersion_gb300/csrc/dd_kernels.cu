// dd_kernels.cu -- the registry of compiled tile configurations.
//
// Each configuration is one template instantiation (dd_kernels_*.cu); the
// registry lists them with their DedispersionConf meaning (threads/items per
// dimension, rows per stage) so that plans and the tuner can pick one at run
// time.  The reference compiles one OpenCL kernel per configuration at run
// time instead (src/DedispersionTest.cpp:339-354); here every configuration
// is compiled ahead of time for sm_103a.  The first entry of each input
// width is the default direct tile (plans created without a configuration
// try the shared-partial-sum tile first for 1-8-bit single-step input, the
// TMEM-window tile for float single-step input).
#include <mutex>
#include <vector>

#include "dd_kernels.cuh"
#include "dd_tmem.cuh"

namespace dd {

const KernelInfo *kernel_registry(int *count) {
  static std::vector<KernelInfo> all;
  static std::once_flag once;
  std::call_once(once, [] {
    for (auto part : {kernels_swar8_a, kernels_swar8_b, kernels_swar8_c, kernels_scalar,
                      kernels_shared8, kernels_swar8_s, kernels_tmem}) {
      int n = 0;
      const KernelInfo *k = part(&n);
      all.insert(all.end(), k, k + n);
    }
  });
  *count = static_cast<int>(all.size());
  return all.data();
}

size_t kernel_smem_bytes(const KernelInfo &k, uint32_t win_samples,
                         uint32_t bits) {
  if (k.family == kFamilyTmem32) return tmem_smem_bytes(win_samples);
  return make_layout(k.family, win_samples, bits, k.channels, k.tile_d).total;
}

uint32_t window_alignment_samples(uint32_t bits) { return align_samples(bits); }

}  // namespace dd
