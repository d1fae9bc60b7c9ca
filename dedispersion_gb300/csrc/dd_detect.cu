// dd_detect.cu -- detection statistics of the dedispersed output: per output
// row (synthesized beam x DM) the exact integer sum, sum of squares and the
// largest sample, for the S/N search that follows dedispersion in a pipeline.
//
// The shared-partial-sum kernel accumulates them in its epilogue from the
// totals still in registers (dd_shared.cuh).  Plans on the other kernels use
// row_stats_kernel below: one block per output row reads the row back.  Both
// give the same integers (the output holds exact integers below 2^24).
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>

#include "../../include/dedisp_gb300.h"
#include "dd_internal.h"

namespace dd {

namespace {

constexpr int kRowThreads = 256;

__device__ __forceinline__ unsigned long long umax64(unsigned long long a, unsigned long long b) {
  return a > b ? a : b;
}

__global__ void __launch_bounds__(kRowThreads) row_stats_kernel(const ProblemDesc P,
                                                                unsigned long long *accum) {
  __shared__ unsigned long long part[3][kRowThreads / 32];
  const uint32_t row = blockIdx.x, g = row / P.nr_dms, d = row % P.nr_dms;
  const float *o = P.out + P.groups[g].out_offset + (uint64_t)d * P.out_dm_stride;
  unsigned long long s1 = 0, s2 = 0, best = 0;
  for (uint32_t t = threadIdx.x; t < P.nr_samples; t += kRowThreads) {
    const uint32_t v = __float2uint_rn(o[t]);
    s1 += v;
    s2 += (unsigned long long)v * v;
    best = umax64(best, ((unsigned long long)v << 32) | (0xFFFFFFFFu - t));
  }
  for (int k = 16; k; k >>= 1) {
    s1 += __shfl_xor_sync(0xffffffffu, s1, k);
    s2 += __shfl_xor_sync(0xffffffffu, s2, k);
    best = umax64(best, __shfl_xor_sync(0xffffffffu, best, k));
  }
  const int w = threadIdx.x >> 5;
  if ((threadIdx.x & 31) == 0) {
    part[0][w] = s1;
    part[1][w] = s2;
    part[2][w] = best;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int i = 1; i < kRowThreads / 32; ++i) {
      s1 += part[0][i];
      s2 += part[1][i];
      best = umax64(best, part[2][i]);
    }
    accum[3ull * row] = s1;
    accum[3ull * row + 1] = s2;
    accum[3ull * row + 2] = best;
  }
}

}  // namespace

// One block per output row of the problem's output (after its dedispersion
// kernel on the same stream).
cudaError_t launch_row_stats(const ProblemDesc &P, unsigned long long *accum, uint32_t rows,
                             cudaStream_t stream) {
  if (rows == 0) return cudaSuccess;
  row_stats_kernel<<<rows, kRowThreads, 0, stream>>>(P, accum);
  return cudaGetLastError();
}

}  // namespace dd

extern "C" dd_status dd_dm_stats_from_accum(const dd_dm_accum *accum, size_t rows,
                                            uint32_t samples, dd_dm_stats *stats) {
  if ((!accum || !stats) && rows) return DD_ERR_INVALID_ARGUMENT;
  for (size_t r = 0; r < rows; r++) {
    dd_dm_stats &s = stats[r];
    std::memset(&s, 0, sizeof(s));
    if (samples == 0) continue;
    const double n = samples;
    s.mean = (double)accum[r].sum / n;
    // Integer moments: n * sum_sq - sum^2 exactly in long double where it fits.
    const long double var =
        ((long double)accum[r].sum_sq * n - (long double)accum[r].sum * accum[r].sum) / (n * n);
    s.stddev = var > 0 ? std::sqrt((double)var) : 0.0;
    s.peak = (float)(accum[r].peak >> 32);
    s.peak_sample = 0xFFFFFFFFu - (uint32_t)(accum[r].peak & 0xFFFFFFFFu);
    s.snr = s.stddev > 0 ? ((double)s.peak - s.mean) / s.stddev : 0.0;
  }
  return DD_OK;
}
