// dd_peak.cu -- measured add throughput of the GPU: the denominator of the
// path's roofline.
//
// The direct-sum dedispersion is bound by 32-bit adds (one per live channel
// and DM-sample), not by HBM, so its roofline needs the machine's add rate.
// dd_measure_add_rate runs two short streams of dependency-free adds on
// every SM -- float adds (FADD) and 32-bit integer adds (the compiler's own
// choice of integer add instructions and pipes) -- times them with CUDA
// events and returns adds per second.  Each thread carries eight chains
// a[j] += a[j + 1 mod 8], so no chain can be folded into a multiply and
// every iteration has eight independent adds; 2048 threads per SM keep the
// pipes full.  No counterpart in the reference.
#include <cuda_runtime.h>

#include <cstdint>

#include "../../include/dedisp_gb300.h"

namespace dd {
void set_last_error(const char *message);
}

namespace {

constexpr int kThreads = 256;
constexpr int kChains = 8;

template <typename T>
__global__ void __launch_bounds__(kThreads) add_stream_kernel(uint32_t iters, uint32_t seed,
                                                              T *sink) {
  T a[kChains];
#pragma unroll
  for (int j = 0; j < kChains; ++j)
    a[j] = static_cast<T>((seed + threadIdx.x * 7u + blockIdx.x + j) & 0xFFu);
#pragma unroll 1
  for (uint32_t i = 0; i < iters; ++i) {
#pragma unroll
    for (int u = 0; u < 16; ++u) {
#pragma unroll
      for (int j = 0; j < kChains; ++j) a[j] = a[j] + a[(j + 1) % kChains];
    }
  }
  T s = a[0];
#pragma unroll
  for (int j = 1; j < kChains; ++j) s = s + a[j];
  // Never true for the seeds used; keeps the chains alive.
  if (s == static_cast<T>(seed) && seed == 0x7FFFFFFFu) sink[threadIdx.x] = s;
}

template <typename T>
cudaError_t time_stream(int blocks, uint32_t iters, T *sink, cudaStream_t st, cudaEvent_t e0,
                        cudaEvent_t e1, float *ms) {
  cudaError_t e = cudaEventRecord(e0, st);
  if (e == cudaSuccess) {
    add_stream_kernel<T><<<blocks, kThreads, 0, st>>>(iters, 1u, sink);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaEventRecord(e1, st);
  if (e == cudaSuccess) e = cudaEventSynchronize(e1);
  if (e == cudaSuccess) e = cudaEventElapsedTime(ms, e0, e1);
  return e;
}

}  // namespace

extern "C" dd_status dd_measure_add_rate(int device, uint32_t repeats, double *fadd_per_s,
                                         double *iadd_per_s) {
  if (!fadd_per_s || !iadd_per_s || repeats == 0) {
    dd::set_last_error("dd_measure_add_rate: NULL output or zero repeats");
    return DD_ERR_INVALID_ARGUMENT;
  }
  int count = 0;
  if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) {
    (void)cudaGetLastError();
    dd::set_last_error("no CUDA device");
    return DD_ERR_NO_DEVICE;
  }
  int prev = 0;
  cudaGetDevice(&prev);
  if (cudaSetDevice(device) != cudaSuccess) {
    (void)cudaGetLastError();
    dd::set_last_error("cannot select the device");
    return DD_ERR_INVALID_ARGUMENT;
  }
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  const int blocks = sms * (2048 / kThreads);
  const uint32_t iters = 4096;  // x 16 x 8 adds per thread: ~10 ms per stream
  const double adds = (double)blocks * kThreads * kChains * 16.0 * iters;
  cudaStream_t st = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  void *sink = nullptr;
  cudaError_t e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreate(&e0);
  if (e == cudaSuccess) e = cudaEventCreate(&e1);
  if (e == cudaSuccess) e = cudaMalloc(&sink, kThreads * sizeof(uint32_t));
  float best_f = 0, best_i = 0;
  for (uint32_t r = 0; r <= repeats && e == cudaSuccess; r++) {  // r = 0 warms up
    float ms_f = 0, ms_i = 0;
    e = time_stream<float>(blocks, iters, static_cast<float *>(sink), st, e0, e1, &ms_f);
    if (e == cudaSuccess)
      e = time_stream<uint32_t>(blocks, iters, static_cast<uint32_t *>(sink), st, e0, e1, &ms_i);
    if (e == cudaSuccess && r > 0) {
      if (best_f == 0 || ms_f < best_f) best_f = ms_f;
      if (best_i == 0 || ms_i < best_i) best_i = ms_i;
    }
  }
  if (sink) cudaFree(sink);
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  if (st) cudaStreamDestroy(st);
  cudaSetDevice(prev);
  if (e != cudaSuccess) {
    (void)cudaGetLastError();
    dd::set_last_error(cudaGetErrorString(e));
    return DD_ERR_CUDA;
  }
  *fadd_per_s = adds / (best_f * 1e-3);
  *iadd_per_s = adds / (best_i * 1e-3);
  return DD_OK;
}
