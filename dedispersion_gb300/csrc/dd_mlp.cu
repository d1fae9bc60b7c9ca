// dd_mlp.cu -- the learned tuner's cost model: a small MLP trained and run
// by hand-written CUDA kernels.
//
// in -> 128 -> 128 -> 128 -> 1, ReLU on the hidden layers, predicting the log
// of a kernel configuration's run time from shape and configuration features.
// Weights are stored in bf16 (the copy every forward and backward pass reads);
// fp32 master weights receive the Adam updates and are rounded to bf16 after
// each step.  All products accumulate in fp32.  Loss: mean squared error.
//
// Parameter layout (flat, fp32 on the host side of the ABI): for each layer,
// W [out][in] then b [out].
//
// No counterpart in the reference, whose tuner is an exhaustive sweep
// (src/DedispersionTuning.cpp:201-437); the sweep stays the arbiter of what is fastest.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <random>
#include <vector>

#include "../../include/dedisp_gb300.h"

namespace dd {
void set_last_error(const char *message);
}

namespace {

constexpr int kRows = 16;      // rows of X per block in the forward kernel
constexpr int kMaxWidth = 256; // widest layer input/output supported

dd_status fail(dd_status code, const char *fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  dd::set_last_error(buf);
  return code;
}

dd_status cuda_fail(cudaError_t e, const char *what) {
  (void)cudaGetLastError();
  return fail(e == cudaErrorMemoryAllocation ? DD_ERR_OUT_OF_MEMORY : DD_ERR_CUDA, "%s: %s",
              what, cudaGetErrorString(e));
}

#define DDM_CUDA(call, what)                           \
  do {                                                 \
    cudaError_t e_ = (call);                           \
    if (e_ != cudaSuccess) return cuda_fail(e_, what); \
  } while (0)

// Z[n][o] = sum_i X[n][i] * W[o][i] + b[o];  Y = relu(Z) or Z.
// Block: O threads (one per output), kRows rows of X staged in shared memory.
__global__ void mlp_forward_kernel(const float *__restrict__ X, const __nv_bfloat16 *__restrict__ W,
                                   const float *__restrict__ b, float *__restrict__ Z,
                                   float *__restrict__ Y, int N, int I, int O, int relu) {
  __shared__ float xs[kRows][kMaxWidth];
  const int n0 = blockIdx.x * kRows;
  for (int k = threadIdx.x; k < kRows * I; k += blockDim.x) {
    const int r = k / I, i = k % I;
    xs[r][i] = (n0 + r < N) ? X[(size_t)(n0 + r) * I + i] : 0.0f;
  }
  __syncthreads();
  const int o = threadIdx.x;
  if (o >= O) return;
  float acc[kRows];
#pragma unroll
  for (int r = 0; r < kRows; ++r) acc[r] = b[o];
  const __nv_bfloat16 *w = W + (size_t)o * I;
  for (int i = 0; i < I; ++i) {
    const float wi = __bfloat162float(w[i]);
#pragma unroll
    for (int r = 0; r < kRows; ++r) acc[r] = fmaf(xs[r][i], wi, acc[r]);
  }
#pragma unroll
  for (int r = 0; r < kRows; ++r) {
    if (n0 + r >= N) break;
    const size_t idx = (size_t)(n0 + r) * O + o;
    if (Z) Z[idx] = acc[r];
    Y[idx] = relu ? fmaxf(acc[r], 0.0f) : acc[r];
  }
}

// dZ = dY * relu'(Z) in place (dY holds dL/dY on entry).
__global__ void relu_backward_kernel(float *dY, const float *Z, size_t count) {
  const size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (k < count && Z[k] <= 0.0f) dY[k] = 0.0f;
}

// dX[n][i] = sum_o dZ[n][o] * W[o][i]
__global__ void mlp_backward_input_kernel(const float *__restrict__ dZ,
                                          const __nv_bfloat16 *__restrict__ W,
                                          float *__restrict__ dX, int N, int I, int O) {
  const size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (k >= (size_t)N * I) return;
  const int n = (int)(k / I), i = (int)(k % I);
  float acc = 0.0f;
  for (int o = 0; o < O; ++o) acc = fmaf(dZ[(size_t)n * O + o], __bfloat162float(W[(size_t)o * I + i]), acc);
  dX[k] = acc;
}

// dW[o][i] = sum_n dZ[n][o] * X[n][i];  db[o] = sum_n dZ[n][o]  (i == I slot).
// One block per o; threads over i (and one extra for the bias), loop over n.
__global__ void mlp_backward_weight_kernel(const float *__restrict__ dZ,
                                           const float *__restrict__ X, float *__restrict__ dW,
                                           float *__restrict__ db, int N, int I, int O) {
  const int o = blockIdx.x;
  for (int i = threadIdx.x; i <= I; i += blockDim.x) {
    float acc = 0.0f;
    if (i < I) {
      for (int n = 0; n < N; ++n) acc = fmaf(dZ[(size_t)n * O + o], X[(size_t)n * I + i], acc);
      dW[(size_t)o * I + i] = acc;
    } else {
      for (int n = 0; n < N; ++n) acc += dZ[(size_t)n * O + o];
      db[o] = acc;
    }
  }
}

// Mean squared error of the single-output prediction and its gradient.
__global__ void mse_kernel(const float *__restrict__ pred, const float *__restrict__ target,
                           float *__restrict__ grad, float *__restrict__ loss, int N) {
  __shared__ float part[256];
  float acc = 0.0f;
  for (int n = threadIdx.x; n < N; n += blockDim.x) {
    const float d = pred[n] - target[n];
    grad[n] = 2.0f * d / (float)N;
    acc = fmaf(d, d, acc);
  }
  part[threadIdx.x] = acc;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) part[threadIdx.x] += part[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) *loss = part[0] / (float)N;
}

// Adam on the fp32 master weights; the bf16 copy of each W follows.
__global__ void adam_kernel(float *__restrict__ p, const float *__restrict__ g,
                            float *__restrict__ m, float *__restrict__ v,
                            __nv_bfloat16 *__restrict__ pbf, const int *__restrict__ bf_index,
                            size_t count, float lr, float b1, float b2, float eps, float c1,
                            float c2) {
  const size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (k >= count) return;
  const float gk = g[k];
  const float mk = b1 * m[k] + (1.0f - b1) * gk;
  const float vk = b2 * v[k] + (1.0f - b2) * gk * gk;
  m[k] = mk;
  v[k] = vk;
  const float pk = p[k] - lr * (mk / c1) / (sqrtf(vk / c2) + eps);
  p[k] = pk;
  const int bi = bf_index[k];
  if (bi >= 0) pbf[bi] = __float2bfloat16_rn(pk);
}

__global__ void to_bf16_kernel(const float *__restrict__ p, __nv_bfloat16 *__restrict__ pbf,
                               const int *__restrict__ bf_index, size_t count) {
  const size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (k < count && bf_index[k] >= 0) pbf[bf_index[k]] = __float2bfloat16_rn(p[k]);
}

struct Layer {
  int in, out;
  size_t w_off, b_off;  // in the flat fp32 parameters
  size_t wbf_off;       // in the bf16 weight copy
  bool relu;
};

}  // namespace

struct dd_mlp {
  int device = 0;
  std::vector<Layer> layers;
  size_t nparams = 0, nbf = 0;
  float *d_p = nullptr, *d_g = nullptr, *d_m = nullptr, *d_v = nullptr;
  __nv_bfloat16 *d_pbf = nullptr;
  int *d_bfi = nullptr;
  // activations for a batch of up to cap rows
  size_t cap = 0;
  std::vector<float *> act;  // act[0] = X, act[l+1] = output of layer l
  std::vector<float *> pre;  // pre-activations of hidden layers
  float *d_grad_a = nullptr, *d_grad_b = nullptr;  // ping-pong dL/dY buffers
  float *d_target = nullptr, *d_loss = nullptr;
  long step = 0;
};

namespace {

void free_batch(dd_mlp *m) {
  for (float *p : m->act) cudaFree(p);
  for (float *p : m->pre) cudaFree(p);
  m->act.clear();
  m->pre.clear();
  if (m->d_grad_a) cudaFree(m->d_grad_a);
  if (m->d_grad_b) cudaFree(m->d_grad_b);
  if (m->d_target) cudaFree(m->d_target);
  m->d_grad_a = m->d_grad_b = m->d_target = nullptr;
  m->cap = 0;
}

dd_status ensure_batch(dd_mlp *m, size_t n) {
  if (n <= m->cap) return DD_OK;
  free_batch(m);
  m->act.assign(m->layers.size() + 1, nullptr);
  m->pre.assign(m->layers.size(), nullptr);
  DDM_CUDA(cudaMalloc(&m->act[0], n * m->layers[0].in * sizeof(float)), "allocate activations");
  int widest = m->layers[0].in;
  for (size_t l = 0; l < m->layers.size(); l++) {
    DDM_CUDA(cudaMalloc(&m->act[l + 1], n * m->layers[l].out * sizeof(float)), "allocate activations");
    DDM_CUDA(cudaMalloc(&m->pre[l], n * m->layers[l].out * sizeof(float)), "allocate activations");
    widest = std::max(widest, m->layers[l].out);
  }
  DDM_CUDA(cudaMalloc(&m->d_grad_a, n * widest * sizeof(float)), "allocate gradients");
  DDM_CUDA(cudaMalloc(&m->d_grad_b, n * widest * sizeof(float)), "allocate gradients");
  DDM_CUDA(cudaMalloc(&m->d_target, n * sizeof(float)), "allocate targets");
  m->cap = n;
  return DD_OK;
}

// Forward over act[0] (n rows); leaves every layer's activations.
dd_status forward(dd_mlp *m, int n) {
  for (size_t l = 0; l < m->layers.size(); l++) {
    const Layer &L = m->layers[l];
    const unsigned blocks = (unsigned)((n + kRows - 1) / kRows);
    const unsigned threads = (unsigned)((L.out + 31) / 32 * 32);
    mlp_forward_kernel<<<blocks, threads>>>(m->act[l], m->d_pbf + L.wbf_off, m->d_p + L.b_off,
                                            m->pre[l], m->act[l + 1], n, L.in, L.out, L.relu);
  }
  DDM_CUDA(cudaGetLastError(), "mlp forward");
  return DD_OK;
}

// Loss and gradients of all parameters into d_g (targets in d_target).
dd_status backward(dd_mlp *m, int n) {
  const size_t L = m->layers.size();
  mse_kernel<<<1, 256>>>(m->act[L], m->d_target, m->d_grad_a, m->d_loss, n);
  float *dy = m->d_grad_a, *dx = m->d_grad_b;
  for (size_t li = L; li-- > 0;) {
    const Layer &ly = m->layers[li];
    const size_t count = (size_t)n * ly.out;
    if (ly.relu)
      relu_backward_kernel<<<(unsigned)((count + 255) / 256), 256>>>(dy, m->pre[li], count);
    mlp_backward_weight_kernel<<<ly.out, 128>>>(dy, m->act[li], m->d_g + ly.w_off,
                                                m->d_g + ly.b_off, n, ly.in, ly.out);
    if (li > 0) {
      const size_t cin = (size_t)n * ly.in;
      mlp_backward_input_kernel<<<(unsigned)((cin + 255) / 256), 256>>>(dy, m->d_pbf + ly.wbf_off,
                                                                       dx, n, ly.in, ly.out);
      std::swap(dy, dx);
    }
  }
  DDM_CUDA(cudaGetLastError(), "mlp backward");
  return DD_OK;
}

}  // namespace

extern "C" {

dd_status dd_mlp_create(dd_mlp **out, uint32_t in_features, uint32_t hidden, uint32_t hidden_layers,
                        uint64_t seed, int device) {
  if (!out) return fail(DD_ERR_INVALID_ARGUMENT, "NULL argument");
  *out = nullptr;
  if (in_features == 0 || in_features > kMaxWidth || hidden == 0 || hidden > kMaxWidth ||
      hidden % 32 || hidden_layers == 0)
    return fail(DD_ERR_INVALID_ARGUMENT, "inputs <= %d, hidden a multiple of 32 <= %d", kMaxWidth,
                kMaxWidth);
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    (void)cudaGetLastError();
    return fail(DD_ERR_NO_DEVICE, "no CUDA device available");
  }
  DDM_CUDA(cudaSetDevice(device), "select device");
  dd_mlp *m = new dd_mlp();
  m->device = device;
  int prev = (int)in_features;
  size_t off = 0, bf = 0;
  for (uint32_t l = 0; l <= hidden_layers; l++) {
    Layer L;
    L.in = prev;
    L.out = l == hidden_layers ? 1 : (int)hidden;
    L.relu = l != hidden_layers;
    L.w_off = off;
    off += (size_t)L.in * L.out;
    L.b_off = off;
    off += L.out;
    L.wbf_off = bf;
    bf += (size_t)L.in * L.out;
    m->layers.push_back(L);
    prev = L.out;
  }
  m->nparams = off;
  m->nbf = bf;
  // He initialisation from a seeded generator; zero biases.
  std::vector<float> p(off, 0.0f);
  std::vector<int> bfi(off, -1);
  std::mt19937_64 rng(seed);
  for (const Layer &L : m->layers) {
    std::normal_distribution<double> nd(0.0, std::sqrt(2.0 / L.in));
    for (size_t k = 0; k < (size_t)L.in * L.out; k++) {
      p[L.w_off + k] = (float)nd(rng);
      bfi[L.w_off + k] = (int)(L.wbf_off + k);
    }
  }
  auto bail = [&](dd_status st) {
    dd_mlp_destroy(m);
    return st;
  };
  cudaError_t e = cudaMalloc(&m->d_p, off * 4);
  if (e == cudaSuccess) e = cudaMalloc(&m->d_g, off * 4);
  if (e == cudaSuccess) e = cudaMalloc(&m->d_m, off * 4);
  if (e == cudaSuccess) e = cudaMalloc(&m->d_v, off * 4);
  if (e == cudaSuccess) e = cudaMalloc(&m->d_pbf, bf * 2);
  if (e == cudaSuccess) e = cudaMalloc(&m->d_bfi, off * 4);
  if (e == cudaSuccess) e = cudaMalloc(&m->d_loss, 4);
  if (e == cudaSuccess) e = cudaMemcpy(m->d_p, p.data(), off * 4, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(m->d_bfi, bfi.data(), off * 4, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemset(m->d_m, 0, off * 4);
  if (e == cudaSuccess) e = cudaMemset(m->d_v, 0, off * 4);
  if (e != cudaSuccess) return bail(cuda_fail(e, "allocate mlp"));
  to_bf16_kernel<<<(unsigned)((off + 255) / 256), 256>>>(m->d_p, m->d_pbf, m->d_bfi, off);
  e = cudaDeviceSynchronize();
  if (e != cudaSuccess) return bail(cuda_fail(e, "initialise mlp"));
  *out = m;
  return DD_OK;
}

dd_status dd_mlp_param_count(const dd_mlp *m, uint64_t *count) {
  if (!m || !count) return fail(DD_ERR_INVALID_ARGUMENT, "NULL argument");
  *count = m->nparams;
  return DD_OK;
}

dd_status dd_mlp_get_params(dd_mlp *m, float *params, uint64_t count) {
  if (!m || !params || count < m->nparams) return fail(DD_ERR_INVALID_ARGUMENT, "bad buffer");
  DDM_CUDA(cudaSetDevice(m->device), "select device");
  DDM_CUDA(cudaMemcpy(params, m->d_p, m->nparams * 4, cudaMemcpyDeviceToHost), "read parameters");
  return DD_OK;
}

dd_status dd_mlp_set_params(dd_mlp *m, const float *params, uint64_t count) {
  if (!m || !params || count < m->nparams) return fail(DD_ERR_INVALID_ARGUMENT, "bad buffer");
  DDM_CUDA(cudaSetDevice(m->device), "select device");
  DDM_CUDA(cudaMemcpy(m->d_p, params, m->nparams * 4, cudaMemcpyHostToDevice), "write parameters");
  to_bf16_kernel<<<(unsigned)((m->nparams + 255) / 256), 256>>>(m->d_p, m->d_pbf, m->d_bfi,
                                                               m->nparams);
  DDM_CUDA(cudaDeviceSynchronize(), "round parameters");
  return DD_OK;
}

dd_status dd_mlp_forward(dd_mlp *m, const float *x, uint32_t n, float *y) {
  if (!m || !x || !y) return fail(DD_ERR_INVALID_ARGUMENT, "NULL argument");
  if (n == 0) return DD_OK;
  DDM_CUDA(cudaSetDevice(m->device), "select device");
  dd_status st = ensure_batch(m, n);
  if (st) return st;
  DDM_CUDA(cudaMemcpy(m->act[0], x, (size_t)n * m->layers[0].in * 4, cudaMemcpyHostToDevice),
           "copy features");
  st = forward(m, (int)n);
  if (st) return st;
  DDM_CUDA(cudaMemcpy(y, m->act.back(), (size_t)n * 4, cudaMemcpyDeviceToHost), "copy predictions");
  return DD_OK;
}

dd_status dd_mlp_gradients(dd_mlp *m, const float *x, const float *target, uint32_t n,
                           float *grad, float *loss) {
  if (!m || !x || !target || !grad || n == 0) return fail(DD_ERR_INVALID_ARGUMENT, "bad argument");
  DDM_CUDA(cudaSetDevice(m->device), "select device");
  dd_status st = ensure_batch(m, n);
  if (st) return st;
  DDM_CUDA(cudaMemcpy(m->act[0], x, (size_t)n * m->layers[0].in * 4, cudaMemcpyHostToDevice),
           "copy features");
  DDM_CUDA(cudaMemcpy(m->d_target, target, (size_t)n * 4, cudaMemcpyHostToDevice), "copy targets");
  st = forward(m, (int)n);
  if (!st) st = backward(m, (int)n);
  if (st) return st;
  DDM_CUDA(cudaMemcpy(grad, m->d_g, m->nparams * 4, cudaMemcpyDeviceToHost), "copy gradients");
  if (loss) DDM_CUDA(cudaMemcpy(loss, m->d_loss, 4, cudaMemcpyDeviceToHost), "copy loss");
  return DD_OK;
}

dd_status dd_mlp_train(dd_mlp *m, const float *x, const float *target, uint32_t n, uint32_t steps,
                       float lr, float *final_loss) {
  if (!m || !x || !target || n == 0) return fail(DD_ERR_INVALID_ARGUMENT, "bad argument");
  DDM_CUDA(cudaSetDevice(m->device), "select device");
  dd_status st = ensure_batch(m, n);
  if (st) return st;
  DDM_CUDA(cudaMemcpy(m->act[0], x, (size_t)n * m->layers[0].in * 4, cudaMemcpyHostToDevice),
           "copy features");
  DDM_CUDA(cudaMemcpy(m->d_target, target, (size_t)n * 4, cudaMemcpyHostToDevice), "copy targets");
  const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
  for (uint32_t s = 0; s < steps; s++) {
    st = forward(m, (int)n);
    if (!st) st = backward(m, (int)n);
    if (st) return st;
    m->step++;
    const float c1 = 1.0f - std::pow(b1, (float)m->step);
    const float c2 = 1.0f - std::pow(b2, (float)m->step);
    adam_kernel<<<(unsigned)((m->nparams + 255) / 256), 256>>>(
        m->d_p, m->d_g, m->d_m, m->d_v, m->d_pbf, m->d_bfi, m->nparams, lr, b1, b2, eps, c1, c2);
  }
  DDM_CUDA(cudaGetLastError(), "mlp train");
  // loss of the final parameters
  st = forward(m, (int)n);
  if (!st) st = backward(m, (int)n);
  if (st) return st;
  if (final_loss) DDM_CUDA(cudaMemcpy(final_loss, m->d_loss, 4, cudaMemcpyDeviceToHost), "copy loss");
  return DD_OK;
}

dd_status dd_mlp_destroy(dd_mlp *m) {
  if (!m) return DD_OK;
  cudaSetDevice(m->device);
  free_batch(m);
  for (void *p : {(void *)m->d_p, (void *)m->d_g, (void *)m->d_m, (void *)m->d_v,
                  (void *)m->d_pbf, (void *)m->d_bfi, (void *)m->d_loss})
    if (p) cudaFree(p);
  delete m;
  return DD_OK;
}

}  // extern "C"
