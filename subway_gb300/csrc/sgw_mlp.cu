// Training and batch inference of the scheduler's network (sgw_mlp.cuh):
// BF16 weights, FP32 accumulation, FP32 master weights updated by Adam.
//
// One training step on n samples:
//   k_mlp_forward   thread per sample: hidden activations and the output
//   k_mlp_backward  thread per sample: output and hidden-layer errors of the
//                   binary cross-entropy loss
//   k_mlp_grad      (parameter, sample-chunk) per thread: error x activation
//                   sums, accumulated into the FP32 gradient
//   k_mlp_adam      thread per parameter: Adam on the FP32 master, BF16 copy
// No counterpart in the reference (it has no scheduler).

#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <cmath>
#include <vector>

#include "sgw_internal.h"
#include "sgw_mlp.cuh"

using namespace sgw;

#define CK(call)                                                                       \
  do {                                                                                 \
    cudaError_t _e = (call);                                                           \
    if (_e != cudaSuccess)                                                             \
      return fail(SGW_ECUDA, "%s failed: %s (%s:%d)", #call, cudaGetErrorString(_e), \
                  __FILE__, __LINE__);                                                 \
  } while (0)

struct sgw_mlp {
  int device = 0;
  float *d_master = nullptr;          // FP32 masters
  __nv_bfloat16 *d_w = nullptr;       // BF16 weights used by every pass
  float *d_m = nullptr, *d_v = nullptr, *d_grad = nullptr;
  float *d_loss = nullptr;
  uint64_t step = 0;
  // per-sample scratch, grown on demand
  uint32_t cap_n = 0;
  float *d_x = nullptr, *d_t = nullptr, *d_y = nullptr;
  float *d_h1 = nullptr, *d_h2 = nullptr, *d_e1 = nullptr, *d_e2 = nullptr, *d_e3 = nullptr;
};

namespace {

constexpr int kT = 128;

__global__ void k_mlp_forward(const __nv_bfloat16 *__restrict__ w, const float *__restrict__ x,
                              uint32_t n, float *__restrict__ y, float *__restrict__ h1o,
                              float *__restrict__ h2o) {
  __shared__ float sw[kMlpParams];
  for (int i = threadIdx.x; i < kMlpParams; i += blockDim.x) sw[i] = __bfloat162float(w[i]);
  __syncthreads();
  const uint32_t b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= n) return;
  float xi[kMlpIn];
#pragma unroll
  for (int k = 0; k < kMlpIn; ++k) xi[k] = x[(size_t)b * kMlpIn + k];
  float h1[kMlpHidden];
#pragma unroll
  for (int u = 0; u < kMlpHidden; ++u) {
    float z = sw[kMlpOffB1 + u];
#pragma unroll
    for (int k = 0; k < kMlpIn; ++k) z += sw[kMlpOffW1 + u * kMlpIn + k] * xi[k];
    h1[u] = fmaxf(z, 0.0f);
    if (h1o) h1o[(size_t)b * kMlpHidden + u] = h1[u];
  }
  float z3 = sw[kMlpOffB3];
  for (int u = 0; u < kMlpHidden; ++u) {
    float z = sw[kMlpOffB2 + u];
#pragma unroll
    for (int j = 0; j < kMlpHidden; ++j) z += sw[kMlpOffW2 + u * kMlpHidden + j] * h1[j];
    const float h = fmaxf(z, 0.0f);
    if (h2o) h2o[(size_t)b * kMlpHidden + u] = h;
    z3 += sw[kMlpOffW3 + u] * h;
  }
  y[b] = sigmoidf_(z3);
}

// Errors of the mean binary cross-entropy: e3 = (y - t) / n at the output,
// e2 = e3 * W3 masked by ReLU', e1 = W2^T e2 masked by ReLU'.
__global__ void k_mlp_backward(const __nv_bfloat16 *__restrict__ w, const float *__restrict__ t,
                               const float *__restrict__ y, const float *__restrict__ h1,
                               const float *__restrict__ h2, uint32_t n, float *__restrict__ e1,
                               float *__restrict__ e2, float *__restrict__ e3, float *loss) {
  __shared__ float sw[kMlpParams];
  __shared__ float s_loss[kT / 32];
  for (int i = threadIdx.x; i < kMlpParams; i += blockDim.x) sw[i] = __bfloat162float(w[i]);
  __syncthreads();
  const uint32_t b = blockIdx.x * blockDim.x + threadIdx.x;
  float l = 0.0f;
  if (b < n) {
    const float yb = y[b], tb = t[b];
    const float eps = 1e-7f;
    const float yc = fminf(fmaxf(yb, eps), 1.0f - eps);
    l = -(tb * logf(yc) + (1.0f - tb) * logf(1.0f - yc)) / (float)n;
    const float d3 = (yb - tb) / (float)n;
    e3[b] = d3;
    float d2[kMlpHidden];
#pragma unroll
    for (int j = 0; j < kMlpHidden; ++j) {
      d2[j] = h2[(size_t)b * kMlpHidden + j] > 0.0f ? d3 * sw[kMlpOffW3 + j] : 0.0f;
      e2[(size_t)b * kMlpHidden + j] = d2[j];
    }
    for (int k = 0; k < kMlpHidden; ++k) {
      float s = 0.0f;
#pragma unroll
      for (int j = 0; j < kMlpHidden; ++j) s += sw[kMlpOffW2 + j * kMlpHidden + k] * d2[j];
      e1[(size_t)b * kMlpHidden + k] = h1[(size_t)b * kMlpHidden + k] > 0.0f ? s : 0.0f;
    }
  }
#pragma unroll
  for (int d = 16; d > 0; d >>= 1) l += __shfl_xor_sync(0xffffffffu, l, d);
  if ((threadIdx.x & 31) == 0) s_loss[threadIdx.x >> 5] = l;
  __syncthreads();
  if (threadIdx.x == 0) {
    float s = 0.0f;
    for (int i = 0; i < kT / 32; ++i) s += s_loss[i];
    atomicAdd(loss, s);
  }
}

// Gradient of parameter p summed over samples [c * chunk, (c+1) * chunk).
__global__ void k_mlp_grad(const float *__restrict__ x, const float *__restrict__ h1,
                           const float *__restrict__ h2, const float *__restrict__ e1,
                           const float *__restrict__ e2, const float *__restrict__ e3, uint32_t n,
                           uint32_t chunk, float *__restrict__ grad) {
  const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= (uint32_t)kMlpParams) return;
  const uint32_t b0 = blockIdx.y * chunk, b1 = min(n, b0 + chunk);
  float s = 0.0f;
  if (p < (uint32_t)kMlpOffB1) {
    const uint32_t i = p / kMlpIn, k = p % kMlpIn;
    for (uint32_t b = b0; b < b1; ++b) s += e1[(size_t)b * kMlpHidden + i] * x[(size_t)b * kMlpIn + k];
  } else if (p < (uint32_t)kMlpOffW2) {
    const uint32_t i = p - kMlpOffB1;
    for (uint32_t b = b0; b < b1; ++b) s += e1[(size_t)b * kMlpHidden + i];
  } else if (p < (uint32_t)kMlpOffB2) {
    const uint32_t q = p - kMlpOffW2, i = q / kMlpHidden, j = q % kMlpHidden;
    for (uint32_t b = b0; b < b1; ++b) s += e2[(size_t)b * kMlpHidden + i] * h1[(size_t)b * kMlpHidden + j];
  } else if (p < (uint32_t)kMlpOffW3) {
    const uint32_t i = p - kMlpOffB2;
    for (uint32_t b = b0; b < b1; ++b) s += e2[(size_t)b * kMlpHidden + i];
  } else if (p < (uint32_t)kMlpOffB3) {
    const uint32_t j = p - kMlpOffW3;
    for (uint32_t b = b0; b < b1; ++b) s += e3[b] * h2[(size_t)b * kMlpHidden + j];
  } else {
    for (uint32_t b = b0; b < b1; ++b) s += e3[b];
  }
  if (b1 > b0) atomicAdd(&grad[p], s);
}

// Adam (Kingma and Ba, ICLR 2015) on the FP32 masters; refreshes the BF16
// copy and clears the gradient.
__global__ void k_mlp_adam(float *master, __nv_bfloat16 *w, float *grad, float *m, float *v, float lr,
                           float beta1, float beta2, float eps, float c1, float c2) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= kMlpParams) return;
  const float g = grad[p];
  const float mp = beta1 * m[p] + (1.0f - beta1) * g;
  const float vp = beta2 * v[p] + (1.0f - beta2) * g * g;
  m[p] = mp;
  v[p] = vp;
  const float upd = lr * (mp / c1) / (sqrtf(vp / c2) + eps);
  master[p] -= upd;
  w[p] = __float2bfloat16(master[p]);
  grad[p] = 0.0f;
}

__global__ void k_mlp_cast(const float *master, __nv_bfloat16 *w) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p < kMlpParams) w[p] = __float2bfloat16(master[p]);
}

int ensure_scratch(sgw_mlp *m, uint32_t n) {
  if (n <= m->cap_n) return SGW_OK;
  cudaFree(m->d_x); cudaFree(m->d_t); cudaFree(m->d_y);
  cudaFree(m->d_h1); cudaFree(m->d_h2); cudaFree(m->d_e1); cudaFree(m->d_e2); cudaFree(m->d_e3);
  m->d_x = m->d_t = m->d_y = m->d_h1 = m->d_h2 = m->d_e1 = m->d_e2 = m->d_e3 = nullptr;
  m->cap_n = 0;
  const size_t nh = (size_t)n * kMlpHidden * sizeof(float);
  CK(cudaMalloc(&m->d_x, (size_t)n * kMlpIn * sizeof(float)));
  CK(cudaMalloc(&m->d_t, (size_t)n * sizeof(float)));
  CK(cudaMalloc(&m->d_y, (size_t)n * sizeof(float)));
  CK(cudaMalloc(&m->d_e3, (size_t)n * sizeof(float)));
  CK(cudaMalloc(&m->d_h1, nh));
  CK(cudaMalloc(&m->d_h2, nh));
  CK(cudaMalloc(&m->d_e1, nh));
  CK(cudaMalloc(&m->d_e2, nh));
  m->cap_n = n;
  return SGW_OK;
}

// One forward + backward pass over the samples already on the device; the
// gradient is accumulated into d_grad (cleared by the caller or by Adam).
int pass(sgw_mlp *m, uint32_t n, float *loss_out) {
  const uint32_t blocks = (n + kT - 1) / kT;
  k_mlp_forward<<<blocks, kT>>>(m->d_w, m->d_x, n, m->d_y, m->d_h1, m->d_h2);
  CK(cudaGetLastError());
  CK(cudaMemset(m->d_loss, 0, sizeof(float)));
  k_mlp_backward<<<blocks, kT>>>(m->d_w, m->d_t, m->d_y, m->d_h1, m->d_h2, n, m->d_e1, m->d_e2, m->d_e3,
                                 m->d_loss);
  CK(cudaGetLastError());
  const uint32_t chunk = std::max<uint32_t>(64, (n + 255) / 256);
  dim3 grid((kMlpParams + 255) / 256, (n + chunk - 1) / chunk);
  k_mlp_grad<<<grid, 256>>>(m->d_x, m->d_h1, m->d_h2, m->d_e1, m->d_e2, m->d_e3, n, chunk, m->d_grad);
  CK(cudaGetLastError());
  if (loss_out) CK(cudaMemcpy(loss_out, m->d_loss, sizeof(float), cudaMemcpyDeviceToHost));
  return SGW_OK;
}

uint64_t mix64(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
  return z ^ (z >> 31);
}

}  // namespace

extern "C" {

int sgw_mlp_create(int device, uint64_t seed, sgw_mlp **out) {
  clear_error();
  if (!out) return fail(SGW_EINVAL, "null argument");
  *out = nullptr;
  CK(cudaSetDevice(device));
  sgw_mlp *m = new (std::nothrow) sgw_mlp();
  if (!m) return fail(SGW_ENOMEM, "mlp object");
  m->device = device;
  const size_t pb = kMlpParams * sizeof(float);
  if (cudaMalloc(&m->d_master, pb) != cudaSuccess || cudaMalloc(&m->d_w, kMlpParams * 2) != cudaSuccess ||
      cudaMalloc(&m->d_m, pb) != cudaSuccess || cudaMalloc(&m->d_v, pb) != cudaSuccess ||
      cudaMalloc(&m->d_grad, pb) != cudaSuccess || cudaMalloc(&m->d_loss, sizeof(float)) != cudaSuccess) {
    sgw_mlp_destroy(m);
    return fail(SGW_ECUDA, "mlp allocation");
  }
  // He-uniform initialisation from SplitMix64; biases start at zero.
  std::vector<float> p(kMlpParams, 0.0f);
  uint64_t s = mix64(seed ^ 0x1f83d9abfb41bd6bULL);
  auto unif = [&]() { s += 0x9e3779b97f4a7c15ULL; return (mix64(s) >> 11) * (1.0 / 9007199254740992.0); };
  auto fill = [&](int off, int cnt, int fan_in) {
    const double a = std::sqrt(6.0 / fan_in);
    for (int i = 0; i < cnt; ++i) p[off + i] = (float)((2.0 * unif() - 1.0) * a);
  };
  fill(kMlpOffW1, kMlpHidden * kMlpIn, kMlpIn);
  fill(kMlpOffW2, kMlpHidden * kMlpHidden, kMlpHidden);
  fill(kMlpOffW3, kMlpHidden, kMlpHidden);
  int st = sgw_mlp_set_params(m, p.data());
  if (st != SGW_OK) { sgw_mlp_destroy(m); return st; }
  *out = m;
  return SGW_OK;
}

int sgw_mlp_destroy(sgw_mlp *m) {
  if (!m) return SGW_OK;
  cudaSetDevice(m->device);
  cudaFree(m->d_master); cudaFree(m->d_w); cudaFree(m->d_m); cudaFree(m->d_v); cudaFree(m->d_grad);
  cudaFree(m->d_loss);
  cudaFree(m->d_x); cudaFree(m->d_t); cudaFree(m->d_y);
  cudaFree(m->d_h1); cudaFree(m->d_h2); cudaFree(m->d_e1); cudaFree(m->d_e2); cudaFree(m->d_e3);
  cudaGetLastError();
  delete m;
  return SGW_OK;
}

int sgw_mlp_set_params(sgw_mlp *m, const float *params) {
  clear_error();
  if (!m || !params) return fail(SGW_EINVAL, "null argument");
  CK(cudaSetDevice(m->device));
  CK(cudaMemcpy(m->d_master, params, kMlpParams * sizeof(float), cudaMemcpyHostToDevice));
  k_mlp_cast<<<(kMlpParams + 255) / 256, 256>>>(m->d_master, m->d_w);
  CK(cudaGetLastError());
  CK(cudaMemset(m->d_m, 0, kMlpParams * sizeof(float)));
  CK(cudaMemset(m->d_v, 0, kMlpParams * sizeof(float)));
  CK(cudaMemset(m->d_grad, 0, kMlpParams * sizeof(float)));
  CK(cudaDeviceSynchronize());
  m->step = 0;
  return SGW_OK;
}

int sgw_mlp_get_params(const sgw_mlp *m, float *params) {
  clear_error();
  if (!m || !params) return fail(SGW_EINVAL, "null argument");
  CK(cudaSetDevice(m->device));
  std::vector<__nv_bfloat16> w(kMlpParams);
  CK(cudaMemcpy(w.data(), m->d_w, kMlpParams * 2, cudaMemcpyDeviceToHost));
  for (int i = 0; i < kMlpParams; ++i) params[i] = __bfloat162float(w[i]);
  return SGW_OK;
}

int sgw_mlp_forward(sgw_mlp *m, const float *x, uint32_t n, float *y) {
  clear_error();
  if (!m || !x || !y) return fail(SGW_EINVAL, "null argument");
  if (n == 0) return SGW_OK;
  CK(cudaSetDevice(m->device));
  int st = ensure_scratch(m, n);
  if (st != SGW_OK) return st;
  CK(cudaMemcpy(m->d_x, x, (size_t)n * kMlpIn * sizeof(float), cudaMemcpyHostToDevice));
  k_mlp_forward<<<(n + kT - 1) / kT, kT>>>(m->d_w, m->d_x, n, m->d_y, nullptr, nullptr);
  CK(cudaGetLastError());
  CK(cudaMemcpy(y, m->d_y, (size_t)n * sizeof(float), cudaMemcpyDeviceToHost));
  return SGW_OK;
}

int sgw_mlp_gradient(sgw_mlp *m, const float *x, const float *t, uint32_t n, float *grad, float *loss) {
  clear_error();
  if (!m || !x || !t || !grad || n == 0) return fail(SGW_EINVAL, "bad argument");
  CK(cudaSetDevice(m->device));
  int st = ensure_scratch(m, n);
  if (st != SGW_OK) return st;
  CK(cudaMemcpy(m->d_x, x, (size_t)n * kMlpIn * sizeof(float), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(m->d_t, t, (size_t)n * sizeof(float), cudaMemcpyHostToDevice));
  CK(cudaMemset(m->d_grad, 0, kMlpParams * sizeof(float)));
  st = pass(m, n, loss);
  if (st != SGW_OK) return st;
  CK(cudaMemcpy(grad, m->d_grad, kMlpParams * sizeof(float), cudaMemcpyDeviceToHost));
  CK(cudaMemset(m->d_grad, 0, kMlpParams * sizeof(float)));
  return SGW_OK;
}

int sgw_mlp_train(sgw_mlp *m, const float *x, const float *t, uint32_t n, uint32_t steps, float lr,
                  float *loss) {
  clear_error();
  if (!m || !x || !t || n == 0 || !(lr > 0.0f)) return fail(SGW_EINVAL, "bad argument");
  CK(cudaSetDevice(m->device));
  int st = ensure_scratch(m, n);
  if (st != SGW_OK) return st;
  CK(cudaMemcpy(m->d_x, x, (size_t)n * kMlpIn * sizeof(float), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(m->d_t, t, (size_t)n * sizeof(float), cudaMemcpyHostToDevice));
  CK(cudaMemset(m->d_grad, 0, kMlpParams * sizeof(float)));
  const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
  for (uint32_t k = 0; k < steps; ++k) {
    st = pass(m, n, nullptr);
    if (st != SGW_OK) return st;
    ++m->step;
    const float c1 = 1.0f - std::pow(b1, (float)m->step), c2 = 1.0f - std::pow(b2, (float)m->step);
    k_mlp_adam<<<(kMlpParams + 255) / 256, 256>>>(m->d_master, m->d_w, m->d_grad, m->d_m, m->d_v, lr, b1, b2,
                                                  eps, c1, c2);
    CK(cudaGetLastError());
  }
  // loss of the final weights
  st = pass(m, n, loss);
  if (st != SGW_OK) return st;
  CK(cudaMemset(m->d_grad, 0, kMlpParams * sizeof(float)));
  CK(cudaDeviceSynchronize());
  return SGW_OK;
}

// File: "SGWMLP1\0", u32 inputs, u32 hidden, then the FP32 masters.
int sgw_mlp_save(const sgw_mlp *m, const char *path) {
  clear_error();
  if (!m || !path) return fail(SGW_EINVAL, "null argument");
  CK(cudaSetDevice(m->device));
  std::vector<float> p(kMlpParams);
  CK(cudaMemcpy(p.data(), m->d_master, kMlpParams * sizeof(float), cudaMemcpyDeviceToHost));
  FILE *f = fopen(path, "wb");
  if (!f) return fail(SGW_EIO, "cannot create %s", path);
  const char magic[8] = {'S', 'G', 'W', 'M', 'L', 'P', '1', 0};
  const uint32_t dims[2] = {(uint32_t)kMlpIn, (uint32_t)kMlpHidden};
  bool ok = fwrite(magic, 1, 8, f) == 8 && fwrite(dims, 4, 2, f) == 2 &&
            fwrite(p.data(), 4, kMlpParams, f) == (size_t)kMlpParams;
  ok = (fclose(f) == 0) && ok;
  return ok ? SGW_OK : fail(SGW_EIO, "write failed for %s", path);
}

int sgw_mlp_load(int device, const char *path, sgw_mlp **out) {
  clear_error();
  if (!path || !out) return fail(SGW_EINVAL, "null argument");
  *out = nullptr;
  FILE *f = fopen(path, "rb");
  if (!f) return fail(SGW_EIO, "cannot open %s", path);
  char magic[8];
  uint32_t dims[2];
  std::vector<float> p(kMlpParams);
  bool ok = fread(magic, 1, 8, f) == 8 && memcmp(magic, "SGWMLP1", 8) == 0 && fread(dims, 4, 2, f) == 2 &&
            dims[0] == (uint32_t)kMlpIn && dims[1] == (uint32_t)kMlpHidden &&
            fread(p.data(), 4, kMlpParams, f) == (size_t)kMlpParams;
  fclose(f);
  if (!ok) return fail(SGW_EFORMAT, "%s is not a scheduler model", path);
  sgw_mlp *m = nullptr;
  int st = sgw_mlp_create(device, 0, &m);
  if (st != SGW_OK) return st;
  st = sgw_mlp_set_params(m, p.data());
  if (st != SGW_OK) { sgw_mlp_destroy(m); return st; }
  *out = m;
  return SGW_OK;
}

}  // extern "C"

namespace sgw {
const void *mlp_device_weights(const sgw_mlp *m) { return m ? m->d_w : nullptr; }
int mlp_device(const sgw_mlp *m) { return m ? m->device : -1; }
}  // namespace sgw
