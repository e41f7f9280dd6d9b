// The scheduler's network: a 3-layer perceptron, 5 inputs -> 64 -> 64 -> 1,
// ReLU hidden layers and a sigmoid output (predicted next-iteration active
// edge fraction of a vertex range).  Weights are stored in BF16, every sum is
// accumulated in FP32.  Shared by the training kernels (sgw_mlp.cu) and the
// engine's per-iteration range statistics kernel (sgw_kernels.cuh).
#pragma once

#include <cuda_bf16.h>
#include <stdint.h>

namespace sgw {

constexpr int kMlpIn = 5;
constexpr int kMlpHidden = 64;
// flat parameter layout: W1[H][IN], b1[H], W2[H][H], b2[H], W3[H], b3
constexpr int kMlpOffW1 = 0;
constexpr int kMlpOffB1 = kMlpOffW1 + kMlpHidden * kMlpIn;
constexpr int kMlpOffW2 = kMlpOffB1 + kMlpHidden;
constexpr int kMlpOffB2 = kMlpOffW2 + kMlpHidden * kMlpHidden;
constexpr int kMlpOffW3 = kMlpOffB2 + kMlpHidden;
constexpr int kMlpOffB3 = kMlpOffW3 + kMlpHidden;
constexpr int kMlpParams = kMlpOffB3 + 1;  // 4609

__device__ __forceinline__ float mlp_w(const __nv_bfloat16 *p, int i) { return __bfloat162float(p[i]); }

__device__ __forceinline__ float sigmoidf_(float z) { return 1.0f / (1.0f + __expf(-z)); }

// Forward pass of one sample by one warp: lane l owns hidden units l and
// l + 32 of both hidden layers.  Returns the output on every lane.
__device__ __forceinline__ float mlp_forward_warp(const __nv_bfloat16 *w, const float x[kMlpIn], int lane) {
  float h1[2], h2[2];
#pragma unroll
  for (int r = 0; r < 2; ++r) {
    const int u = lane + 32 * r;
    float z = mlp_w(w, kMlpOffB1 + u);
#pragma unroll
    for (int k = 0; k < kMlpIn; ++k) z += mlp_w(w, kMlpOffW1 + u * kMlpIn + k) * x[k];
    h1[r] = fmaxf(z, 0.0f);
  }
  float z2[2] = {mlp_w(w, kMlpOffB2 + lane), mlp_w(w, kMlpOffB2 + lane + 32)};
  for (int j = 0; j < kMlpHidden; ++j) {
    const float hj = __shfl_sync(0xffffffffu, h1[j >> 5], j & 31);
#pragma unroll
    for (int r = 0; r < 2; ++r) z2[r] += mlp_w(w, kMlpOffW2 + (lane + 32 * r) * kMlpHidden + j) * hj;
  }
  h2[0] = fmaxf(z2[0], 0.0f);
  h2[1] = fmaxf(z2[1], 0.0f);
  float z3 = mlp_w(w, kMlpOffW3 + lane) * h2[0] + mlp_w(w, kMlpOffW3 + lane + 32) * h2[1];
#pragma unroll
  for (int d = 16; d > 0; d >>= 1) z3 += __shfl_xor_sync(0xffffffffu, z3, d);
  return sigmoidf_(z3 + mlp_w(w, kMlpOffB3));
}

}  // namespace sgw
