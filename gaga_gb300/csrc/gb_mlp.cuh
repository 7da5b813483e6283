// gb_mlp.cuh -- the learned warm start's network: parameter layout, activation, features and
// the per-coordinate forward pass (shared by gb_learned.cu and the resident kernel).
#pragma once
#include <cuda_bf16.h>

#define ML_IN 4
#define ML_H 64
#define ML_OFF_W1 0
#define ML_OFF_B1 (ML_OFF_W1 + ML_H * ML_IN)
#define ML_OFF_W2 (ML_OFF_B1 + ML_H)
#define ML_OFF_B2 (ML_OFF_W2 + ML_H * ML_H)
#define ML_OFF_W3 (ML_OFF_B2 + ML_H)
#define ML_OFF_B3 (ML_OFF_W3 + ML_H)
#define ML_P (ML_OFF_B3 + 1)  // 4545 parameters
#define ML_RANK_BINS 4096

static_assert(ML_P == 4545, "parameter count");

__device__ __forceinline__ float ml_gelu(float a) { return 0.5f * a * (1.0f + erff(a * 0.70710678118654752f)); }
__device__ __forceinline__ float ml_gelu_grad(float a) {
  return 0.5f * (1.0f + erff(a * 0.70710678118654752f)) + a * 0.39894228040143268f * expf(-0.5f * a * a);
}
__device__ __forceinline__ float ml_bf16(float v) { return __bfloat162float(__float2bfloat16_rn(v)); }

__device__ __forceinline__ void ml_features(float gi, float gmax, int b, const int *cum, const int *counts, int n,
                                            float delta, float rho, float f[ML_IN]) {
  f[0] = gmax > 0.0f ? fabsf(gi) / gmax : 0.0f;
  f[1] = ((float)cum[b] + 0.5f * (float)counts[b]) / (float)n;
  f[2] = delta;
  f[3] = rho;
}

// the parameters, BF16-rounded, into shared memory
static __device__ void ml_load_params(const float *__restrict__ p, float *sp) {
  for (int i = threadIdx.x; i < ML_P; i += blockDim.x) sp[i] = ml_bf16(p[i]);
  __syncthreads();
}

// one coordinate through the network (thread-local, weights in shared memory)
static __device__ float ml_forward1(const float *sp, const float f[ML_IN]) {
  float h1[ML_H];
#pragma unroll
  for (int j = 0; j < ML_H; ++j) {
    float a = sp[ML_OFF_B1 + j];
#pragma unroll
    for (int q = 0; q < ML_IN; ++q) a = fmaf(sp[ML_OFF_W1 + j * ML_IN + q], f[q], a);
    h1[j] = ml_gelu(a);
  }
  float out = sp[ML_OFF_B3];
  for (int j = 0; j < ML_H; ++j) {
    float a = sp[ML_OFF_B2 + j];
    const float *w = sp + ML_OFF_W2 + j * ML_H;
#pragma unroll
    for (int i = 0; i < ML_H; ++i) a = fmaf(w[i], h1[i], a);
    out = fmaf(sp[ML_OFF_W3 + j], ml_gelu(a), out);
  }
  return out;
}

