// gb_learned.cu -- learned warm start for CGIHT: a per-coordinate MLP 4 -> 64 -> 64 -> 1.
//
// Features of coordinate i of a problem (y, A, k):  g = A^T y,
//   f0 = |g_i| / max_j |g_j|          f1 = rank fraction of |g_i| (0 = largest)
//   f2 = delta = m / n                f3 = rho = k / m
// The network (GELU hidden layers, weights rounded to BF16 at every use, FP32 math and
// accumulation) predicts w_i = x_i / g_i of the final solution, so x0 = H_k(w . g) proposes
// both the initial support and a per-coordinate step.  The rank fraction comes from a
// 4096-bin histogram of |g| (bin 0 holds the largest magnitudes): (coordinates in
// larger-magnitude bins + half of the own bin) / n.
//
// Training runs on the GPU with the kernels below: a forward + backward kernel that
// accumulates each block's gradient in shared memory in a fixed order, and a kernel that
// sums the block partials in block order (deterministic) and applies an Adam step.
//
// Parameter layout (FP32 master copy): W1[64][4] b1[64] W2[64][64] b2[64] W3[64] b3.
#include <cuda_bf16.h>
#include <math.h>
#include <string.h>

#include <algorithm>
#include <random>
#include <vector>

#include "gb_internal.cuh"

#include "gb_mlp.cuh"

#define ML_TILE 64            // samples per training tile
#define ML_TRAIN_BLOCKS 64

// ------------------------------------------------------------------ features
// histogram of |g| over ML_RANK_BINS bins below max|g| (read from red[R_XMAX] when st is
// given, else from *gmax)
__global__ void k_ml_rank_hist(const GbState *st, int pf, const float *__restrict__ g, int n, const float *gmax,
                               int *__restrict__ bins, int *__restrict__ counts) {
  if (st && !gb_pred(st, pf)) return;
  if (st) n = dimv(st, n);
  const float mx = st ? (float)st->red[R_XMAX] : *gmax;
  const float slope = mx > 0.0f ? (float)(ML_RANK_BINS - 1) / mx : 0.0f;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    int b = (int)((mx - fabsf(g[i])) * slope);
    b = min(max(b, 0), ML_RANK_BINS - 1);
    bins[i] = b;
    atomicAdd(&counts[b], 1);
  }
}

// counts -> exclusive prefix (cum), one block of 1024 threads, 4 bins each
__global__ void __launch_bounds__(1024) k_ml_rank_scan(const GbState *st, int pf, const int *__restrict__ counts,
                                                       int *__restrict__ cum) {
  if (st && !gb_pred(st, pf)) return;
  __shared__ int s[1024];
  const int t = threadIdx.x;
  int c[4], tot = 0;
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    c[q] = counts[t * 4 + q];
    tot += c[q];
  }
  s[t] = tot;
  __syncthreads();
  for (int off = 1; off < 1024; off <<= 1) {
    const int v = t >= off ? s[t - off] : 0;
    __syncthreads();
    s[t] += v;
    __syncthreads();
  }
  int run = s[t] - tot;
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    cum[t * 4 + q] = run;
    run += c[q];
  }
}

// features of every coordinate (n x 4, row-major) for training data
__global__ void k_ml_features(const float *__restrict__ g, int n, const float *gmax, const int *__restrict__ bins,
                              const int *__restrict__ cum, const int *__restrict__ counts, float delta, float rho,
                              float *__restrict__ feat) {
  const float mx = *gmax;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    float f[ML_IN];
    ml_features(g[i], mx, bins[i], cum, counts, n, delta, rho, f);
#pragma unroll
    for (int q = 0; q < ML_IN; ++q) feat[(size_t)i * ML_IN + q] = f[q];
  }
}

// solver prologue: x_i = g_i * net(features_i) with g = A^T y in x on entry
__global__ void __launch_bounds__(256) k_ml_warm(const GbState *st, int pf, float *__restrict__ x, int n,
                                                 const int *__restrict__ bins, const int *__restrict__ cum,
                                                 const int *__restrict__ counts, const float *__restrict__ params) {
  if (!gb_pred(st, pf)) return;
  __shared__ float sp[ML_P];
  n = dimv(st, n);
  ml_load_params(params, sp);
  const float mx = (float)st->red[R_XMAX];
  const float delta = (float)st->m / (float)st->n, rho = (float)st->k / (float)st->m;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const float gi = x[i];
    float f[ML_IN];
    ml_features(gi, mx, bins[i], cum, counts, n, delta, rho, f);
    x[i] = gi * ml_forward1(sp, f);
  }
}

// plain inference on feature rows (tests and evaluation)
__global__ void __launch_bounds__(256) k_ml_forward(const float *__restrict__ params, const float *__restrict__ feat,
                                                    int ns, float *__restrict__ out) {
  __shared__ float sp[ML_P];
  ml_load_params(params, sp);
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < ns; i += gridDim.x * blockDim.x) {
    float f[ML_IN];
#pragma unroll
    for (int q = 0; q < ML_IN; ++q) f[q] = feat[(size_t)i * ML_IN + q];
    out[i] = ml_forward1(sp, f);
  }
}

// ------------------------------------------------------------------ training
// Gradient of L = sum_s (out_s - t_s)^2 * scale over the samples idx[0 .. ns) assigned to
// this block (tiles blockIdx.x, blockIdx.x + gridDim.x, ...), BF16-rounded weights in the
// forward pass.  Each gradient entry is accumulated by one fixed thread in sample order;
// the block's partial goes to partial[blockIdx.x][ML_P], its loss to lossp[blockIdx.x].
__global__ void __launch_bounds__(256) k_ml_grad(const float *__restrict__ params, const float *__restrict__ feat,
                                                 const float *__restrict__ tgt, const int *__restrict__ idx, int ns,
                                                 float scale, float *__restrict__ partial,
                                                 float *__restrict__ lossp) {
  extern __shared__ float ml_sm[];
  float *sp = ml_sm;                       // ML_P
  float *gp = sp + ML_P;                   // ML_P gradient accumulators
  float *F = gp + ML_P;                    // [ML_TILE][4]
  float *A1 = F + ML_TILE * ML_IN;         // [ML_TILE][64] pre-activations
  float *H1 = A1 + ML_TILE * ML_H;         // [ML_TILE][64] gelu(A1), later dA1
  float *A2 = H1 + ML_TILE * ML_H;         // [ML_TILE][64]
  float *D2 = A2 + ML_TILE * ML_H;         // [ML_TILE][64] dA2
  float *dout = D2 + ML_TILE * ML_H;       // [ML_TILE]
  __shared__ float red[8];
  const int t = threadIdx.x;
  ml_load_params(params, sp);
  for (int i = t; i < ML_P; i += 256) gp[i] = 0.0f;
  float loss = 0.0f;
  const int ntiles = (ns + ML_TILE - 1) / ML_TILE;
  for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const int s0 = tile * ML_TILE, cnt = min(ML_TILE, ns - s0);
    __syncthreads();
    for (int e = t; e < ML_TILE * ML_IN; e += 256) {
      const int s = e / ML_IN, q = e % ML_IN;
      F[e] = s < cnt ? feat[(size_t)idx[s0 + s] * ML_IN + q] : 0.0f;
    }
    __syncthreads();
    // layer 1
    for (int e = t; e < ML_TILE * ML_H; e += 256) {
      const int s = e / ML_H, j = e % ML_H;
      float a = sp[ML_OFF_B1 + j];
#pragma unroll
      for (int q = 0; q < ML_IN; ++q) a = fmaf(sp[ML_OFF_W1 + j * ML_IN + q], F[s * ML_IN + q], a);
      A1[e] = a;
      H1[e] = ml_gelu(a);
    }
    __syncthreads();
    // layer 2
    for (int e = t; e < ML_TILE * ML_H; e += 256) {
      const int s = e / ML_H, j = e % ML_H;
      float a = sp[ML_OFF_B2 + j];
      const float *w = sp + ML_OFF_W2 + j * ML_H;
      const float *h = H1 + s * ML_H;
      for (int i = 0; i < ML_H; ++i) a = fmaf(w[i], h[i], a);
      A2[e] = a;
    }
    __syncthreads();
    // output and dL/dout: 4 threads per sample, 16 terms each
    {
      const int s = t >> 2, part = t & 3;
      float o = 0.0f;
      for (int j = part * 16; j < part * 16 + 16; ++j) o = fmaf(sp[ML_OFF_W3 + j], ml_gelu(A2[s * ML_H + j]), o);
      o += __shfl_xor_sync(0xffffffffu, o, 1);
      o += __shfl_xor_sync(0xffffffffu, o, 2);
      if (part == 0) {
        float d = 0.0f;
        if (s < cnt) {
          const float r = o + sp[ML_OFF_B3] - tgt[idx[s0 + s]];
          loss = fmaf(r * r, scale, loss);
          d = 2.0f * r * scale;
        }
        dout[s] = d;
      }
    }
    __syncthreads();
    // dA2, and W3 / b3 gradients (thread j < 64 owns W3[j]; thread 64 owns b3)
    for (int e = t; e < ML_TILE * ML_H; e += 256) {
      const int s = e / ML_H, j = e % ML_H;
      D2[e] = dout[s] * sp[ML_OFF_W3 + j] * ml_gelu_grad(A2[e]);
    }
    if (t < ML_H) {
      float acc = 0.0f;
      for (int s = 0; s < ML_TILE; ++s) acc = fmaf(dout[s], ml_gelu(A2[s * ML_H + t]), acc);
      gp[ML_OFF_W3 + t] += acc;
    } else if (t == ML_H) {
      float acc = 0.0f;
      for (int s = 0; s < ML_TILE; ++s) acc += dout[s];
      gp[ML_OFF_B3] += acc;
    }
    __syncthreads();
    // W2, b2 gradients: thread t owns entries t, t + 256, ... of W2 (row j, column i)
    for (int e = t; e < ML_H * ML_H; e += 256) {
      const int j = e / ML_H, i = e % ML_H;
      float acc = 0.0f;
      for (int s = 0; s < ML_TILE; ++s) acc = fmaf(D2[s * ML_H + j], H1[s * ML_H + i], acc);
      gp[ML_OFF_W2 + e] += acc;
    }
    if (t < ML_H) {
      float acc = 0.0f;
      for (int s = 0; s < ML_TILE; ++s) acc += D2[s * ML_H + t];
      gp[ML_OFF_B2 + t] += acc;
    }
    __syncthreads();
    // dA1 = (W2^T dA2) * gelu'(A1), into H1
    for (int e = t; e < ML_TILE * ML_H; e += 256) {
      const int s = e / ML_H, i = e % ML_H;
      float acc = 0.0f;
      for (int j = 0; j < ML_H; ++j) acc = fmaf(sp[ML_OFF_W2 + j * ML_H + i], D2[s * ML_H + j], acc);
      H1[e] = acc * ml_gelu_grad(A1[e]);
    }
    __syncthreads();
    // W1, b1 gradients
    for (int e = t; e < ML_H * ML_IN; e += 256) {
      const int i = e / ML_IN, q = e % ML_IN;
      float acc = 0.0f;
      for (int s = 0; s < ML_TILE; ++s) acc = fmaf(H1[s * ML_H + i], F[s * ML_IN + q], acc);
      gp[ML_OFF_W1 + e] += acc;
    }
    if (t < ML_H) {
      float acc = 0.0f;
      for (int s = 0; s < ML_TILE; ++s) acc += H1[s * ML_H + t];
      gp[ML_OFF_B1 + t] += acc;
    }
  }
  __syncthreads();
  for (int i = t; i < ML_P; i += 256) partial[(size_t)blockIdx.x * ML_P + i] = gp[i];
  // block loss in a fixed order: samples are owned by threads t % 4 == 0
  loss = warp_sum(loss);
  if ((t & 31) == 0) red[t >> 5] = loss;
  __syncthreads();
  if (t == 0) {
    float l = 0.0f;
    for (int w = 0; w < 8; ++w) l += red[w];
    lossp[blockIdx.x] = l;
  }
}

// Sum the block partials in block order; with lr > 0 apply Adam to the FP32 master copy,
// else write the gradient to grad_out.  loss_out[0] = sum of the block losses.
__global__ void k_ml_adam(const float *__restrict__ partial, int nblocks, const float *__restrict__ lossp,
                          float *__restrict__ params, float *__restrict__ m, float *__restrict__ v, float lr, int step,
                          float *__restrict__ grad_out, float *__restrict__ loss_out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i == 0 && loss_out) {
    float l = 0.0f;
    for (int b = 0; b < nblocks; ++b) l += lossp[b];
    loss_out[0] = l;
  }
  if (i >= ML_P) return;
  float g = 0.0f;
  for (int b = 0; b < nblocks; ++b) g += partial[(size_t)b * ML_P + i];
  if (grad_out) grad_out[i] = g;
  if (lr > 0.0f) {
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    const float mi = b1 * m[i] + (1.0f - b1) * g;
    const float vi = b2 * v[i] + (1.0f - b2) * g * g;
    m[i] = mi;
    v[i] = vi;
    const float mh = mi / (1.0f - powf(b1, (float)step)), vh = vi / (1.0f - powf(b2, (float)step));
    params[i] -= lr * mh / (sqrtf(vh) + eps);
  }
}

static size_t ml_grad_smem() { return (size_t)(2 * ML_P + ML_TILE * ML_IN + 4 * ML_TILE * ML_H + ML_TILE) * 4; }

// ------------------------------------------------------------------ solver integration
void enq_learned_warm(GbWork &w, cudaStream_t s, int pf) {
  // x holds g = A^T y and red[R_XMAX] its max magnitude (solver prologue)
  const int n = argN(w);
  cudaMemsetAsync(w.ml_counts, 0, sizeof(int) * ML_RANK_BINS, s);
  k_ml_rank_hist<<<w.red_blocks, 256, 0, s>>>(w.st, pf, w.x, n, nullptr, w.bins, w.ml_counts);
  k_ml_rank_scan<<<1, 1024, 0, s>>>(w.st, pf, w.ml_counts, w.ml_cum);
  k_ml_warm<<<w.red_blocks, 256, 0, s>>>(w.st, pf, w.x, n, w.bins, w.ml_cum, w.ml_counts, w.ml_params);
}

int gb_ml_num_params() { return ML_P; }
int gb_ml_rank_bins() { return ML_RANK_BINS; }

// ------------------------------------------------------------------ C ABI
namespace {
struct DevBuf {
  std::vector<void *> p;
  ~DevBuf() {
    for (void *q : p) cudaFree(q);
  }
  template <class T>
  gb_status get(T **out, size_t count) {
    void *q = nullptr;
    GB_CUDA_TRY(cudaMalloc(&q, std::max<size_t>(count, 1) * sizeof(T)));
    p.push_back(q);
    *out = (T *)q;
    return GB_OK;
  }
};

__global__ void k_ml_absmax(const float *__restrict__ g, int n, float *out) {
  __shared__ float sm[32];
  float v = 0.0f;
  for (int i = threadIdx.x; i < n; i += blockDim.x) v = fmaxf(v, fabsf(g[i]));
  v = block_reduce<1>(v, sm);
  if (threadIdx.x == 0) *out = v;
}
}  // namespace

extern "C" int gb_cs_mlp_num_params(void) { return ML_P; }

extern "C" gb_status gb_cs_mlp_features(const float *d_g, int n, int m, int k, float *d_feat, void *stream) {
  if (!d_g || !d_feat || n < 1 || m < 1 || k < 1) {
    gb_set_error_message("gb_cs_mlp_features: bad arguments", __FILE__, __LINE__);
    return GB_BAD_ARG;
  }
  cudaStream_t s = (cudaStream_t)stream;
  DevBuf b;
  float *gmax;
  int *bins, *counts, *cum;
  GB_TRY(b.get(&gmax, 1));
  GB_TRY(b.get(&bins, n));
  GB_TRY(b.get(&counts, ML_RANK_BINS));
  GB_TRY(b.get(&cum, ML_RANK_BINS));
  GB_CUDA_TRY(cudaMemsetAsync(counts, 0, sizeof(int) * ML_RANK_BINS, s));
  k_ml_absmax<<<1, 1024, 0, s>>>(d_g, n, gmax);
  k_ml_rank_hist<<<256, 256, 0, s>>>(nullptr, 0, d_g, n, gmax, bins, counts);
  k_ml_rank_scan<<<1, 1024, 0, s>>>(nullptr, 0, counts, cum);
  k_ml_features<<<256, 256, 0, s>>>(d_g, n, gmax, bins, cum, counts, (float)m / (float)n, (float)k / (float)m,
                                    d_feat);
  GB_CUDA_TRY(cudaGetLastError());
  GB_CUDA_TRY(cudaStreamSynchronize(s));
  return GB_OK;
}

extern "C" gb_status gb_cs_mlp_forward(const float *d_params, const float *d_feat, int ns, float *d_out,
                                       void *stream) {
  if (!d_params || !d_feat || !d_out || ns < 1) {
    gb_set_error_message("gb_cs_mlp_forward: bad arguments", __FILE__, __LINE__);
    return GB_BAD_ARG;
  }
  k_ml_forward<<<std::min(1024, (ns + 255) / 256), 256, 0, (cudaStream_t)stream>>>(d_params, d_feat, ns, d_out);
  GB_CUDA_TRY(cudaGetLastError());
  return GB_OK;
}

static gb_status ml_grad_launch(const float *params, const float *feat, const float *tgt, const int *idx, int ns,
                                float scale, float *partial, float *lossp, cudaStream_t s) {
  static std::atomic<unsigned long long> attr_done{0};
  GB_TRY(gb_once_per_device(attr_done, []() -> gb_status {
    GB_CUDA_TRY(cudaFuncSetAttribute(k_ml_grad, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ml_grad_smem()));
    return GB_OK;
  }));
  k_ml_grad<<<ML_TRAIN_BLOCKS, 256, ml_grad_smem(), s>>>(params, feat, tgt, idx, ns, scale, partial, lossp);
  GB_CUDA_TRY(cudaGetLastError());
  return GB_OK;
}

extern "C" gb_status gb_cs_mlp_grad(const float *d_params, const float *d_feat, const float *d_tgt, int ns,
                                    float *d_grad, float *d_loss, void *stream) {
  if (!d_params || !d_feat || !d_tgt || !d_grad || ns < 1) {
    gb_set_error_message("gb_cs_mlp_grad: bad arguments", __FILE__, __LINE__);
    return GB_BAD_ARG;
  }
  cudaStream_t s = (cudaStream_t)stream;
  DevBuf b;
  int *idx;
  float *partial, *lossp;
  GB_TRY(b.get(&idx, ns));
  GB_TRY(b.get(&partial, (size_t)ML_TRAIN_BLOCKS * ML_P));
  GB_TRY(b.get(&lossp, ML_TRAIN_BLOCKS));
  std::vector<int> h(ns);
  for (int i = 0; i < ns; ++i) h[i] = i;
  GB_CUDA_TRY(cudaMemcpyAsync(idx, h.data(), sizeof(int) * ns, cudaMemcpyHostToDevice, s));
  GB_TRY(ml_grad_launch(d_params, d_feat, d_tgt, idx, ns, 1.0f / (float)ns, partial, lossp, s));
  k_ml_adam<<<(ML_P + 255) / 256, 256, 0, s>>>(partial, ML_TRAIN_BLOCKS, lossp, nullptr, nullptr, nullptr, 0.0f, 0,
                                               d_grad, d_loss);
  GB_CUDA_TRY(cudaGetLastError());
  GB_CUDA_TRY(cudaStreamSynchronize(s));
  return GB_OK;
}

extern "C" gb_status gb_cs_mlp_train(float *d_params, const float *d_feat, const float *d_tgt, int ns, int batch,
                                     int epochs, float lr, unsigned int seed, float *h_epoch_loss, void *stream) {
  if (!d_params || !d_feat || !d_tgt || ns < 1 || batch < 1 || epochs < 1 || !(lr > 0.0f)) {
    gb_set_error_message("gb_cs_mlp_train: bad arguments", __FILE__, __LINE__);
    return GB_BAD_ARG;
  }
  cudaStream_t s = (cudaStream_t)stream;
  DevBuf b;
  int *idx;
  float *partial, *lossp, *m, *v, *loss;
  GB_TRY(b.get(&idx, ns));
  GB_TRY(b.get(&partial, (size_t)ML_TRAIN_BLOCKS * ML_P));
  GB_TRY(b.get(&lossp, ML_TRAIN_BLOCKS));
  GB_TRY(b.get(&m, ML_P));
  GB_TRY(b.get(&v, ML_P));
  const int steps_per_epoch = (ns + batch - 1) / batch;
  GB_TRY(b.get(&loss, (size_t)steps_per_epoch * epochs));
  GB_CUDA_TRY(cudaMemsetAsync(m, 0, sizeof(float) * ML_P, s));
  GB_CUDA_TRY(cudaMemsetAsync(v, 0, sizeof(float) * ML_P, s));
  std::vector<int> perm(ns);
  for (int i = 0; i < ns; ++i) perm[i] = i;
  std::mt19937 rng(seed);
  int step = 0;
  for (int e = 0; e < epochs; ++e) {
    std::shuffle(perm.begin(), perm.end(), rng);
    GB_CUDA_TRY(cudaMemcpyAsync(idx, perm.data(), sizeof(int) * ns, cudaMemcpyHostToDevice, s));
    GB_CUDA_TRY(cudaStreamSynchronize(s));  // perm is rewritten next epoch
    for (int b0 = 0; b0 < ns; b0 += batch) {
      const int nb = std::min(batch, ns - b0);
      GB_TRY(ml_grad_launch(d_params, d_feat, d_tgt, idx + b0, nb, 1.0f / (float)nb, partial, lossp, s));
      ++step;
      k_ml_adam<<<(ML_P + 255) / 256, 256, 0, s>>>(partial, ML_TRAIN_BLOCKS, lossp, d_params, m, v, lr, step,
                                                   nullptr, loss + (step - 1));
    }
  }
  GB_CUDA_TRY(cudaGetLastError());
  std::vector<float> hl((size_t)steps_per_epoch * epochs);
  GB_CUDA_TRY(cudaMemcpyAsync(hl.data(), loss, sizeof(float) * hl.size(), cudaMemcpyDeviceToHost, s));
  GB_CUDA_TRY(cudaStreamSynchronize(s));
  if (h_epoch_loss)
    for (int e = 0; e < epochs; ++e) {
      double a = 0.0;
      for (int q = 0; q < steps_per_epoch; ++q) a += hl[(size_t)e * steps_per_epoch + q];
      h_epoch_loss[e] = (float)(a / steps_per_epoch);
    }
  return GB_OK;
}
