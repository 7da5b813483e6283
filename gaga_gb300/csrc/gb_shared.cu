// gb_shared.cu -- batched form for trials that share one dense A (BF16 tensor-core GEMMs).
//
// T trials y_t = A x0_t with the same Gaussian A run NIHT in lockstep.  The operator
// applications of all trials become three GEMMs per iteration (gb_gemm.cu):
//
//   R  = Y - [A_hi | A_lo | A_hi] . [X_hi ; X_hi ; X_lo]   residual, ~FP32 accurate:
//        A and X are split into BF16 high and low parts, the A_lo X_lo term is dropped
//   G  = A_hi^T . bf16(R)                                  gradients
//   Q  = A_hi . bf16(x_thres)                              step-size products
//
// with FP32 accumulation.  Everything else of an iteration -- the reference's scalar
// logic (gb_ctrl.cuh), the restriction to the support, the update, LinearBinning and the
// k-th bin -- runs in one CTA per trial.  The loop is a CUDA graph WHILE node that runs
// while any trial is active.  Trials that stop with ||y - A x|| <= tol are then debiased:
// least squares on their final support by conjugate gradients on the normal equations,
// again as split-precision GEMMs over all trials, with the CG scalars in FP64 (FP64
// arithmetic is a small fraction of the FP32 rate on this part, so no product runs in
// it).  The verdict is the relative l2 error against the planted x0.
//
// CGIHT (restartFlag off, GAGA/gaga/algorithms.cu:3689-3942) runs in lockstep the same
// way, with four products per pass: the residual R and G = A^T R for every active trial,
// then Q = A p for the direction on the support (the restricted-CG branch's new direction,
// the unrestricted branch's previous one) and, for the trials in the unrestricted branch
// only, Q2 = A g_S (functions.cu:1004-1220); Q and Q2 are one GEMM over both trial lists.  With the learned warm start the prologue
// starts each trial from H_k(w . A^T y) (w from the per-coordinate network, gb_mlp.cuh);
// a trial that gives it up after 10 iterations is restarted inside the loop from the plain
// start H_k(A^T y), its iterations added.
//
// The shared A is drawn from `seed` exactly as gb_cs_generate_and_solve draws it; trial
// t's x0 uses the key seed + 1 + first_trial + t.
#include <cuda_bf16.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <vector>

#include "gb_ctrl.cuh"
#include "gb_mlp.cuh"
#include "gb_philox.cuh"

#define SH_THREADS 256
#define SH_CG_MAX 20       // debias iterations
#define SH_NBINS_MAX 1640  // num_bins = max(n/20, 1000) <= 1638 for n <= 32768

namespace {

struct ShDev {
  int m, n, T, Tp, maxiter;
  int kg, kq;               // K of the A^T r and A x_thres products (m or 3m, n or 3n)
  double *flops;            // algorithmic GEMM flops of all trials
  int prec;                 // bit 0: split A^T r; bit 1: split A x_thres (else BF16 operands)
  float tol_rel;
  unsigned int seed, first;
  const int *kreq;
  float *A32;               // m x n column-major (lda = m)
  __nv_bfloat16 *Acat;      // m x 3n row-major: [A_hi | A_lo | A_hi]
  __nv_bfloat16 *ATcat;     // n x 3m row-major: [A_hi^T | A_lo^T | A_hi^T]
  float *X0, *X, *G, *Y, *R, *Q;
  __nv_bfloat16 *Xcat, *XTbf, *Rbf;  // Tp x 3n, Tp x 3n (x_thres, split or not), Tp x m
  int *bins;
  GbState *st;
  float *P;                 // debias search directions, Tp x n
  __nv_bfloat16 *Rcat;      // debias residual split, Tp x 3m
  int *act, *act_cnt;       // trials still iterating (ascending) and their count
  int alg;                  // GB_ALG_NIHT or GB_ALG_CGIHT
  const float *ml;          // CGIHT: learned warm start's network parameters (null: plain start)
  float *GP, *GPT;          // CGIHT: grad_previous and grad_prev_thres (Tp x n)
  float *G0;                // CGIHT with the learned start: A^T y, the plain restart's start
  float *Q2;                // CGIHT: A g_S of the unrestricted-branch trials (Tp x m, = Q + Tp m)
  __nv_bfloat16 *XT2;       // its BF16 operand (Tp x kq, = XTbf + Tp kq)
  int *bins_prev;           // CGIHT: bins before this pass's binning (support evolution)
  GbState *st0;             // CGIHT with the learned start: each trial's plain initial state
  int *act_q, *act_q_cnt;   // CGIHT: trials whose pass runs the direction product
  int *act_u, *act_u_cnt;   // CGIHT: the unrestricted-branch trials among them
  int *act_qu, *act_qu_cnt; // CGIHT: act_q, then act_u + Tp (rows of Q2 / XT2 past Q / XTbf):
                            // Q = A p and Q2 = A g_S as one GEMM
  int *fallbacks;           // CGIHT: trials restarted from the plain start
  int *iters;
  float *err;
  int *ok;
};

// ------------------------------------------------------------------ operands
__global__ void k_sh_genA(float *A32, int m, int n, uint32_t seed) {
  const int lane = threadIdx.x & 31;
  const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, nw = (gridDim.x * blockDim.x) >> 5;
  for (int j = gw; j < n; j += nw) gbgen::gen_dense_column(A32 + (size_t)j * m, j, m, seed, 0u, 1, lane, 32);
}

// BF16 operands: rows [hi | lo | hi] of A (Acat, through a 32x32 shared-memory transpose)
// and of A^T (ATcat, straight from the column-major A)
__global__ void k_sh_split(const float *__restrict__ A32, __nv_bfloat16 *__restrict__ Acat,
                           __nv_bfloat16 *__restrict__ ATcat, int m, int n) {
  __shared__ float tile[32][33];
  const int i0 = blockIdx.x * 32, j0 = blockIdx.y * 32;
  for (int r = threadIdx.y; r < 32; r += 8) {
    const int j = j0 + r, i = i0 + threadIdx.x;
    const float v = A32[(size_t)j * m + i];
    tile[r][threadIdx.x] = v;
    const __nv_bfloat16 hi = __float2bfloat16_rn(v);
    const size_t row = (size_t)j * 3 * m;
    ATcat[row + i] = hi;
    ATcat[row + m + i] = __float2bfloat16_rn(v - __bfloat162float(hi));
    ATcat[row + 2 * m + i] = hi;
  }
  __syncthreads();
  for (int r = threadIdx.y; r < 32; r += 8) {
    const int i = i0 + r, j = j0 + threadIdx.x;
    const float v = tile[threadIdx.x][r];
    const __nv_bfloat16 hi = __float2bfloat16_rn(v);
    const __nv_bfloat16 lo = __float2bfloat16_rn(v - __bfloat162float(hi));
    const size_t row = (size_t)i * 3 * n;
    Acat[row + j] = hi;
    Acat[row + n + j] = lo;
    Acat[row + 2 * n + j] = hi;
  }
}

// ------------------------------------------------------------------ CTA helpers
__device__ float cta_sum(float v, float *sm) {
  v = warp_sum(v);
  __syncthreads();
  if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = v;
  __syncthreads();
  float t = 0.0f;
  for (int w = 0; w < SH_THREADS / 32; ++w) t += sm[w];
  return t;
}
__device__ float cta_max(float v, float *sm) {
  v = warp_max(v);
  __syncthreads();
  if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = v;
  __syncthreads();
  float t = 0.0f;
  for (int w = 0; w < SH_THREADS / 32; ++w) t = fmaxf(t, sm[w]);
  return t;
}
__device__ double cta_sumd(double v, double *sm) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  __syncthreads();
  if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = v;
  __syncthreads();
  double t = 0.0;
  for (int w = 0; w < SH_THREADS / 32; ++w) t += sm[w];
  return t;
}

// first bin whose cumulative count reaches k (the host scan of FindSupportSet,
// GAGA/gaga/functions.cu:414-420); results for every thread
__device__ void cta_kbin(const int *hist, int max_bin, int k, int *k_bin, int *sum, int *scan) {
  __shared__ int res[2];
  const int t = threadIdx.x;
  const int per = (max_bin + SH_THREADS - 1) / SH_THREADS;
  const int b0 = t * per, b1 = min(b0 + per, max_bin);
  int c = 0;
  for (int b = b0; b < b1; ++b) c += hist[b];
  scan[t] = c;
  if (t == 0) { res[0] = -2; res[1] = 0; }
  __syncthreads();
  for (int off = 1; off < SH_THREADS; off <<= 1) {
    const int v = t >= off ? scan[t - off] : 0;
    __syncthreads();
    scan[t] += v;
    __syncthreads();
  }
  const int incl = scan[t], excl = incl - c;
  if (k > 0 && excl < k && incl >= k) {
    int a = excl;
    for (int b = b0; b < b1; ++b) {
      a += hist[b];
      if (a >= k) { res[0] = b; res[1] = a; break; }
    }
  }
  __syncthreads();
  if (k <= 0) { *k_bin = -1; *sum = 0; }
  else if (res[0] == -2) { *k_bin = max_bin - 1; *sum = scan[SH_THREADS - 1]; }
  else { *k_bin = res[0]; *sum = res[1]; }
  __syncthreads();
}

// FindSupportSet on x (GAGA/gaga/functions.cu:397-436) when binning this iteration, then
// Threshold (functions.cu:374-378); refreshes the BF16 high/low parts of x
__device__ void cta_support(GbState *st, float *x, int *bins, int n, __nv_bfloat16 *xcat, int *hist, int *scan) {
  if (st->flags[F_DOBIN]) {
    const int max_bin = st->max_bin;
    for (int b = threadIdx.x; b < max_bin; b += SH_THREADS) hist[b] = 0;
    __syncthreads();
    const float intercept = st->max_value, slope = st->slope;
    const float small_f = __double2float_rd((double)intercept * 0.000001);
    for (int j = threadIdx.x; j < n; j += SH_THREADS) {
      bool counted;
      const int b = lin_bin(x[j], slope, intercept, small_f, counted);
      bins[j] = b;
      if (counted && b < max_bin) atomicAdd(&hist[b], 1);
    }
    __syncthreads();
    int k_bin, sum;
    cta_kbin(hist, max_bin, st->k, &k_bin, &sum, scan);
    if (threadIdx.x == 0) {
      if (sum < st->k) {
        st->alpha_bin = st->alpha_bin * 0.5f;
        st->max_bin = (int)((float)st->num_bins * (1.0f - st->alpha_bin));
      }
      st->min_val = intercept - (float)(k_bin + 1) / slope;
      st->k_bin = k_bin;
      st->sum = sum;
    }
    __syncthreads();
  }
  const int kb = st->k_bin;
  for (int j = threadIdx.x; j < n; j += SH_THREADS) {
    float v = x[j];
    if (bins[j] > kb) {
      v = 0.0f;
      x[j] = 0.0f;
    }
    const __nv_bfloat16 hi = __float2bfloat16_rn(v);
    const __nv_bfloat16 lo = __float2bfloat16_rn(v - __bfloat162float(hi));
    xcat[j] = hi;
    xcat[n + j] = hi;
    xcat[2 * n + j] = lo;
  }
  __syncthreads();
}

// ------------------------------------------------------------------ problem per trial
// x0 with createVector's binned support (GAGA/gaga/createVector.cu:207-300), key seed+1+t
__global__ void __launch_bounds__(SH_THREADS) k_sh_genx(ShDev d) {
  extern __shared__ int shist[];  // n counters
  __shared__ float sm[32];
  __shared__ int scan[SH_THREADS];
  const int t = blockIdx.x, n = d.n;
  float *x0 = d.X0 + (size_t)t * n;
  int *bins = d.bins + (size_t)t * n;
  if (t >= d.T) {
    for (int j = threadIdx.x; j < n; j += SH_THREADS) x0[j] = 0.0f;
    return;
  }
  const uint32_t key = d.seed + 1u + d.first + (uint32_t)t;
  float mx = 0.0f;
  for (int j = threadIdx.x; j < n; j += SH_THREADS) {
    const float u = gbgen::uniform_at(key, 0u, gbgen::ST_VALUES, (uint64_t)j);
    x0[j] = signbit(u - 0.5f) ? -1.0f : 1.0f;
    mx = fmaxf(mx, gbgen::uniform_at(key, 0u, gbgen::ST_SUPPORT, (uint64_t)j));
    shist[j] = 0;
  }
  const float keymax = cta_max(mx, sm);
  const float slope = ((float)(n - 1) / keymax);
  const float small_f = __double2float_rd((double)keymax * 0.000001);
  for (int j = threadIdx.x; j < n; j += SH_THREADS) {
    bool counted;
    int b = lin_bin(gbgen::uniform_at(key, 0u, gbgen::ST_SUPPORT, (uint64_t)j), slope, keymax, small_f, counted);
    if (!counted) b = n;  // keys below the cutoff never enter the support
    bins[j] = b;
    if (counted && b < n) atomicAdd(&shist[b], 1);
  }
  __syncthreads();
  int k_bin, sum;
  cta_kbin(shist, n, d.kreq[t], &k_bin, &sum, scan);
  for (int j = threadIdx.x; j < n; j += SH_THREADS)
    if (bins[j] > k_bin) x0[j] = 0.0f;
  if (threadIdx.x == 0) d.st[t].k = sum;
}

// y_t = A x0_t in FP32, summed over the support in ascending column order; ||y||; initial
// solver state (initial_state in gb_solver.cu) with tol = tol_rel ||y||
__global__ void __launch_bounds__(SH_THREADS) k_sh_y(ShDev d) {
  extern __shared__ int ssup[];  // support list (n) then values
  __shared__ double smd[32];
  __shared__ int cnt_s;
  const int t = blockIdx.x, n = d.n, m = d.m;
  const float *x0 = d.X0 + (size_t)t * n;
  float *y = d.Y + (size_t)t * m;
  __nv_bfloat16 *ybf = d.Rbf + (size_t)t * m;
  GbState *st = d.st + t;
  if (t >= d.T) {
    for (int i = threadIdx.x; i < m; i += SH_THREADS) {
      y[i] = 0.0f;
      ybf[i] = __float2bfloat16_rn(0.0f);
      for (int c = 0; c < 3; ++c) d.Rcat[(size_t)t * 3 * m + c * m + i] = __float2bfloat16_rn(0.0f);
    }
    if (threadIdx.x == 0) { memset(st, 0, sizeof(GbState)); st->active = 0; }
    return;
  }
  if (threadIdx.x == 0) cnt_s = 0;
  __syncthreads();
  // ordered support list: one warp-ballot pass per 256 columns
  __shared__ int wcnt[SH_THREADS / 32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int j0 = 0; j0 < n; j0 += SH_THREADS) {
    const int j = j0 + threadIdx.x;
    const bool in = j < n && x0[j] != 0.0f;
    const unsigned bal = __ballot_sync(0xffffffffu, in);
    if (lane == 0) wcnt[w] = __popc(bal);
    __syncthreads();
    int wb = 0, tot = 0;
    for (int q = 0; q < SH_THREADS / 32; ++q) {
      if (q < w) wb += wcnt[q];
      tot += wcnt[q];
    }
    if (in) ssup[cnt_s + wb + __popc(bal & ((1u << lane) - 1u))] = j;
    __syncthreads();
    if (threadIdx.x == 0) cnt_s += tot;
    __syncthreads();
  }
  const int s = cnt_s;
  double y2 = 0.0;
  for (int i = threadIdx.x; i < m; i += SH_THREADS) {
    float acc = 0.0f;
    for (int c = 0; c < s; ++c) {
      const int j = ssup[c];
      acc = acc + d.A32[(size_t)j * m + i] * x0[j];
    }
    y[i] = acc;
    const __nv_bfloat16 hi = __float2bfloat16_rn(acc);
    ybf[i] = hi;
    __nv_bfloat16 *yc = d.Rcat + (size_t)t * 3 * m;
    yc[i] = hi;
    yc[m + i] = hi;
    yc[2 * m + i] = __float2bfloat16_rn(acc - __bfloat162float(hi));
    y2 += (double)acc * (double)acc;
  }
  const double ys = cta_sumd(y2, smd);
  if (threadIdx.x == 0) {
    const int ks = st->k;
    memset(st, 0, sizeof(GbState));
    st->m = m; st->n = n; st->k = ks; st->lda = m;
    st->num_bins = max(n / 20, 1000);
    st->maxiter = d.maxiter;
    st->alg = d.alg;
    st->learned = d.ml ? 1 : 0;
    st->tol = d.tol_rel * (float)sqrt(ys);
    st->active = 1; st->cycle = 1; st->pass_limit = d.maxiter + 4;
    st->resid_diff = 1.0f;
    for (int j = 0; j < 16; ++j) { st->prev[j] = 0.0f; st->evol[j] = 1.0f; }
    st->alpha_bin = 0.25f;
    st->max_bin = (int)((float)st->num_bins * (1.0f - st->alpha_bin));
    st->beta_to_zero = 1; st->supp_change = 1;
    st->flags[F_ALWAYS] = 1;
    st->op_kind = GB_OP_DENSE;
    st->trial = t;
    st->red[R_RES] = ys;
  }
}

// ------------------------------------------------------------------ NIHT in lockstep
// x = H_k(A^T y) (algorithms.cu:1335-1354) from G = A_hi^T bf16(y)
__global__ void __launch_bounds__(SH_THREADS) k_sh_init(ShDev d) {
  __shared__ float sm[32];
  __shared__ int hist[SH_NBINS_MAX];
  __shared__ int scan[SH_THREADS];
  const int t = blockIdx.x, n = d.n;
  GbState *st = d.st + t;
  if (t >= d.T) return;
  float *x = d.X + (size_t)t * n;
  const float *g = d.G + (size_t)t * n;
  if (threadIdx.x == 0) ctrl_phase(st, C_INIT0, 0);
  float mx = 0.0f;
  for (int j = threadIdx.x; j < n; j += SH_THREADS) {
    const float v = g[j];
    x[j] = v;
    mx = fmaxf(mx, fabsf(v));
  }
  mx = cta_max(mx, sm);
  if (threadIdx.x == 0) {
    st->red[R_XMAX] = mx;
    ctrl_phase(st, C_INIT_BINPREP, 0);
  }
  __syncthreads();
  cta_support(st, x, d.bins + (size_t)t * n, n, d.Xcat + (size_t)t * 3 * n, hist, scan);
  if (threadIdx.x == 0) ctrl_phase(st, C_INIT_DONE, 0);
}

// ||r||^2, then x_thres = g restricted to the support, ||x_thres||^2, max|g|
__global__ void __launch_bounds__(SH_THREADS) k_sh_mask(ShDev d) {
  __shared__ float sm[32];
  const int t = blockIdx.x, n = d.n, m = d.m;
  GbState *st = d.st + t;
  if (t >= d.T || !st->active) return;
  const float *r = d.R + (size_t)t * m;
  float r2 = 0.0f;
  for (int i = threadIdx.x; i < m; i += SH_THREADS) r2 = fmaf(r[i], r[i], r2);
  r2 = cta_sum(r2, sm);
  if (threadIdx.x == 0) {
    st->red[R_RES] = r2;
    ctrl_phase(st, C_PUSH_RES, 0);
  }
  const float *g = d.G + (size_t)t * n;
  const int *bins = d.bins + (size_t)t * n;
  const int kb = st->k_bin;
  float s2 = 0.0f, gm = 0.0f;
  for (int j = threadIdx.x; j < n; j += SH_THREADS) {
    const float v = g[j];
    const float o = bins[j] <= kb ? v : 0.0f;
    const __nv_bfloat16 hi = __float2bfloat16_rn(o);
    if (d.prec & 2) {
      __nv_bfloat16 *xt = d.XTbf + (size_t)t * 3 * n;
      xt[j] = hi;
      xt[n + j] = hi;
      xt[2 * n + j] = __float2bfloat16_rn(o - __bfloat162float(hi));
    } else {
      d.XTbf[(size_t)t * n + j] = hi;
    }
    s2 = fmaf(o, o, s2);
    gm = fmaxf(gm, fabsf(v));
  }
  s2 = cta_sum(s2, sm);
  gm = cta_max(gm, sm);
  if (threadIdx.x == 0) {
    st->red[R_XT] = s2;
    st->red[R_GMAX] = gm;
  }
}

// step size (RestrictedSD), x += mu g, FindSupportSet + Threshold, stopping rules
__global__ void __launch_bounds__(SH_THREADS) k_sh_step(ShDev d) {
  __shared__ float sm[32];
  __shared__ int hist[SH_NBINS_MAX];
  __shared__ int scan[SH_THREADS];
  const int t = blockIdx.x, n = d.n, m = d.m;
  GbState *st = d.st + t;
  if (t >= d.T || !st->active) return;
  const float *q = d.Q + (size_t)t * m;
  float q2 = 0.0f;
  for (int i = threadIdx.x; i < m; i += SH_THREADS) q2 = fmaf(q[i], q[i], q2);
  q2 = cta_sum(q2, sm);
  if (threadIdx.x == 0) {
    st->red[R_AXT] = q2;
    ctrl_phase(st, C_SD_MU, 0);
  }
  __syncthreads();
  const float mu = st->mu;
  float *x = d.X + (size_t)t * n;
  const float *g = d.G + (size_t)t * n;
  float mx = 0.0f;
  for (int j = threadIdx.x; j < n; j += SH_THREADS) {
    const float o = fmaf(mu, g[j], x[j]);
    x[j] = o;
    mx = fmaxf(mx, fabsf(o));
  }
  mx = cta_max(mx, sm);
  if (threadIdx.x == 0) {
    st->red[R_XMAX] = mx;
    ctrl_phase(st, C_BINPREP, 0);
  }
  __syncthreads();
  cta_support(st, x, d.bins + (size_t)t * n, n, d.Xcat + (size_t)t * 3 * n, hist, scan);
  if (threadIdx.x == 0) {
    ctrl_phase(st, C_NIHT_STOP, 0);
  }
}

// ------------------------------------------------------------------ CGIHT in lockstep
__device__ __forceinline__ void put_bf(__nv_bfloat16 *row, int n, int j, float v, bool split) {
  const __nv_bfloat16 hi = __float2bfloat16_rn(v);
  if (split) {
    row[j] = hi;
    row[n + j] = hi;
    row[2 * n + j] = __float2bfloat16_rn(v - __bfloat162float(hi));
  } else {
    row[j] = hi;
  }
}

// cta_support with CGIHT's support evolution: the bins before a new binning go to
// bins_prev, and st->changed is set when an entry of the previous support (bin <=
// k_bin_prev) left it (checkSupportEvolution, GAGA/gaga/kernels.cu:178-193)
__device__ void cta_support_evol(GbState *st, float *x, int *bins, int *bins_prev, int n, __nv_bfloat16 *xcat,
                                 int *hist, int *scan) {
  const bool dobin = st->flags[F_DOBIN] != 0;
  if (dobin) {
    const int max_bin = st->max_bin;
    for (int b = threadIdx.x; b < max_bin; b += SH_THREADS) hist[b] = 0;
    __syncthreads();
    const float intercept = st->max_value, slope = st->slope;
    const float small_f = __double2float_rd((double)intercept * 0.000001);
    for (int j = threadIdx.x; j < n; j += SH_THREADS) {
      bool counted;
      const int b = lin_bin(x[j], slope, intercept, small_f, counted);
      bins_prev[j] = bins[j];
      bins[j] = b;
      if (counted && b < max_bin) atomicAdd(&hist[b], 1);
    }
    __syncthreads();
    int k_bin, sum;
    cta_kbin(hist, max_bin, st->k, &k_bin, &sum, scan);
    if (threadIdx.x == 0) {
      if (sum < st->k) {
        st->alpha_bin = st->alpha_bin * 0.5f;
        st->max_bin = (int)((float)st->num_bins * (1.0f - st->alpha_bin));
      }
      st->min_val = intercept - (float)(k_bin + 1) / slope;
      st->k_bin = k_bin;
      st->sum = sum;
    }
    __syncthreads();
  }
  const int kb = st->k_bin, kbp = st->k_bin_prev;
  int changed = 0;
  for (int j = threadIdx.x; j < n; j += SH_THREADS) {
    float v = x[j];
    const int b = bins[j];
    if (b > kb) {
      v = 0.0f;
      x[j] = 0.0f;
    }
    if (dobin && bins_prev[j] <= kbp && b > kb) changed = 1;
    const __nv_bfloat16 hi = __float2bfloat16_rn(v);
    xcat[j] = hi;
    xcat[n + j] = hi;
    xcat[2 * n + j] = __float2bfloat16_rn(v - __bfloat162float(hi));
  }
  changed = __syncthreads_or(changed);
  if (threadIdx.x == 0 && changed) st->changed = 1;
  __syncthreads();
}

// the start x = H_k(v) of a trial (FindSupportSet + Threshold, algorithms.cu:3776-3790)
// from v already in x; every thread calls it
__device__ void cta_start_support(ShDev &d, int t, GbState *st, float *x, int *hist, int *scan, float *sm) {
  const int n = d.n;
  float mx = 0.0f;
  for (int j = threadIdx.x; j < n; j += SH_THREADS) mx = fmaxf(mx, fabsf(x[j]));
  mx = cta_max(mx, sm);
  if (threadIdx.x == 0) {
    st->red[R_XMAX] = mx;
    ctrl_phase(st, C_INIT_BINPREP, 0);
  }
  __syncthreads();
  cta_support(st, x, d.bins + (size_t)t * n, n, d.Xcat + (size_t)t * 3 * n, hist, scan);
}

// CGIHT prologue, first part: x = A^T y (G), with the learned start x = g . net(features
// of g) (the single-trial k_ml_rank_hist / k_ml_warm in one CTA), then H_k(x).  The
// plain initial state is kept for a fallback.  Dynamic shared memory: the network's
// parameters, then the rank histogram and its prefix (reused for the bin counts).
__global__ void __launch_bounds__(SH_THREADS) k_sc_init(ShDev d) {
  extern __shared__ float dyn[];
  __shared__ float sm[32];
  __shared__ int scan[SH_THREADS];
  const int t = blockIdx.x, n = d.n;
  if (t >= d.T) return;
  GbState *st = d.st + t;
  float *x = d.X + (size_t)t * n;
  const float *g = d.G + (size_t)t * n;
  int *counts = (int *)(dyn + (d.ml ? ML_P : 0));
  int *cum = counts + ML_RANK_BINS;
  if (threadIdx.x == 0) {
    ctrl_phase(st, C_INIT0, 0);
    if (d.ml) {
      d.st0[t] = *st;
      d.st0[t].learned = 0;
    }
  }
  float mx = 0.0f;
  for (int j = threadIdx.x; j < n; j += SH_THREADS) {
    const float v = g[j];
    x[j] = v;
    if (d.ml) d.G0[(size_t)t * n + j] = v;
    mx = fmaxf(mx, fabsf(v));
  }
  mx = cta_max(mx, sm);
  if (d.ml) {
    // rank histogram of |g| below max|g| (bin 0: the largest), its exclusive prefix
    int *rb = d.bins + (size_t)t * n;
    for (int b = threadIdx.x; b < ML_RANK_BINS; b += SH_THREADS) counts[b] = 0;
    __syncthreads();
    const float slope = mx > 0.0f ? (float)(ML_RANK_BINS - 1) / mx : 0.0f;
    for (int j = threadIdx.x; j < n; j += SH_THREADS) {
      int b = (int)((mx - fabsf(g[j])) * slope);
      b = min(max(b, 0), ML_RANK_BINS - 1);
      rb[j] = b;
      atomicAdd(&counts[b], 1);
    }
    __syncthreads();
    constexpr int PER = ML_RANK_BINS / SH_THREADS;
    int c[PER], tot = 0;
#pragma unroll
    for (int q = 0; q < PER; ++q) {
      c[q] = counts[threadIdx.x * PER + q];
      tot += c[q];
    }
    scan[threadIdx.x] = tot;
    __syncthreads();
    for (int off = 1; off < SH_THREADS; off <<= 1) {
      const int v = threadIdx.x >= off ? scan[threadIdx.x - off] : 0;
      __syncthreads();
      scan[threadIdx.x] += v;
      __syncthreads();
    }
    int run = scan[threadIdx.x] - tot;
#pragma unroll
    for (int q = 0; q < PER; ++q) {
      cum[threadIdx.x * PER + q] = run;
      run += c[q];
    }
    ml_load_params(d.ml, dyn);
    const float delta = (float)d.m / (float)n, rho = (float)st->k / (float)d.m;
    for (int j = threadIdx.x; j < n; j += SH_THREADS) {
      const float gi = g[j];
      float f[ML_IN];
      ml_features(gi, mx, rb[j], cum, counts, n, delta, rho, f);
      x[j] = gi * ml_forward1(dyn, f);
    }
    __syncthreads();
  }
  cta_start_support(d, t, st, x, counts, scan, sm);
}

// grad_previous = A^T r0, grad_prev_thres, and CGIHT's loop start (algorithms.cu:3791-3808)
__device__ void cta_cgiht_prologue(ShDev &d, int t, GbState *st, float r2) {
  const int n = d.n;
  const float *g = d.G + (size_t)t * n;
  float *gp = d.GP + (size_t)t * n, *gpt = d.GPT + (size_t)t * n;
  const int *bins = d.bins + (size_t)t * n;
  const int kb = st->k_bin;
  for (int j = threadIdx.x; j < n; j += SH_THREADS) {
    const float v = g[j];
    gp[j] = v;
    gpt[j] = bins[j] <= kb ? v : 0.0f;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    st->red[R_RES] = r2;
    ctrl_phase(st, C_CGIHT_INIT, 0);
  }
  __syncthreads();
}

// CGIHT prologue, second part: after R = Y - A x and G = A^T R of every trial
__global__ void __launch_bounds__(SH_THREADS) k_sc_init2(ShDev d) {
  __shared__ float sm[32];
  const int t = blockIdx.x, m = d.m;
  if (t >= d.T) return;
  GbState *st = d.st + t;
  const float *r = d.R + (size_t)t * m;
  float r2 = 0.0f;
  for (int i = threadIdx.x; i < m; i += SH_THREADS) r2 = fmaf(r[i], r[i], r2);
  r2 = cta_sum(r2, sm);
  cta_cgiht_prologue(d, t, st, r2);
}

// CGIHT pass, first part (after R and G): ||r||^2 into the history; the restricted branch's
// beta and new direction p (functions.cu:1020-1074), or the unrestricted branch's operands
// p_prev_S and g_S (functions.cu:1134-1147); the direction product(s) follow
__global__ void __launch_bounds__(SH_THREADS) k_sc_dir(ShDev d) {
  __shared__ float sm[32];
  const int t = blockIdx.x, n = d.n, m = d.m;
  if (t >= d.T) return;
  GbState *st = d.st + t;
  if (!st->active) return;
  const float *r = d.R + (size_t)t * m;
  float r2 = 0.0f;
  for (int i = threadIdx.x; i < m; i += SH_THREADS) r2 = fmaf(r[i], r[i], r2);
  r2 = cta_sum(r2, sm);
  if (st->fell_back == 1) {
    // plain restart after an abandoned warm start: this pass is its prologue
    cta_cgiht_prologue(d, t, st, r2);
    if (threadIdx.x == 0) {
      st->fell_back = 2;
      st->sh_prologue = 1;
    }
    return;
  }
  if (threadIdx.x == 0) {
    st->red[R_RES] = r2;
    ctrl_phase(st, C_PUSH_RES, 0);
  }
  const float *g = d.G + (size_t)t * n;
  const int *bins = d.bins + (size_t)t * n;
  const int kb = st->k_bin;
  const bool split = (d.prec & 2) != 0;
  const size_t row = (size_t)t * (split ? 3 * n : n);
  float s2 = 0.0f;
  for (int j = threadIdx.x; j < n; j += SH_THREADS) {
    const float o = bins[j] <= kb ? g[j] : 0.0f;
    s2 = fmaf(o, o, s2);
  }
  s2 = cta_sum(s2, sm);
  if (threadIdx.x == 0) {
    st->red[R_XT] = s2;
    ctrl_phase(st, C_RCG_BETA, 0);
  }
  __syncthreads();
  float *gp = d.GP + (size_t)t * n, *gpt = d.GPT + (size_t)t * n;
  if (st->flags[F_RCG]) {
    const float beta = st->cg_beta;
    float gm = 0.0f;
    for (int j = threadIdx.x; j < n; j += SH_THREADS) {
      const float v = fmaf(1.0f, g[j], beta * gp[j]);
      gp[j] = v;
      const float pt = bins[j] <= kb ? v : 0.0f;
      gpt[j] = pt;
      put_bf(d.XTbf + row, n, j, pt, split);
      gm = fmaxf(gm, fabsf(v));
    }
    gm = cta_max(gm, sm);
    if (threadIdx.x == 0) st->red[R_GMAX] = gm;
  } else {
    for (int j = threadIdx.x; j < n; j += SH_THREADS) {
      put_bf(d.XTbf + row, n, j, gpt[j], split);
      put_bf(d.XT2 + row, n, j, bins[j] <= kb ? g[j] : 0.0f, split);
    }
  }
}

// CGIHT pass, second part (after Q = A p, and Q2 = A g_S for the unrestricted branch):
// alpha (and the unrestricted branch's beta, direction and A p), x += alpha p, the
// support and its evolution, the stopping rules; a learned start given up after 10
// iterations restarts from the plain start H_k(A^T y)
__global__ void __launch_bounds__(SH_THREADS) k_sc_step(ShDev d) {
  __shared__ float sm[32];
  __shared__ int hist[SH_NBINS_MAX];
  __shared__ int scan[SH_THREADS];
  const int t = blockIdx.x, n = d.n, m = d.m;
  if (t >= d.T) return;
  GbState *st = d.st + t;
  if (!st->active) return;
  if (st->sh_prologue) {
    __syncthreads();
    if (threadIdx.x == 0) {
      st->sh_prologue = 0;
      st->sh_flops += 2.0 * (3.0 * m * (double)n + (double)n * d.kg);
    }
    return;
  }
  const float *q = d.Q + (size_t)t * m;
  const float *g = d.G + (size_t)t * n;
  int *bins = d.bins + (size_t)t * n;
  float *gp = d.GP + (size_t)t * n, *gpt = d.GPT + (size_t)t * n;
  const int kb = st->k_bin;
  const bool ucg = st->flags[F_UCG] != 0;
  if (!ucg) {
    float q2 = 0.0f;
    for (int i = threadIdx.x; i < m; i += SH_THREADS) q2 = fmaf(q[i], q[i], q2);
    q2 = cta_sum(q2, sm);
    if (threadIdx.x == 0) {
      st->red[R_AXT] = q2;
      ctrl_phase(st, C_RCG_ALPHA, 0);
    }
  } else {
    // beta = -<A p_prev_S, A g_S> / ||A p_prev_S||^2 (functions.cu:1169-1178)
    const float *q2u = d.Q2 + (size_t)t * m;
    float d1 = 0.0f, d2 = 0.0f;
    for (int i = threadIdx.x; i < m; i += SH_THREADS) {
      d1 = fmaf(q[i], q2u[i], d1);
      d2 = fmaf(q[i], q[i], d2);
    }
    d1 = cta_sum(d1, sm);
    d2 = cta_sum(d2, sm);
    if (threadIdx.x == 0) {
      st->red[R_DOT1] = d1;
      st->red[R_DOT2] = d2;
      ctrl_phase(st, C_UCG_BETA, 0);
    }
    __syncthreads();
    const float beta = st->cg_beta;
    float gm = 0.0f, d3 = 0.0f, d4 = 0.0f;
    for (int j = threadIdx.x; j < n; j += SH_THREADS) {
      const float v = fmaf(1.0f, g[j], beta * gp[j]);
      gp[j] = v;
      const float pt = bins[j] <= kb ? v : 0.0f;
      gpt[j] = pt;
      gm = fmaxf(gm, fabsf(v));
      d3 = fmaf(pt, bins[j] <= kb ? g[j] : 0.0f, d3);
    }
    for (int i = threadIdx.x; i < m; i += SH_THREADS) {
      const float ap = fmaf(1.0f, q2u[i], beta * q[i]);  // A p = beta A p_prev_S + A g_S
      d4 = fmaf(ap, ap, d4);
    }
    gm = cta_max(gm, sm);
    d3 = cta_sum(d3, sm);
    d4 = cta_sum(d4, sm);
    if (threadIdx.x == 0) {
      st->red[R_GMAX] = gm;
      st->red[R_DOT3] = d3;
      st->red[R_DOT4] = d4;
      ctrl_phase(st, C_UCG_ALPHA, 0);
    }
  }
  __syncthreads();
  // x += alpha grad_previous (algorithms.cu:3840-3845 through the CG step functions)
  const float alpha = st->cg_alpha;
  float *x = d.X + (size_t)t * n;
  float mx = 0.0f;
  for (int j = threadIdx.x; j < n; j += SH_THREADS) {
    const float o = fmaf(alpha, gp[j], x[j]);
    x[j] = o;
    mx = fmaxf(mx, fabsf(o));
  }
  mx = cta_max(mx, sm);
  if (threadIdx.x == 0) {
    st->red[R_XMAX] = mx;
    st->sh_flops += 2.0 * (3.0 * m * (double)n + (double)n * d.kg + (double)m * d.kq * (ucg ? 2 : 1));
    ctrl_phase(st, C_CGIHT_BINDEC, 0);
    ctrl_phase(st, C_BINPREP, 0);
  }
  __syncthreads();
  cta_support_evol(st, x, bins, d.bins_prev + (size_t)t * n, n, d.Xcat + (size_t)t * 3 * n, hist, scan);
  if (threadIdx.x == 0) ctrl_phase(st, C_CGIHT_POST, 0);
  __syncthreads();
  if (st->flags[F_REMASK]) {
    const int kb2 = st->k_bin;
    for (int j = threadIdx.x; j < n; j += SH_THREADS) gpt[j] = bins[j] <= kb2 ? gp[j] : 0.0f;
  }
  __syncthreads();
  if (threadIdx.x == 0) ctrl_phase(st, C_CGIHT_STOP, 0);
  __syncthreads();
  if (d.ml && st->fell_back == 1 && !st->active && st->stop_reason == 8) {
    // the warm start did not lower the residual within 10 iterations: the plain start,
    // its prologue in the next pass
    __syncthreads();
    if (threadIdx.x == 0) {
      const int warm = st->iter;
      const double fl = st->sh_flops;
      *st = d.st0[t];
      st->warm_iters = warm;
      st->sh_flops = fl;
      st->fell_back = 1;
      atomicAdd(d.fallbacks, 1);
    }
    __syncthreads();
    for (int j = threadIdx.x; j < n; j += SH_THREADS) x[j] = d.G0[(size_t)t * n + j];
    __syncthreads();
    cta_start_support(d, t, st, x, hist, scan, sm);
  }
}

// Ordered list of the trials that satisfy `on`, written to list / *count; every thread of
// the 1024-thread block calls it, each owning a contiguous run of trials.
template <class F>
__device__ int cta_list(int T, F on, int *list, int *count) {
  __shared__ int wsum[32];
  const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
  const int per = (T + 1023) / 1024, b0 = min(tid * per, T), b1 = min(b0 + per, T);
  int c = 0;
  for (int t = b0; t < b1; ++t) c += on(t) ? 1 : 0;
  int incl = c;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int v = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += v;
  }
  __syncthreads();
  if (lane == 31) wsum[w] = incl;
  __syncthreads();
  if (w == 0) {
    int v = wsum[lane];
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int u = __shfl_up_sync(0xffffffffu, v, o);
      if (lane >= o) v += u;
    }
    wsum[lane] = v;  // inclusive warp totals
  }
  __syncthreads();
  int pos = incl - c + (w > 0 ? wsum[w - 1] : 0);
  for (int t = b0; t < b1; ++t)
    if (on(t)) list[pos++] = t;
  const int total = wsum[31];
  if (tid == 0) *count = total;
  return total;
}

// The GEMMs' column maps and the loop condition: which 0 -> the active trials (NIHT and
// CGIHT; CGIHT also the trials that run this pass's direction product -- not the ones in a
// restart's prologue -- and the unrestricted-branch trials among them), bounded by
// max_passes; which 1 -> the debias trials (F_CG).  One block of 1024 threads.
__global__ void __launch_bounds__(1024) k_sh_list(ShDev d, int which, int *passes, int max_passes,
                                                  cudaGraphConditionalHandle h) {
  const int T = d.T;
  int total;
  if (which == 0) {
    total = cta_list(T, [&](int t) { return d.st[t].active != 0; }, d.act, d.act_cnt);
    if (d.alg == GB_ALG_CGIHT) {
      cta_list(T, [&](int t) { return d.st[t].active != 0 && d.st[t].fell_back != 1; }, d.act_q, d.act_q_cnt);
      cta_list(T, [&](int t) { return d.st[t].active != 0 && d.st[t].fell_back != 1 && d.st[t].flags[F_UCG] != 0; },
               d.act_u, d.act_u_cnt);
      __syncthreads();
      const int cq = *d.act_q_cnt, cu = *d.act_u_cnt;
      for (int i = threadIdx.x; i < cq + cu; i += blockDim.x) d.act_qu[i] = i < cq ? d.act_q[i] : d.act_u[i - cq] + d.Tp;
      if (threadIdx.x == 0) *d.act_qu_cnt = cq + cu;
    }
  } else {
    total = cta_list(T, [&](int t) { return d.st[t].flags[F_CG] != 0; }, d.act, d.act_cnt);
  }
  if (threadIdx.x == 0) {
    unsigned go = total > 0 ? 1u : 0u;
    if (which == 0) {
      const int p = ++passes[0];
      if (p > max_passes) go = 0u;
    }
    if (h) cudaGraphSetConditional(h, go);
  }
}

// ------------------------------------------------------------------ debias and verdict
// Least squares on the final support of every trial that reached ||y - A x|| <= tol:
// conjugate gradients on the normal equations A_S^T A_S z = A_S^T y started from the NIHT
// solution (CGNR).  The products of all trials run in lockstep as split-precision GEMMs
//   q = [A_hi | A_lo | A_hi] . [p_hi ; p_hi ; p_lo]      g = [A_hi^T | A_lo^T | A_hi^T] . [r_hi ; r_hi ; r_lo]
// (FP32 accumulation, ~2^-17 relative error); the scalars are kept in FP64 and r is
// updated recursively in FP32.  A trial leaves the loop when ||A_S^T r||^2 <= 1e-12 of its
// starting value or after SH_CG_MAX iterations.

// trials that reached the residual tolerance enter the debias
__global__ void k_cg_flags(ShDev d) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= d.T) return;
  GbState *st = d.st + t;
  st->flags[F_CG] = st->stop_reason == 1 ? 1 : 0;
  st->it_cg = 0;
}

// r = y - A x from the last residual GEMM; split r for the A^T product
__global__ void __launch_bounds__(SH_THREADS) k_cg_start(ShDev d) {
  const int t = blockIdx.x, m = d.m;
  GbState *st = d.st + t;
  const bool on = t < d.T && st->flags[F_CG];
  const float *r = d.R + (size_t)t * m;
  __nv_bfloat16 *rc = d.Rcat + (size_t)t * 3 * m;
  for (int i = threadIdx.x; i < m; i += SH_THREADS) {
    const float v = on ? r[i] : 0.0f;
    const __nv_bfloat16 hi = __float2bfloat16_rn(v);
    rc[i] = hi;
    rc[m + i] = hi;
    rc[2 * m + i] = __float2bfloat16_rn(v - __bfloat162float(hi));
  }
}

// g = P_S A^T r ; gamma = ||g||^2 ; p = g + beta p ; convergence test ; split p
__global__ void __launch_bounds__(SH_THREADS) k_cg_dir(ShDev d) {
  __shared__ double smd[32];
  const int t = blockIdx.x, n = d.n;
  if (t >= d.T) return;
  GbState *st = d.st + t;
  if (!st->flags[F_CG]) return;
  const float *g = d.G + (size_t)t * n;
  const int *bins = d.bins + (size_t)t * n;
  const int kb = st->k_bin;
  double gg = 0.0;
  for (int j = threadIdx.x; j < n; j += SH_THREADS) {
    const double v = bins[j] <= kb ? (double)g[j] : 0.0;
    gg += v * v;
  }
  gg = cta_sumd(gg, smd);
  const int it = st->it_cg;
  const double gamma_prev = st->red[R_DOT1];
  if (it == 0) st->red[R_DOT2] = gg;  // every thread reads the same values before this
  const double gamma0 = it == 0 ? gg : st->red[R_DOT2];
  const bool go = it < SH_CG_MAX && gg > 1e-12 * gamma0 && gg > 0.0;
  const float beta = it == 0 ? 0.0f : (float)(gg / gamma_prev);
  float *p = d.P + (size_t)t * n;
  __nv_bfloat16 *pc = d.Xcat + (size_t)t * 3 * n;
  if (go) {
    for (int j = threadIdx.x; j < n; j += SH_THREADS) {
      const float v = bins[j] <= kb ? fmaf(beta, it == 0 ? 0.0f : p[j], g[j]) : 0.0f;
      p[j] = v;
      const __nv_bfloat16 hi = __float2bfloat16_rn(v);
      pc[j] = hi;
      pc[n + j] = hi;
      pc[2 * n + j] = __float2bfloat16_rn(v - __bfloat162float(hi));
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    st->red[R_DOT1] = gg;
    st->flags[F_CG] = go ? 1 : 0;
  }
}

// alpha = gamma / ||q||^2 ; x += alpha p ; r -= alpha q ; split r
__global__ void __launch_bounds__(SH_THREADS) k_cg_step(ShDev d) {
  __shared__ double smd[32];
  const int t = blockIdx.x, n = d.n, m = d.m;
  if (t >= d.T) return;
  GbState *st = d.st + t;
  if (!st->flags[F_CG]) return;
  const float *q = d.Q + (size_t)t * m;
  double qq = 0.0;
  for (int i = threadIdx.x; i < m; i += SH_THREADS) qq += (double)q[i] * (double)q[i];
  qq = cta_sumd(qq, smd);
  const float alpha = qq > 0.0 ? (float)(st->red[R_DOT1] / qq) : 0.0f;
  float *x = d.X + (size_t)t * n;
  const float *p = d.P + (size_t)t * n;
  for (int j = threadIdx.x; j < n; j += SH_THREADS) x[j] = fmaf(alpha, p[j], x[j]);
  float *r = d.R + (size_t)t * m;
  __nv_bfloat16 *rc = d.Rcat + (size_t)t * 3 * m;
  for (int i = threadIdx.x; i < m; i += SH_THREADS) {
    const float v = fmaf(-alpha, q[i], r[i]);
    r[i] = v;
    const __nv_bfloat16 hi = __float2bfloat16_rn(v);
    rc[i] = hi;
    rc[m + i] = hi;
    rc[2 * m + i] = __float2bfloat16_rn(v - __bfloat162float(hi));
  }
  __syncthreads();
  if (threadIdx.x == 0) st->it_cg++;
}

// relative l2 error against x0 (GAGA/gaga/results.cu:468-475) and the verdict
__global__ void __launch_bounds__(SH_THREADS) k_sh_verdict(ShDev d) {
  __shared__ double smd[32];
  const int t = blockIdx.x, n = d.n;
  if (t >= d.T) return;
  const float *x = d.X + (size_t)t * n;
  const float *x0 = d.X0 + (size_t)t * n;
  double e2 = 0.0, x2 = 0.0;
  for (int j = threadIdx.x; j < n; j += SH_THREADS) {
    const double df = (double)x0[j] - (double)x[j];
    e2 += df * df;
    x2 += (double)x0[j] * (double)x0[j];
  }
  e2 = cta_sumd(e2, smd);
  x2 = cta_sumd(x2, smd);
  if (threadIdx.x == 0) {
    const float rel = (float)(sqrt(e2) / sqrt(x2));
    const GbState *st = d.st + t;
    d.iters[t] = st->iter + st->warm_iters;
    d.err[t] = rel;
    d.ok[t] = rel <= 1e-3f ? 1 : 0;
    // GEMM flops this trial used: the initial A^T y, each iteration (CGIHT: counted per
    // pass, plus its prologue's residual and gradient), and the debias
    const double mn3 = 3.0 * d.m * (double)d.n;
    double f = 2.0 * d.n * (double)d.kg;
    if (d.alg == GB_ALG_CGIHT) f += st->sh_flops + 2.0 * (mn3 + (double)d.n * d.kg);
    else f += st->iter * 2.0 * (mn3 + (double)d.n * d.kg + (double)d.m * d.kq);
    if (st->stop_reason == 1) f += (2.0 + st->it_cg) * 2.0 * mn3 * 2.0;
    atomicAdd(d.flops, f);
  }
}

struct Buf {
  std::vector<void *> p;
  ~Buf() {
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

}  // namespace

static thread_local float g_sh_ms = 0.0f;
static thread_local double g_sh_gemm_flops = 0.0;
static thread_local int g_sh_fallbacks = 0;

extern "C" gb_status gb_cs_solve_shared_batch(const gb_shared_batch *b, int *iters_out, float *rel_err_out,
                                              int *success_out, int *num_success) {
  if (!b || !b->k || b->ntrials < 1 || b->m < 128 || b->n < 128 || b->m % 128 || b->n % 128 || b->m > b->n ||
      b->n > 32768 || b->maxiter < 0 || b->precision < 0 || b->precision > 3) {
    gb_set_error_message("shared batch: m, n multiples of 128 with 128 <= m <= n <= 32768, ntrials >= 1", __FILE__,
                         __LINE__);
    return GB_BAD_ARG;
  }
  if ((b->alg != GB_ALG_NIHT && b->alg != GB_ALG_CGIHT) || (b->learned_params && b->alg != GB_ALG_CGIHT)) {
    gb_set_error_message("shared batch: alg is NIHT or CGIHT; the learned warm start is for CGIHT", __FILE__,
                         __LINE__);
    return GB_BAD_ARG;
  }
  const bool cgiht = b->alg == GB_ALG_CGIHT;
  const int m = b->m, n = b->n, T = b->ntrials, Tp = (T + 255) / 256 * 256;  // tcgen05 N tile
  for (int t = 0; t < T; ++t)
    if (b->k[t] < 1 || b->k[t] > m) {
      gb_set_error_message("shared batch: every k must satisfy 1 <= k <= m", __FILE__, __LINE__);
      return GB_BAD_ARG;
    }
  cudaStream_t s = (cudaStream_t)b->stream;
  Buf buf;
  ShDev d;
  memset(&d, 0, sizeof(d));
  d.m = m; d.n = n; d.T = T; d.Tp = Tp; d.maxiter = b->maxiter; d.tol_rel = b->tol_rel; d.seed = b->seed;
  d.prec = b->precision;
  d.first = b->first_trial;
  d.alg = b->alg;
  d.ml = b->learned_params;
  const int kg = (d.prec & 1) ? 3 * m : m, kq = (d.prec & 2) ? 3 * n : n;  // K of A^T r and A x_thres
  d.kg = kg;
  d.kq = kq;
  int *dk;
  GB_TRY(buf.get(&dk, T));
  GB_CUDA_TRY(cudaMemcpyAsync(dk, b->k, sizeof(int) * T, cudaMemcpyHostToDevice, s));
  d.kreq = dk;
  GB_TRY(buf.get(&d.A32, (size_t)m * n));
  GB_TRY(buf.get(&d.Acat, (size_t)m * 3 * n));
  GB_TRY(buf.get(&d.ATcat, (size_t)n * 3 * m));
  for (float **v : {&d.X0, &d.X, &d.G}) GB_TRY(buf.get(v, (size_t)Tp * n));
  // CGIHT keeps Q2 and XT2 right after Q and XTbf (one GEMM forms both direction products)
  const size_t qrows = cgiht ? 2 * (size_t)Tp : (size_t)Tp;
  for (float **v : {&d.Y, &d.R}) GB_TRY(buf.get(v, (size_t)Tp * m));
  GB_TRY(buf.get(&d.Q, qrows * m));
  GB_TRY(buf.get(&d.Xcat, (size_t)Tp * 3 * n));
  GB_TRY(buf.get(&d.XTbf, qrows * 3 * n));
  GB_TRY(buf.get(&d.Rbf, (size_t)Tp * m));
  GB_TRY(buf.get(&d.bins, (size_t)Tp * n));
  GB_TRY(buf.get(&d.st, (size_t)Tp));
  GB_TRY(buf.get(&d.P, (size_t)Tp * n));
  GB_TRY(buf.get(&d.Rcat, (size_t)Tp * 3 * m));
  GB_TRY(buf.get(&d.iters, T));
  GB_TRY(buf.get(&d.err, T));
  GB_TRY(buf.get(&d.ok, T));
  int *passes;
  GB_TRY(buf.get(&passes, 1));
  GB_TRY(buf.get(&d.act, Tp));
  GB_TRY(buf.get(&d.act_cnt, 1));
  if (cgiht) {
    for (float **v : {&d.GP, &d.GPT}) GB_TRY(buf.get(v, (size_t)Tp * n));
    d.Q2 = d.Q + (size_t)Tp * m;
    d.XT2 = d.XTbf + (size_t)Tp * kq;
    GB_TRY(buf.get(&d.bins_prev, (size_t)Tp * n));
    GB_TRY(buf.get(&d.act_q, Tp));
    GB_TRY(buf.get(&d.act_q_cnt, 1));
    GB_TRY(buf.get(&d.act_u, Tp));
    GB_TRY(buf.get(&d.act_u_cnt, 1));
    GB_TRY(buf.get(&d.act_qu, 2 * (size_t)Tp));
    GB_TRY(buf.get(&d.act_qu_cnt, 1));
    GB_TRY(buf.get(&d.fallbacks, 1));
    GB_CUDA_TRY(cudaMemsetAsync(d.fallbacks, 0, sizeof(int), s));
    GB_CUDA_TRY(cudaMemsetAsync(d.bins_prev, 0, sizeof(int) * (size_t)Tp * n, s));
    if (d.ml) {
      GB_TRY(buf.get(&d.G0, (size_t)Tp * n));
      GB_TRY(buf.get(&d.st0, (size_t)Tp));
    }
  }
  const int max_passes = d.maxiter + 4 + (d.ml ? 11 : 0);
  GB_TRY(buf.get(&d.flops, 1));
  GB_CUDA_TRY(cudaMemsetAsync(d.flops, 0, sizeof(double), s));
  // split-K workspace of the GEMMs over the active trials (they run one after another)
  int dev = 0, sms = 0;
  GB_CUDA_TRY(cudaGetDevice(&dev));
  GB_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  GbGemmWs ws = {};
  ws.num_sms = sms;
  ws.part_tiles = 4 * sms;  // room for the joined Q / Q2 call's split partials
  ws.ticket_count = (n / 128) * (Tp / 128);
  GB_TRY(buf.get(&ws.part, (size_t)ws.part_tiles * 128 * 128));
  GB_TRY(buf.get(&ws.tickets, ws.ticket_count));
  ws.gather_elems = qrows * 3 * std::max(m, n);  // widest B operand: Tp x 3n (CGIHT's [p; g_S]: 2 Tp x kq)
  {
    __nv_bfloat16 *gbuf = nullptr;
    GB_TRY(buf.get(&gbuf, ws.gather_elems));
    ws.gather = gbuf;
  }
  GB_CUDA_TRY(cudaMemsetAsync(ws.tickets, 0, sizeof(unsigned) * ws.ticket_count, s));
  // Ct[Tp x M] = [Y -] A . B^T over all trials, or over the listed ones (map / count)
  auto gemm_map = [&](const void *A, const void *B, float *C, int M, int K, int lda, int ldb, const float *Y, void *Cb,
                      int split, const int *map, const int *count, cudaStream_t st, int N = 0) {
    GbGemm g = {};
    g.A = A; g.B = B; g.Ct = C; g.M = M; g.N = N > 0 ? N : Tp; g.K = K; g.lda = lda; g.ldb = ldb; g.Y = Y; g.Cb = Cb;
    g.split_rows = g.N > Tp;  // the joined Q / Q2 call: each block split as its own call would be
    g.cb_split = split;
    if (map) {
      g.nmap = map;
      g.ncount = count;
      g.ws = &ws;
    }
    return gb_gemm(g, st);
  };
  auto gemm = [&](const void *A, const void *B, float *C, int M, int K, int lda, int ldb, const float *Y, void *Cb,
                  int split, bool mapped, cudaStream_t st) {
    return gemm_map(A, B, C, M, K, lda, ldb, Y, Cb, split, mapped ? d.act : nullptr, mapped ? d.act_cnt : nullptr,
                    st);
  };
  GB_CUDA_TRY(cudaMemsetAsync(passes, 0, sizeof(int), s));
  GB_CUDA_TRY(cudaMemsetAsync(d.st, 0, sizeof(GbState) * Tp, s));
  const int smem_n = n * (int)sizeof(int);
  GB_CUDA_TRY(cudaFuncSetAttribute(k_sh_genx, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_n));
  GB_CUDA_TRY(cudaFuncSetAttribute(k_sh_y, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_n));
  cudaEvent_t e0, e1;
  GB_CUDA_TRY(cudaEventCreate(&e0));
  GB_CUDA_TRY(cudaEventCreate(&e1));
  GB_CUDA_TRY(cudaEventRecord(e0, s));
  // ---- problem and operands
  k_sh_genA<<<2048, 256, 0, s>>>(d.A32, m, n, b->seed);
  k_sh_split<<<dim3(m / 32, n / 32), dim3(32, 8), 0, s>>>(d.A32, d.Acat, d.ATcat, m, n);
  k_sh_genx<<<Tp, SH_THREADS, smem_n, s>>>(d);
  k_sh_y<<<Tp, SH_THREADS, smem_n, s>>>(d);
  // ---- x = H_k(A^T y): G = A_hi^T bf16(y) (Rbf holds bf16(y) here)
  GB_TRY(gemm(d.ATcat, (d.prec & 1) ? (const void *)d.Rcat : d.Rbf, d.G, n, kg, 3 * m, kg, nullptr, nullptr, 0, false,
              s));
  const int split_r = (d.prec & 1) != 0;
  void *rb = split_r ? (void *)d.Rcat : (void *)d.Rbf;
  if (!cgiht) {
    k_sh_init<<<Tp, SH_THREADS, 0, s>>>(d);
  } else {
    // CGIHT: x = H_k(A^T y) or the learned start, then r0 = y - A x, grad_previous = A^T r0
    const int smem = (ML_P + 2 * ML_RANK_BINS) * (int)sizeof(float);
    GB_CUDA_TRY(cudaFuncSetAttribute(k_sc_init, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
    k_sc_init<<<Tp, SH_THREADS, smem, s>>>(d);
    GB_TRY(gemm(d.Acat, d.Xcat, d.R, m, 3 * n, 3 * n, 3 * n, d.Y, rb, split_r, false, s));
    GB_TRY(gemm(d.ATcat, rb, d.G, n, kg, 3 * m, kg, nullptr, nullptr, 0, false, s));
    k_sc_init2<<<Tp, SH_THREADS, 0, s>>>(d);
  }
  GB_CUDA_TRY(cudaGetLastError());
  // ---- NIHT / CGIHT iterations in lockstep, WHILE any trial is active; then the debias
  // R = Y - A X (and its BF16 form for the next product), G = A^T R over the active trials;
  // NIHT then Q = A x_thres, CGIHT Q = A p and (unrestricted branch) Q2 = A g_S
  auto iter_body = [&](cudaStream_t c) -> gb_status {
    gb_status r = gemm(d.Acat, d.Xcat, d.R, m, 3 * n, 3 * n, 3 * n, d.Y, rb, split_r, true, c);
    if (r == GB_OK) r = gemm(d.ATcat, rb, d.G, n, kg, 3 * m, kg, nullptr, nullptr, 0, true, c);
    if (!cgiht) {
      k_sh_mask<<<Tp, SH_THREADS, 0, c>>>(d);
      if (r == GB_OK) r = gemm(d.Acat, d.XTbf, d.Q, m, kq, 3 * n, kq, nullptr, nullptr, 0, true, c);
      k_sh_step<<<Tp, SH_THREADS, 0, c>>>(d);
    } else {
      k_sc_dir<<<Tp, SH_THREADS, 0, c>>>(d);
      // Q = A p (act_q) and Q2 = A g_S (act_u) in one GEMM over the concatenated list: while
      // both fit one 256-column tile, A streams once per pass instead of twice
      if (r == GB_OK)
        r = gemm_map(d.Acat, d.XTbf, d.Q, m, kq, 3 * n, kq, nullptr, nullptr, 0, d.act_qu, d.act_qu_cnt, c, 2 * Tp);
      k_sc_step<<<Tp, SH_THREADS, 0, c>>>(d);
    }
    return r;
  };
  // debias of the converged trials: r = y - A x, g = A^T r, then CG in lockstep while any
  // of them iterates
  auto cg_prologue = [&](cudaStream_t c) -> gb_status {
    k_cg_flags<<<(Tp + 255) / 256, 256, 0, c>>>(d);
    k_sh_list<<<1, 1024, 0, c>>>(d, 1, passes, max_passes, 0);
    gb_status r = gemm(d.Acat, d.Xcat, d.R, m, 3 * n, 3 * n, 3 * n, d.Y, nullptr, 0, true, c);
    if (r == GB_OK) {
      k_cg_start<<<Tp, SH_THREADS, 0, c>>>(d);
      r = gemm(d.ATcat, d.Rcat, d.G, n, 3 * m, 3 * m, 3 * m, nullptr, nullptr, 0, true, c);
    }
    if (r == GB_OK) k_cg_dir<<<Tp, SH_THREADS, 0, c>>>(d);
    return r;
  };
  auto cg_body = [&](cudaStream_t c) -> gb_status {
    gb_status r = gemm(d.Acat, d.Xcat, d.Q, m, 3 * n, 3 * n, 3 * n, nullptr, nullptr, 0, true, c);  // q = A p
    k_cg_step<<<Tp, SH_THREADS, 0, c>>>(d);
    if (r == GB_OK) r = gemm(d.ATcat, d.Rcat, d.G, n, 3 * m, 3 * m, 3 * m, nullptr, nullptr, 0, true, c);
    k_cg_dir<<<Tp, SH_THREADS, 0, c>>>(d);
    return r;
  };
  cudaStream_t c0 = nullptr, c1 = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  gb_status rc = GB_OK;
  // GB_CS_EAGER=1: the same kernels launched one by one from the host, the loop conditions
  // read back after every pass (slower; for profilers that cannot see inside graphs with
  // conditional nodes)
  static const bool eager = getenv("GB_CS_EAGER") && atoi(getenv("GB_CS_EAGER")) != 0;
  if (eager) {
    auto go = [&](int which, bool *more) -> gb_status {
      k_sh_list<<<1, 1024, 0, s>>>(d, which, passes, max_passes, 0);
      int cnt = 0, p = 0;
      GB_CUDA_TRY(cudaMemcpyAsync(&cnt, d.act_cnt, sizeof(int), cudaMemcpyDeviceToHost, s));
      GB_CUDA_TRY(cudaMemcpyAsync(&p, passes, sizeof(int), cudaMemcpyDeviceToHost, s));
      GB_CUDA_TRY(cudaStreamSynchronize(s));
      *more = cnt > 0 && (which != 0 || p <= max_passes);
      return GB_OK;
    };
    bool more = false;
    rc = go(0, &more);
    while (rc == GB_OK && more) {
      rc = iter_body(s);
      if (rc == GB_OK) rc = go(0, &more);
    }
    if (rc == GB_OK) rc = cg_prologue(s);
    if (rc == GB_OK) rc = go(1, &more);
    for (int guard = 0; rc == GB_OK && more && guard <= 4 * SH_CG_MAX; ++guard) {
      rc = cg_body(s);
      if (rc == GB_OK) rc = go(1, &more);
    }
  } else {
    GB_CUDA_TRY(cudaStreamCreateWithFlags(&c0, cudaStreamNonBlocking));
    GB_CUDA_TRY(cudaStreamCreateWithFlags(&c1, cudaStreamNonBlocking));
    cudaError_t e = cudaStreamBeginCapture(c0, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) {
      gb_set_error_message(cudaGetErrorString(e), __FILE__, __LINE__);
      rc = GB_CUDA_ERROR;
    }
    cudaGraphConditionalHandle h = 0;
    if (rc == GB_OK) rc = gb_make_handle(c0, &h);
    if (rc == GB_OK) {
      k_sh_list<<<1, 1024, 0, c0>>>(d, 0, passes, max_passes, h);
      rc = gb_open_while(c0, c1, h);
    }
    if (rc == GB_OK) {
      rc = iter_body(c1);
      k_sh_list<<<1, 1024, 0, c1>>>(d, 0, passes, max_passes, h);
      gb_status rc2 = gb_close_while(c1);
      if (rc == GB_OK) rc = rc2;
    }
    cudaGraphConditionalHandle h2 = 0;
    if (rc == GB_OK) rc = cg_prologue(c0);
    if (rc == GB_OK) rc = gb_make_handle(c0, &h2);
    if (rc == GB_OK) {
      k_sh_list<<<1, 1024, 0, c0>>>(d, 1, passes, max_passes, h2);
      rc = gb_open_while(c0, c1, h2);
    }
    if (rc == GB_OK) {
      rc = cg_body(c1);
      k_sh_list<<<1, 1024, 0, c1>>>(d, 1, passes, max_passes, h2);
      gb_status rc2 = gb_close_while(c1);
      if (rc == GB_OK) rc = rc2;
    }
    cudaGraph_t g2 = nullptr;
    cudaError_t e2 = cudaStreamEndCapture(c0, &g2);
    if (rc == GB_OK && e2 != cudaSuccess) {
      gb_set_error_message(cudaGetErrorString(e2), __FILE__, __LINE__);
      rc = GB_CUDA_ERROR;
    }
    graph = g2;
    if (rc == GB_OK) {
      e = cudaGraphInstantiate(&exec, graph, 0);
      if (e == cudaSuccess) e = cudaGraphLaunch(exec, s);
      if (e != cudaSuccess) {
        gb_set_error_message(cudaGetErrorString(e), __FILE__, __LINE__);
        rc = GB_CUDA_ERROR;
      }
    }
  }
  if (rc == GB_OK) {
    k_sh_verdict<<<Tp, SH_THREADS, 0, s>>>(d);
    cudaEventRecord(e1, s);
    if (b->d_A_out) cudaMemcpyAsync(b->d_A_out, d.A32, sizeof(float) * (size_t)m * n, cudaMemcpyDeviceToDevice, s);
    if (b->d_Y_out) cudaMemcpyAsync(b->d_Y_out, d.Y, sizeof(float) * (size_t)T * m, cudaMemcpyDeviceToDevice, s);
    if (b->d_X0_out) cudaMemcpyAsync(b->d_X0_out, d.X0, sizeof(float) * (size_t)T * n, cudaMemcpyDeviceToDevice, s);
    if (b->d_X_out) cudaMemcpyAsync(b->d_X_out, d.X, sizeof(float) * (size_t)T * n, cudaMemcpyDeviceToDevice, s);
    std::vector<int> hit(T), hok(T);
    std::vector<float> herr(T);
    double hflops = 0.0;
    int hfb = 0;
    if (d.fallbacks) cudaMemcpyAsync(&hfb, d.fallbacks, sizeof(int), cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(hit.data(), d.iters, sizeof(int) * T, cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(herr.data(), d.err, sizeof(float) * T, cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(hok.data(), d.ok, sizeof(int) * T, cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(&hflops, d.flops, sizeof(double), cudaMemcpyDeviceToHost, s);
    cudaError_t e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
      gb_set_error_message(cudaGetErrorString(e), __FILE__, __LINE__);
      rc = GB_CUDA_ERROR;
    } else if ((rc = gb_gemm_tc_check()) != GB_OK) {
      // a tcgen05 GEMM gave up on a wait: results are not valid
    } else {
      cudaEventElapsedTime(&g_sh_ms, e0, e1);
      g_sh_gemm_flops = hflops;
      g_sh_fallbacks = hfb;
      int ns = 0;
      for (int t = 0; t < T; ++t) {
        if (iters_out) iters_out[t] = hit[t];
        if (rel_err_out) rel_err_out[t] = herr[t];
        if (success_out) success_out[t] = hok[t];
        ns += hok[t];
      }
      if (num_success) *num_success = ns;
    }
  }
  if (exec) cudaGraphExecDestroy(exec);
  if (graph) cudaGraphDestroy(graph);
  if (c0) cudaStreamDestroy(c0);
  if (c1) cudaStreamDestroy(c1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return rc;
}

extern "C" void gb_cs_shared_last_stats(double *gemm_flops, float *ms) {
  if (gemm_flops) *gemm_flops = g_sh_gemm_flops;
  if (ms) *ms = g_sh_ms;
}

extern "C" int gb_cs_shared_last_fallbacks(void) { return g_sh_fallbacks; }
