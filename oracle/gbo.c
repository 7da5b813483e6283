/*
 * gbo.c -- CPU oracle (test infrastructure only; see gbo.h).
 *
 * Build: oracle/build.py (gcc -O2 -fopenmp -ffp-contract=off).  Floating-point
 * contraction is disabled so that every multiply-add below is exactly the
 * operation written; where the reference's nvcc build fuses a multiply-add
 * (cuBLAS saxpy, `slope * intercept + 1.0f` in LinearBinning) an explicit fmaf
 * is written instead.
 */
#include "gbo.h"

#include <float.h>
#include <limits.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* ------------------------------------------------------------------ */
/* Philox-4x32-10 (Salmon, Moraes, Dror, Shaw: "Parallel random numbers: as easy
 * as 1, 2, 3", SC'11).  The reference uses cuRAND's default generator, which is
 * not reproducible outside that closed library; problems are therefore generated
 * from this counter-based generator and handed to every implementation. */
void gbo_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
  uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3];
  uint32_t k0 = key[0], k1 = key[1];
  for (int r = 0; r < 10; ++r) {
    uint64_t p0 = (uint64_t)0xD2511F53u * c0;
    uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
    uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
    uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
    uint32_t n0 = hi1 ^ c1 ^ k0, n2 = hi0 ^ c3 ^ k1;
    c0 = n0; c1 = lo1; c2 = n2; c3 = lo0;
    k0 += 0x9E3779B9u; k1 += 0xBB67AE85u;
  }
  out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

/* uniform on (0,1): 24 random bits, centred in their cell (exact in float) */
float gbo_u01(uint32_t x) { return ((float)(x >> 8) + 0.5f) * (1.0f / 16777216.0f); }

enum { ST_MATRIX = 1, ST_VALUES = 2, ST_SUPPORT = 3, ST_ROWS = 4, ST_SMV = 5, ST_SIGNS = 6 };
static const uint32_t KEY_HI = 0x6A09E667u;

static void draw4(uint32_t seed, uint32_t trial, uint32_t stream, uint64_t block, uint32_t out[4]) {
  uint32_t ctr[4] = {(uint32_t)block, (uint32_t)(block >> 32), stream, trial};
  uint32_t key[2] = {seed, KEY_HI};
  gbo_philox4x32_10(ctr, key, out);
}

static float box_muller(uint32_t a, uint32_t b, int second) {
  double u1 = gbo_u01(a), u2 = gbo_u01(b);
  double r = sqrt(-2.0 * log(u1));
  double t = 6.283185307179586 * u2;
  return (float)(second ? r * sin(t) : r * cos(t));
}

/* element e of a gaussian stream: one Philox call gives 4 normals */
static float gauss_at(uint32_t seed, uint32_t trial, uint32_t stream, uint64_t e) {
  uint32_t o[4];
  draw4(seed, trial, stream, e >> 2, o);
  int lane = (int)(e & 3);
  return lane < 2 ? box_muller(o[0], o[1], lane) : box_muller(o[2], o[3], lane - 2);
}

static float uniform_at(uint32_t seed, uint32_t trial, uint32_t stream, uint64_t e) {
  uint32_t o[4];
  draw4(seed, trial, stream, e >> 2, o);
  return gbo_u01(o[e & 3]);
}

/* createMeasurements_gen (GAGA/gaga/createMeasurements_gen.cu:81-100): N(0,1) or
 * +-1 entries, scaled by 1/sqrt(m) in float. */
void gbo_gen_dense(int m, int n, int lda, int ens, uint32_t seed, uint32_t trial, float *A) {
  float scale = sqrtf((float)m);
  scale = 1.0f / scale;
#pragma omp parallel for schedule(static)
  for (int j = 0; j < n; ++j) {
    for (int i = 0; i < m; ++i) {
      uint64_t e = (uint64_t)j * (uint64_t)m + (uint64_t)i;
      float v;
      if (ens == 2) v = signbit(uniform_at(seed, trial, ST_MATRIX, e) - 0.5f) ? -1.0f : 1.0f;
      else v = gauss_at(seed, trial, ST_MATRIX, e);
      A[(size_t)j * lda + i] = v * scale;
    }
    for (int i = m; i < lda; ++i) A[(size_t)j * lda + i] = 0.0f;
  }
}

/* createVector (GAGA/gaga/createVector.cu:207-300) with the value distributions of
 * createProblem_gen (GAGA/gaga/createProblem_gen.cu:70-95 / sign_pattern). */
int gbo_gen_vector(int n, int k, int vec_dist, uint32_t seed, uint32_t trial, float *x) {
  float *vals = (float *)malloc(sizeof(float) * n);
  float *keys = (float *)malloc(sizeof(float) * n);
  int *bins = (int *)malloc(sizeof(int) * n);
  int *cnt = (int *)calloc((size_t)n, sizeof(int));
  for (int i = 0; i < n; ++i) {
    float u = uniform_at(seed, trial, ST_VALUES, (uint64_t)i);
    if (vec_dist == 1) vals[i] = signbit(u - 0.5f) ? -1.0f : 1.0f;
    else if (vec_dist == 2) vals[i] = gauss_at(seed, trial, ST_VALUES, (uint64_t)i);
    else vals[i] = u;
    keys[i] = uniform_at(seed, trial, ST_SUPPORT, (uint64_t)i);
  }
  float max_value = gbo_max_magnitude(keys, n);
  float slope = ((float)(n - 1) / max_value);
  gbo_linear_binning(keys, n, n, n, slope, max_value, bins, cnt);
  int k_bin = 0, sum = 0;
  while ((sum < k) & (k_bin < n)) { sum += cnt[k_bin]; k_bin++; }
  k_bin -= 1;
  for (int i = 0; i < n; ++i) x[i] = (bins[i] <= k_bin) ? vals[i] : 0.0f;
  free(vals); free(keys); free(bins); free(cnt);
  return sum;
}

void gbo_gen_dct_rows(int n, int m, uint32_t seed, uint32_t trial, int *rows) {
  int *idx = (int *)malloc(sizeof(int) * n);
  for (int i = 0; i < n; ++i) idx[i] = i;
  for (int j = n - 1; j > n - m; --j) {
    float u = uniform_at(seed, trial, ST_ROWS, (uint64_t)j);
    int kk = (int)((float)j * u);
    int t = idx[j]; idx[j] = idx[kk]; idx[kk] = t;
  }
  for (int j = 0; j < m; ++j) rows[j] = idx[n - 1 - j];
  free(idx);
}

void gbo_gen_smv(int m, int n, int d, int ens, uint32_t seed, uint32_t trial, int *rows, float *vals) {
  float scale = 1.0f;
  if (ens == 1 || ens == 2) { scale = sqrtf((float)d); scale = 1.0f / scale; }
#pragma omp parallel for schedule(static)
  for (int j = 0; j < n; ++j) {
    int have = 0;
    uint64_t draw = 0;
    while (have < d) {
      uint32_t o[4];
      uint32_t ctr[4] = {(uint32_t)j, (uint32_t)draw, ST_SMV, trial};
      uint32_t key[2] = {seed, KEY_HI};
      gbo_philox4x32_10(ctr, key, o);
      draw++;
      for (int q = 0; q < 4 && have < d; ++q) {
        int r = (int)((float)m * gbo_u01(o[q]));
        if (r == m) r = m - 1;
        int dup = 0;
        for (int t = 0; t < have; ++t) dup |= (rows[(size_t)j * d + t] == r);
        if (!dup) rows[(size_t)j * d + have++] = r;
      }
    }
    for (int t = 0; t < d; ++t) {
      float v = 1.0f;
      if (ens == 2) v = signbit(uniform_at(seed, trial, ST_SIGNS, (uint64_t)j * d + t) - 0.5f) ? -1.0f : 1.0f;
      vals[(size_t)j * d + t] = v * scale;
    }
  }
}

/* ------------------------------------------------------------------ */
/* reductions: FP64 accumulation, FP32 result */
static float dotf(const float *a, const float *b, int n) {
  double s = 0.0;
  for (int i = 0; i < n; ++i) s += (double)a[i] * (double)b[i];
  return (float)s;
}
static float nrm2f(const float *a, int n) {
  double s = 0.0;
  for (int i = 0; i < n; ++i) s += (double)a[i] * (double)a[i];
  return (float)sqrt(s);
}
/* cublasSaxpy: y = alpha*x + y, fused */
static void saxpy(int n, float alpha, const float *x, float *y) {
  for (int i = 0; i < n; ++i) y[i] = fmaf(alpha, x[i], y[i]);
}
static void sscal(int n, float alpha, float *x) {
  for (int i = 0; i < n; ++i) x[i] = alpha * x[i];
}

/* MaxMagnitude (GAGA/gaga/functions.cu:382-393): |v| at the first index of max |v| */
float gbo_max_magnitude(const float *v, int n) {
  float best = -1.0f;
  for (int i = 0; i < n; ++i) {
    float a = fabsf(v[i]);
    if (a > best) best = a;
  }
  return best < 0.0f ? 0.0f : best;
}

/* ------------------------------------------------------------------ */
/* Operators */

static void dense_A(const gbo_op *op, const float *x, float *y) {
  int m = op->m, n = op->n, lda = op->lda;
  int *nz = (int *)malloc(sizeof(int) * (n > 0 ? n : 1));
  int cnt = 0;
  for (int j = 0; j < n; ++j)
    if (x[j] != 0.0f) nz[cnt++] = j;
  /* gen_matvec_sparse (GAGA/Matrices/gen_gpu.cu:79-132) reads only the
   * columns where x is nonzero */
#pragma omp parallel for schedule(static)
  for (int i0 = 0; i0 < m; i0 += 256) {
    int i1 = i0 + 256 < m ? i0 + 256 : m;
    float acc[256];
    for (int i = i0; i < i1; ++i) acc[i - i0] = 0.0f;
    for (int t = 0; t < cnt; ++t) {
      int j = nz[t];
      float xj = x[j];
      const float *col = op->A + (size_t)j * lda;
      for (int i = i0; i < i1; ++i) acc[i - i0] = acc[i - i0] + col[i] * xj;
    }
    for (int i = i0; i < i1; ++i) y[i] = acc[i - i0];
  }
  free(nz);
}

static void dense_AT(const gbo_op *op, const float *r, float *g) {
  int m = op->m, n = op->n, lda = op->lda;
#pragma omp parallel for schedule(static)
  for (int j = 0; j < n; ++j) {
    const float *col = op->A + (size_t)j * lda;
    float s[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    int i = 0;
    for (; i + 8 <= m; i += 8)
      for (int q = 0; q < 8; ++q) s[q] = s[q] + col[i + q] * r[i + q];
    for (; i < m; ++i) s[0] = s[0] + col[i] * r[i];
    g[j] = ((s[0] + s[1]) + (s[2] + s[3])) + ((s[4] + s[5]) + (s[6] + s[7]));
  }
}

/* iterative radix-2 complex FFT in double; sign -1 forward, +1 inverse (unnormalised) */
static void fft_d(double *re, double *im, int N, int sign) {
  for (int i = 1, j = 0; i < N; ++i) {
    int bit = N >> 1;
    for (; j & bit; bit >>= 1) j ^= bit;
    j ^= bit;
    if (i < j) {
      double t = re[i]; re[i] = re[j]; re[j] = t;
      t = im[i]; im[i] = im[j]; im[j] = t;
    }
  }
  for (int len = 2; len <= N; len <<= 1) {
    double ang = sign * 2.0 * M_PI / len;
    int half = len >> 1;
#pragma omp parallel for schedule(static) if (N >= (1 << 16))
    for (int i = 0; i < N; i += len) {
      for (int q = 0; q < half; ++q) {
        double wr = cos(ang * q), wi = sin(ang * q);
        double ur = re[i + q], ui = im[i + q];
        double vr = re[i + q + half] * wr - im[i + q + half] * wi;
        double vi = re[i + q + half] * wi + im[i + q + half] * wr;
        re[i + q] = ur + vr; im[i + q] = ui + vi;
        re[i + q + half] = ur - vr; im[i + q + half] = ui - vi;
      }
    }
  }
}

/* Orthonormal DCT-II by Makhoul's reordering (as GAGA/Matrices/dct_gpu.cu:121-206,
 * __split + C2C + __fft2dct), evaluated in FP64. */
void gbo_dct2(int N, const float *x, float *out) {
  double *re = (double *)malloc(sizeof(double) * N), *im = (double *)calloc((size_t)N, sizeof(double));
  for (int m = 0; m < N / 2; ++m) { re[m] = x[2 * m]; re[N - 1 - m] = x[2 * m + 1]; }
  fft_d(re, im, N, -1);
  for (int k = 0; k < N; ++k) {
    double f = k * M_PI / (2.0 * N);
    double w = k == 0 ? sqrt(1.0 / N) : sqrt(2.0 / N);
    out[k] = (float)(w * (re[k] * cos(f) + im[k] * sin(f)));
  }
  free(re); free(im);
}

/* Its transpose, DCT-III (as __dct2fft + inverse C2C + __gather, dct_gpu.cu:121-206,287-314) */
void gbo_dct3(int N, const float *X, float *out) {
  double *re = (double *)malloc(sizeof(double) * N), *im = (double *)malloc(sizeof(double) * N);
  for (int k = 0; k < N; ++k) {
    double f = k * M_PI / (2.0 * N);
    double w = k == 0 ? sqrt(1.0 / N) : sqrt(2.0 / N);
    re[k] = w * X[k] * cos(f);
    im[k] = w * X[k] * sin(f);
  }
  fft_d(re, im, N, +1);
  for (int m = 0; m < N / 2; ++m) { out[2 * m] = (float)re[m]; out[2 * m + 1] = (float)re[N - 1 - m]; }
  free(re); free(im);
}

static void dct_A(const gbo_op *op, const float *x, float *y) {
  float *full = (float *)malloc(sizeof(float) * op->n);
  gbo_dct2(op->n, x, full);
  for (int i = 0; i < op->m; ++i) y[i] = full[op->dct_rows[i]];
  free(full);
}

static void dct_AT(const gbo_op *op, const float *r, float *g) {
  float *full = (float *)calloc((size_t)op->n, sizeof(float));
  for (int i = 0; i < op->m; ++i) full[op->dct_rows[i]] = r[i];
  gbo_dct3(op->n, full, g);
  free(full);
}

/* sparse_matvec / sparse_matvecT (GAGA/Matrices/smv_gpu.cu:29-47); nonzeros summed in
 * storage order (the reference's atomicAdd order is unspecified) */
static void smv_A(const gbo_op *op, const float *x, float *y) {
  int d = op->d;
  for (int i = 0; i < op->m; ++i) y[i] = 0.0f;
  for (int j = 0; j < op->n; ++j) {
    if (x[j] == 0.0f) continue;
    for (int t = 0; t < d; ++t) {
      float v = op->smv_vals[(size_t)j * d + t] * x[j];
      if (v != 0.0f) y[op->smv_rows[(size_t)j * d + t]] += v;
    }
  }
}

static void smv_AT(const gbo_op *op, const float *r, float *g) {
  int d = op->d;
#pragma omp parallel for schedule(static)
  for (int j = 0; j < op->n; ++j) {
    float s = 0.0f;
    for (int t = 0; t < d; ++t) s = s + op->smv_vals[(size_t)j * d + t] * r[op->smv_rows[(size_t)j * d + t]];
    g[j] = s;
  }
}

void gbo_A(const gbo_op *op, const float *x, float *y) {
  if (op->kind == GBO_OP_DENSE) dense_A(op, x, y);
  else if (op->kind == GBO_OP_DCT) dct_A(op, x, y);
  else smv_A(op, x, y);
}
void gbo_AT(const gbo_op *op, const float *r, float *g) {
  if (op->kind == GBO_OP_DENSE) dense_AT(op, r, g);
  else if (op->kind == GBO_OP_DCT) dct_AT(op, r, g);
  else smv_AT(op, r, g);
}

/* ------------------------------------------------------------------ */
/* Support selection */

/* float -> int32 conversion with round-toward-zero and saturation, NaN -> 0: the
 * semantics of the GPU conversion the reference kernel performs when it stores a
 * float expression into an int (cvt.rzi.s32.f32). */
int gbo_f2i_rz(float v) {
  if (v != v) return 0;
  if (v >= 2147483648.0f) return INT_MAX;
  if (v <= -2147483648.0f) return INT_MIN;
  return (int)v;
}

/* LinearBinning (GAGA/gaga/kernels.cu:135-146).  The magnitude test is done in double
 * (`intercept * .000001` is a double product); bins use FP32 `slope*(intercept-t)`
 * clamped at 0; tiny entries get bin (int)(slope*intercept + 1.0f), which nvcc
 * contracts to one fused multiply-add. */
void gbo_linear_binning(const float *v, int n, int num_bins, int max_bin, float slope,
                        float intercept, int *bins, int *counters) {
  (void)num_bins;
  double small = (double)intercept * 0.000001;
  for (int i = 0; i < n; ++i) {
    float t = fabsf(v[i]);
    if ((double)t > small) {
      float b = slope * (intercept - t);
      int bi = gbo_f2i_rz(fmaxf(0.0f, b));
      bins[i] = bi;
      if (bi < max_bin) counters[bi] += 1;
    } else {
      bins[i] = gbo_f2i_rz(fmaf(slope, intercept, 1.0f));
    }
  }
}

/* FindSupportSet (GAGA/gaga/functions.cu:397-436) */
int gbo_find_support_set(const float *v, int *bins, int *counters, float slope, float intercept,
                         float max_change, gbo_bin_state *st, int n, int k) {
  float min_val = st->min_val;
  int max_bin = st->max_bin;
  int k_bin = st->k_bin;
  int sum = st->sum; /* the reference returns an uninitialised sum on this path */
  if (min_val > max_change) {
    min_val = min_val - max_change;
  } else {
    memset(counters, 0, sizeof(int) * st->num_bins);
    gbo_linear_binning(v, n, st->num_bins, max_bin, slope, intercept, bins, counters);
    k_bin = 0;
    sum = 0;
    while ((sum < k) & (k_bin < max_bin)) {
      sum = sum + counters[k_bin];
      k_bin++;
    }
    k_bin = k_bin - 1;
    if (sum < k) {
      st->alpha = st->alpha * 0.5f;
      st->max_bin = (int)((float)st->num_bins * (1.0f - st->alpha));
    }
    min_val = intercept - (float)(k_bin + 1) / slope;
  }
  st->min_val = min_val;
  st->k_bin = k_bin;
  st->sum = sum;
  return sum;
}

/* threshold (GAGA/gaga/kernels.cu:74-81) */
void gbo_threshold(float *v, const int *bins, int k_bin, int n) {
  for (int i = 0; i < n; ++i)
    if (bins[i] > k_bin) v[i] = 0.0f;
}

/* zero_vector_float + threshold_one (GAGA/gaga/kernels.cu:64-71,100-105) */
static void masked_copy(const float *src, float *dst, const int *bins, int k_bin, int n) {
  for (int i = 0; i < n; ++i) dst[i] = (bins[i] <= k_bin) ? src[i] : 0.0f;
}

/* ------------------------------------------------------------------ */
/* Solver workspace */
typedef struct {
  const gbo_op *op;
  int m, n, k;
  const float *y;
  float *x, *xt, *grad, *gp, *gpt, *resid, *ru;
  int *bins, *bins_prev, *counters;
  float prev[16];
} ws_t;

static void push16(float *a, float v) {
  for (int j = 0; j < 15; ++j) a[j] = a[j + 1];
  a[15] = v;
}

static float max_list(const float *a, int n) {
  float m = a[0];
  for (int j = 1; j < n; ++j)
    if (a[j] > m) m = a[j];
  return m;
}

/* resid = y - A x, via copy + saxpy(-1) as the reference does */
static void residual(ws_t *w, const float *x, float *resid, float *tmp) {
  gbo_A(w->op, x, tmp);
  for (int i = 0; i < w->m; ++i) resid[i] = fmaf(-1.0f, tmp[i], w->y[i]);
}

/* RestrictedSD_S_gen (GAGA/gaga/functions.cu:659-745) */
static float restricted_sd(ws_t *w, int k_bin) {
  int m = w->m, n = w->n;
  residual(w, w->x, w->resid, w->ru);
  push16(w->prev, nrm2f(w->resid, m));
  gbo_AT(w->op, w->resid, w->grad);
  masked_copy(w->grad, w->xt, w->bins, k_bin, n);
  gbo_A(w->op, w->xt, w->ru);
  float err = nrm2f(w->ru, m);
  float mu = nrm2f(w->xt, n);
  if (mu < 400.0f * err) {
    mu = mu / err;
    mu = mu * mu;
  } else {
    mu = 0.0f;
  }
  saxpy(n, mu, w->grad, w->x);
  return 2.0f * mu * gbo_max_magnitude(w->grad, n);
}

/* RestrictedCG_S_gen (GAGA/gaga/functions.cu:922-1000); prevCG receives ||y-Ax||^2 */
static void restricted_cg(ws_t *w, float *prevcg, float *mu, int k_bin) {
  int m = w->m, n = w->n;
  float alpha, beta;
  gbo_A(w->op, w->grad, w->resid);
  alpha = dotf(w->resid, w->resid, m);
  if (*mu < 1000.0f * alpha) alpha = *mu / alpha;
  else alpha = 0.0f;
  saxpy(n, alpha, w->grad, w->x);
  gbo_AT(w->op, w->resid, w->xt);
  gbo_threshold(w->xt, w->bins, k_bin, n);
  saxpy(n, -alpha, w->xt, w->gp);
  beta = *mu;
  *mu = dotf(w->gp, w->gp, n);
  if (*mu < 1000.0f * beta) beta = *mu / beta;
  else beta = 0.0f;
  sscal(n, beta, w->grad);
  saxpy(n, 1.0f, w->gp, w->grad);
  for (int j = 0; j < 15; ++j) prevcg[j] = prevcg[j + 1];
  residual(w, w->x, w->resid, w->ru);
  prevcg[15] = dotf(w->resid, w->resid, m);
}

/* RestrictedCGwithSupportEvolution_S_gen (GAGA/gaga/functions.cu:1004-1102) */
static float rcg_support_evolution(ws_t *w, float *mu, int beta_to_zero, int k_bin) {
  int m = w->m, n = w->n;
  float alpha, beta;
  residual(w, w->x, w->resid, w->ru);
  push16(w->prev, nrm2f(w->resid, m));
  gbo_AT(w->op, w->resid, w->grad);
  masked_copy(w->grad, w->xt, w->bins, k_bin, n);
  if (beta_to_zero == 1) {
    beta = 0.0f;
    *mu = dotf(w->xt, w->xt, n);
  } else {
    beta = *mu;
    *mu = dotf(w->xt, w->xt, n);
    if (*mu < 1000.0f * beta) beta = *mu / beta;
    else beta = 0.0f;
  }
  sscal(n, beta, w->gp);
  saxpy(n, 1.0f, w->grad, w->gp);
  masked_copy(w->gp, w->gpt, w->bins, k_bin, n);
  gbo_A(w->op, w->gpt, w->ru);
  alpha = dotf(w->ru, w->ru, m);
  if (*mu < 1000.0f * alpha) alpha = *mu / alpha;
  else alpha = 0.0f;
  saxpy(n, alpha, w->gp, w->x);
  return 2.0f * alpha * gbo_max_magnitude(w->gp, n);
}

/* UnrestrictedCG_S_gen (GAGA/gaga/functions.cu:1107-1220) */
static float unrestricted_cg(ws_t *w, float *mu, int beta_to_zero, int k_bin) {
  int m = w->m, n = w->n;
  gbo_A(w->op, w->x, w->ru);
  saxpy(m, -1.0f, w->y, w->ru);
  sscal(m, -1.0f, w->ru);
  push16(w->prev, nrm2f(w->ru, m));
  gbo_AT(w->op, w->ru, w->grad);
  masked_copy(w->grad, w->xt, w->bins, k_bin, n);
  gbo_A(w->op, w->gpt, w->resid);
  gbo_A(w->op, w->xt, w->ru);
  float beta;
  if (beta_to_zero == 1) {
    beta = 0.0f;
  } else {
    float bn = dotf(w->resid, w->ru, m);
    float bd = dotf(w->resid, w->resid, m);
    beta = -bn / bd;
  }
  sscal(n, beta, w->gp);
  saxpy(n, 1.0f, w->grad, w->gp);
  masked_copy(w->gp, w->gpt, w->bins, k_bin, n);
  sscal(m, beta, w->resid);
  saxpy(m, 1.0f, w->ru, w->resid);
  float an = dotf(w->gpt, w->xt, n);
  float ad = dotf(w->resid, w->resid, m);
  float alpha = an / ad;
  saxpy(n, alpha, w->gp, w->x);
  *mu = dotf(w->xt, w->xt, n);
  return 2.0f * alpha * gbo_max_magnitude(w->gp, n);
}

/* The stopping bookkeeping shared by the loops (e.g. GAGA/gaga/algorithms.cu:1398-1421). */
typedef struct {
  float err, err_start, tol, resid_diff, evol[16];
  int fail, cycle;
} stop_t;

static int keep_going(const stop_t *s, int iter, int maxiter) {
  return (s->err > s->tol) & (iter < maxiter) & (s->err < (100.0f * s->err_start)) &
         ((double)s->resid_diff > 0.01 * (double)s->tol) & (s->fail == 0) & (s->cycle != 0);
}

static void stop_update(stop_t *s, const float *prev, int iter, int fail_after) {
  for (int j = 0; j < 15; ++j) s->evol[j] = s->evol[j + 1];
  s->evol[15] = prev[14] - prev[15];
  s->resid_diff = max_list(s->evol, 16);
  for (int j = 0; j < 15; ++j)
    if ((prev[15] == prev[j]) && (iter > 4)) s->cycle = 0;
  if (iter > fail_after) {
    float root = 1.0f / 15.0f;
    float rate = prev[15] / prev[0];
    rate = powf(rate, root);
    if (rate > 0.999f) s->fail = 1;
  }
}

/* The timing variants' bookkeeping (GAGA/gaga/algorithms_timings.cu:610-624, 1509-1523):
 * no cycle test, and the rate test takes the 1/16-th root. */
static void stop_update_timing(stop_t *s, const float *prev, int iter, int fail_after) {
  for (int j = 0; j < 15; ++j) s->evol[j] = s->evol[j + 1];
  s->evol[15] = prev[14] - prev[15];
  s->resid_diff = max_list(s->evol, 16);
  if (iter > fail_after) {
    float rate = powf(prev[15] / prev[0], 1.0f / 16.0f);
    if (rate > 0.999f) s->fail = 1;
  }
}

static int cmp_float_asc(const void *a, const void *b) {
  const float x = *(const float *)a, y = *(const float *)b;
  return (x > y) - (x < y);
}

/* FindSupportSet_sort (GAGA/gaga/functions.cu:446-465): while the threshold T exceeds the
 * largest possible change, lower it by max_change and threshold (threshold_and_support,
 * kernels.cu:85-95: |v| < T -> v = 0, bin 2); otherwise T = the k-th largest |v| (thrust::sort
 * of |v| ascending, element n-k), every bin set to 1 (one_vector_int), then the threshold.
 * Bins of entries that survive a dynamic threshold keep their previous value. */
float gbo_find_support_set_sort(float *v, int *bins, float T, float max_change, float *buf, int n, int k) {
  if (T > max_change) {
    T = T - max_change;
  } else {
    for (int i = 0; i < n; ++i) buf[i] = fabsf(v[i]);
    qsort(buf, (size_t)n, sizeof(float), cmp_float_asc);
    T = buf[n - k];
    for (int i = 0; i < n; ++i) bins[i] = 1;
  }
  for (int i = 0; i < n; ++i)
    if (fabsf(v[i]) < T) {
      v[i] = 0.0f;
      bins[i] = 2;
    }
  return T;
}

/* The support step of NIHT_S_timings_* / HTP_S_timings_* (algorithms_timings.cu:566-599, 1392-1425)
 * after RestrictedSD returned max_change. */
static void timing_support_step(const gbo_opts *o, float *x, ws_t *w, gbo_bin_state *bs, float max_change,
                                float *max_value, float *slope, float *T, float *buf, int n, int k) {
  if (o->supp_flag < 2 && bs->min_val <= max_change) {
    *max_value = gbo_max_magnitude(x, n);
    *slope = ((float)(o->num_bins - 1) / *max_value);
  }
  if (o->supp_flag == 0 || o->supp_flag == 1) {
    /* supportFlag 1 passes max_value as maxChange: a binning every iteration */
    gbo_find_support_set(x, w->bins, w->counters, *slope, *max_value, o->supp_flag == 1 ? *max_value : max_change,
                         bs, n, k);
    gbo_threshold(x, w->bins, bs->k_bin, n);
  } else {
    bs->k_bin = 1;
    /* supportFlag 3 passes T as maxChange: T > T fails, a sort every iteration */
    *T = gbo_find_support_set_sort(x, w->bins, *T, o->supp_flag == 2 ? max_change : *T, buf, n, k);
  }
}

int gbo_solve(const gbo_op *op, const float *y, int k, const gbo_opts *o, float *x, gbo_info *info) {
#ifdef _OPENMP
  int saved_threads = omp_get_max_threads();
  if (o->threads > 0) omp_set_num_threads(o->threads);
#endif
  ws_t w;
  memset(&w, 0, sizeof(w));
  w.op = op; w.m = op->m; w.n = op->n; w.k = k; w.y = y; w.x = x;
  int m = op->m, n = op->n;
  int n_ucg = 0, n_rcg = 0; /* CGIHT's two step kinds, counted for the caller */
  w.xt = (float *)calloc((size_t)n, sizeof(float));
  w.grad = (float *)calloc((size_t)n, sizeof(float));
  w.gp = (float *)calloc((size_t)n, sizeof(float));
  w.gpt = (float *)calloc((size_t)n, sizeof(float));
  w.resid = (float *)calloc((size_t)m, sizeof(float));
  w.ru = (float *)calloc((size_t)m, sizeof(float));
  w.bins = (int *)calloc((size_t)n, sizeof(int));
  w.bins_prev = (int *)calloc((size_t)n, sizeof(int));
  w.counters = (int *)calloc((size_t)o->num_bins, sizeof(int));

  gbo_bin_state bs;
  bs.num_bins = o->num_bins;
  /* ThresholdSD / ThresholdCG start with alpha = 0, i.e. MaxBin = num_bins
   * (GAGA/gaga/algorithms.cu:800-802,1838-1840) */
  bs.alpha = (o->alg == GBO_HT_SD || o->alg == GBO_HT_CG) ? 0.0f : 0.25f;
  /* the timing variants take alpha from the options (gaga_gen.cu:329, algorithms_timings.cu:477) */
  const int timing = o->timing && (o->alg == GBO_NIHT || o->alg == GBO_HTP);
  if (timing) bs.alpha = o->alpha;
  bs.max_bin = (int)((float)o->num_bins * (1.0f - bs.alpha));
  bs.min_val = 0.0f;
  bs.k_bin = 0;
  bs.sum = 0;
  int iter = 0;
  float mu = 0.0f;

  stop_t s;
  memcpy(w.resid, y, sizeof(float) * m);
  s.err = nrm2f(w.resid, m);
  s.err_start = s.err;
  s.tol = o->tol;
  s.resid_diff = 1.0f;
  for (int j = 0; j < 16; ++j) { w.prev[j] = 0.0f; s.evol[j] = 1.0f; }
  s.fail = 0;
  s.cycle = 1;

  float max_value, slope;
  if (o->alg == GBO_IHT) {
    /* IHT_S_gen (GAGA/gaga/algorithms.cu:347-478): x starts at 0; the bins keep the scale
     * of A^T y for the whole solve; fixed step mu = 0.65 (gaga_gen.cu, case 2) */
    const float mu_iht = 0.65f;
    memset(x, 0, sizeof(float) * n);
    gbo_AT(op, w.resid, w.grad);
    max_value = gbo_max_magnitude(w.grad, n);
    slope = ((float)(o->num_bins - 1) / max_value);
    while ((s.err > s.tol) & (iter < o->maxiter) & (s.err < (100.0f * s.err_start)) &
           ((double)s.resid_diff > 0.01 * (double)s.tol) & (s.fail == 0)) {
      gbo_AT(op, w.resid, w.grad);
      float max_change = 2.0f * mu_iht * gbo_max_magnitude(w.grad, n);
      saxpy(n, mu_iht, w.grad, x);
      gbo_find_support_set(x, w.bins, w.counters, slope, max_value, max_change, &bs, n, k);
      gbo_threshold(x, w.bins, bs.k_bin, n);
      residual(&w, x, w.resid, w.ru);
      s.err = nrm2f(w.resid, m);
      push16(w.prev, s.err);
      for (int j = 0; j < 15; ++j) s.evol[j] = s.evol[j + 1];
      s.evol[15] = w.prev[14] - w.prev[15];
      s.resid_diff = max_list(s.evol, 16);
      if (iter > 749) {
        float rate = powf(w.prev[15] / w.prev[0], 1.0f / 15.0f);
        if (rate > 0.999f) s.fail = 1;
      }
      iter++;
    }
    goto done;
  }

  /* Set the linear bins: x = H_k(A^T y) */
  gbo_AT(op, y, x);
  max_value = gbo_max_magnitude(x, n);
  slope = ((float)(o->num_bins - 1) / max_value);
  /* HTP (and NIHT_dct) pass max_value as maxChange to force binning; with
   * minVal = 0 every algorithm bins here. */
  gbo_find_support_set(x, w.bins, w.counters, slope, max_value,
                       (o->alg == GBO_HTP || o->alg == GBO_CSMPSP || o->alg == GBO_CGIHT_PROJ) ? max_value : 1.0f,
                       &bs, n, k);
  gbo_threshold(x, w.bins, bs.k_bin, n);

  if (o->alg == GBO_FIHT || o->alg == GBO_ALPS) {
    /* FIHT_S_gen / ALPS_S_gen (GAGA/gaga/algorithms.cu:5430-5706, 6263-6534) with
     * RestrictedFIHT_S_gen / RestrictedALPS_S_gen (GAGA/gaga/functions.cu:1668-1843) */
    float *x_prev = w.gp, *extra = w.gpt, *vt = w.xt;
    /* the step-size guards are 1000 x the denominator in the _dct forms
     * (functions.cu:1867,1918,1948,2022; algorithms.cu:5912,6741) and 400 x in the _gen
     * and _smv forms (functions.cu:1682,1733,1765,1840,2051,2102,2132,2206;
     * algorithms.cu:5633,6188,6463,7022) */
    const float guard = op->kind == GBO_OP_DCT ? 1000.0f : 400.0f;
    float *Apv = (float *)calloc((size_t)m, sizeof(float));
    float *Aex = (float *)calloc((size_t)m, sizeof(float));
    float *ru = w.ru;
    /* one more iteration: x = H_k(x + A^T (y - A x)) */
    gbo_A(op, x, ru);
    saxpy(m, -1.0f, ru, w.resid);
    s.err = nrm2f(w.resid, m);
    w.prev[15] = s.err;
    gbo_AT(op, w.resid, w.grad);
    memcpy(x_prev, x, sizeof(float) * n);
    memcpy(Apv, ru, sizeof(float) * m);
    saxpy(n, 1.0f, w.grad, x);
    bs.min_val = 0.0f;
    max_value = gbo_max_magnitude(x, n);
    slope = ((float)(o->num_bins - 1) / max_value);
    gbo_find_support_set(x, w.bins, w.counters, slope, max_value, 1.0f, &bs, n, k);
    gbo_threshold(x, w.bins, bs.k_bin, n);
    gbo_A(op, x, ru);
    memcpy(w.resid, y, sizeof(float) * m);
    saxpy(m, -1.0f, ru, w.resid);
    s.err = nrm2f(w.resid, m);
    push16(w.prev, s.err);
    for (int j = 0; j < 15; ++j) s.evol[j] = s.evol[j + 1];
    s.evol[15] = w.prev[14] - w.prev[15];
    s.resid_diff = max_list(s.evol, 16);
    while (keep_going(&s, iter, o->maxiter)) {
      /* extrapolated point v = x + tau (x_prev - x), tau from the residual line search */
      saxpy(m, -1.0f, ru, Apv);
      float tau = dotf(w.resid, Apv, m), tmp = dotf(Apv, Apv, m);
      if (fabsf(tau) < guard * fabsf(tmp)) tau = tau / tmp;
      else tau = 0.0f;
      memcpy(extra, x, sizeof(float) * n);
      saxpy(n, -1.0f, x, x_prev);
      saxpy(n, tau, x_prev, extra);
      memcpy(Aex, ru, sizeof(float) * m);
      saxpy(m, tau, Apv, Aex);
      memcpy(w.resid, y, sizeof(float) * m);
      saxpy(m, -1.0f, Aex, w.resid);
      gbo_AT(op, w.resid, w.grad);
      memcpy(x_prev, x, sizeof(float) * n);
      memcpy(Apv, ru, sizeof(float) * m);
      if (o->alg == GBO_FIHT) {
        /* threshold_two: the gradient on the support of v */
        for (int i = 0; i < n; ++i) vt[i] = extra[i] == 0.0f ? 0.0f : w.grad[i];
      } else {
        /* threshold_three, a local FindSupportSet on it (the bin state is passed by value,
         * so alpha/MaxBin/minVal/k_bin changes stay local), threshold, threshold_four */
        for (int i = 0; i < n; ++i) vt[i] = extra[i] == 0.0f ? w.grad[i] : 0.0f;
        gbo_bin_state local = bs;
        local.min_val = 0.0f;
        float mv = gbo_max_magnitude(vt, n);
        float sl = ((float)(o->num_bins - 1) / mv);
        gbo_find_support_set(vt, w.bins, w.counters, sl, mv, 1.0f, &local, n, k);
        bs.sum = local.sum;
        gbo_threshold(vt, w.bins, local.k_bin, n);
        for (int i = 0; i < n; ++i)
          if (extra[i] != 0.0f) vt[i] = w.grad[i];
      }
      gbo_A(op, vt, Aex);
      float mu2 = dotf(vt, vt, n);
      tmp = dotf(Aex, Aex, m);
      if (mu2 < guard * tmp) mu2 = mu2 / tmp;
      else mu2 = 1.0f;
      memcpy(x, extra, sizeof(float) * n);
      saxpy(n, mu2, w.grad, x);
      /* new support */
      bs.min_val = 0.0f;
      max_value = gbo_max_magnitude(x, n);
      slope = ((float)(o->num_bins - 1) / max_value);
      gbo_find_support_set(x, w.bins, w.counters, slope, max_value, 1.0f, &bs, n, k);
      gbo_threshold(x, w.bins, bs.k_bin, n);
      gbo_A(op, x, ru);
      memcpy(w.resid, y, sizeof(float) * m);
      saxpy(m, -1.0f, ru, w.resid);
      /* steepest descent on the support */
      gbo_AT(op, w.resid, w.grad);
      masked_copy(w.grad, vt, w.bins, bs.k_bin, n);
      gbo_A(op, vt, Aex);
      mu2 = dotf(vt, vt, n);
      tmp = dotf(Aex, Aex, m);
      if (mu2 < guard * tmp) mu2 = mu2 / tmp;
      else mu2 = 1.0f;
      saxpy(n, mu2, vt, x);
      saxpy(m, mu2, Aex, ru);
      memcpy(w.resid, y, sizeof(float) * m);
      saxpy(m, -1.0f, ru, w.resid);
      s.err = nrm2f(w.resid, m);
      push16(w.prev, s.err);
      stop_update(&s, w.prev, iter, 749);
      iter++;
    }
    free(Apv);
    free(Aex);
    goto done;
  }
  if (o->alg == GBO_CGIHT_PROJ) {
    /* CGIHTprojected_S_gen (GAGA/gaga/algorithms.cu:4486-4690) */
    float *vt = w.xt, *p = w.gp, *gpt = w.gpt, *ru = w.ru;
    float *Ap = (float *)calloc((size_t)m, sizeof(float));
    float *diff = (float *)calloc((size_t)n, sizeof(float));
    gbo_A(op, x, ru);
    saxpy(m, -1.0f, ru, w.resid);
    s.err = nrm2f(w.resid, m);
    w.prev[15] = s.err;
    gbo_AT(op, w.resid, w.grad);
    masked_copy(w.grad, vt, w.bins, bs.k_bin, n);
    gbo_A(op, vt, ru);
    for (int j = 0; j < 15; ++j) s.evol[j] = s.evol[j + 1];
    s.evol[15] = w.prev[14] - w.prev[15];
    int supp_change = 1;
    while (keep_going(&s, iter, o->maxiter)) {
      float tmp;
      if (supp_change) {
        mu = dotf(vt, vt, n);
        tmp = dotf(ru, ru, m);
        if (mu < 400.0f * tmp) mu = mu / tmp;
        else mu = 1.0f;
        saxpy(n, mu, w.grad, x);
        bs.min_val = 0.0f;
        max_value = gbo_max_magnitude(x, n);
        slope = ((float)(o->num_bins - 1) / max_value);
        gbo_find_support_set(x, w.bins, w.counters, slope, max_value, 1.0f, &bs, n, k);
        gbo_threshold(x, w.bins, bs.k_bin, n);
        gbo_A(op, x, ru);
        memcpy(w.resid, y, sizeof(float) * m);
        saxpy(m, -1.0f, ru, w.resid);
        gbo_AT(op, w.resid, w.grad);
        masked_copy(w.grad, vt, w.bins, bs.k_bin, n);
        gbo_A(op, vt, ru);
        memcpy(p, vt, sizeof(float) * n);
        memcpy(Ap, ru, sizeof(float) * m);
      } else {
        mu = dotf(vt, vt, n);
        tmp = dotf(Ap, Ap, m);
        if (mu < 400.0f * tmp) mu = mu / tmp;
        else mu = 1.0f;
        saxpy(n, mu, p, x);
        gbo_A(op, x, ru);
        memcpy(w.resid, y, sizeof(float) * m);
        saxpy(m, -1.0f, ru, w.resid);
        memcpy(gpt, vt, sizeof(float) * n);
        gbo_AT(op, w.resid, w.grad);
        masked_copy(w.grad, vt, w.bins, bs.k_bin, n);
        gbo_A(op, vt, ru);
        float beta = dotf(vt, vt, n);
        tmp = dotf(gpt, gpt, n);
        if (beta < 400.0f * tmp) beta = beta / tmp;
        else beta = 0.0f;
        sscal(n, beta, p);
        saxpy(n, 1.0f, vt, p);
        sscal(m, beta, Ap);
        saxpy(m, 1.0f, ru, Ap);
      }
      memcpy(diff, w.grad, sizeof(float) * n);
      saxpy(n, -1.0f, p, diff);
      float pf = nrm2f(diff, n);
      tmp = nrm2f(vt, n);
      if (pf < 1000.0f * tmp) {
        pf = pf / tmp;
        supp_change = pf > o->proj_frac_tol ? 1 : 0;
      } else {
        supp_change = 1;
      }
      s.err = nrm2f(w.resid, m);
      push16(w.prev, s.err);
      stop_update(&s, w.prev, iter, 749);
      iter++;
    }
    free(Ap);
    free(diff);
    goto done;
  }

  if (o->alg == GBO_CSMPSP) {
    /* CSMPSP_S_gen (GAGA/gaga/algorithms.cu:3372-3688), with the two places where the
     * reference's operator forms differ: _gen and _smv reset minVal before both forced
     * binnings of the loop (algorithms.cu:3540,3606; 3225,3291), _dct does not, so its
     * FindSupportSet may skip the binning and keep the previous bins and k-th bin
     * (algorithms.cu:2907,2973); the loop's CG projection has no stall test in _gen
     * (algorithms.cu:3600) and has one in _dct and _smv (algorithms.cu:2963,3285). */
    const int reset_min = op->kind != GBO_OP_DCT;
    const int loop_stall = op->kind != GBO_OP_DENSE;
    int k_bin_grad = 0;
    const float tol_cg = s.tol * s.tol;
    const float tol2 = 10.0f * tol_cg;
    float prevcg[16], evolcg[16], errcg, diffcg;
    int itcg;
    /* one CG projection on the support of x (stall test on the CG history when `stall`) */
#define CSMPSP_PROJECT(stall)                                                  \
    do {                                                                       \
      itcg = 0;                                                                \
      for (int j = 0; j < 16; ++j) { prevcg[j] = 0.0f; evolcg[j] = 1.0f; }    \
      diffcg = 1.0f;                                                           \
      prevcg[15] = w.prev[15];                                                 \
      residual(&w, x, w.resid, w.ru);                                          \
      gbo_AT(op, w.resid, w.grad);                                             \
      gbo_threshold(w.grad, w.bins, bs.k_bin, n);                              \
      memcpy(w.gp, w.grad, sizeof(float) * n);                                 \
      mu = dotf(w.gp, w.gp, n);                                                \
      errcg = dotf(w.resid, w.resid, m);                                       \
      prevcg[15] = errcg;                                                      \
      while ((errcg > tol_cg) & (itcg < 15) & (diffcg > tol2)) {               \
        restricted_cg(&w, prevcg, &mu, bs.k_bin);                              \
        errcg = prevcg[15];                                                    \
        itcg++;                                                                \
        for (int j = 0; j < 15; ++j) evolcg[j] = evolcg[j + 1];                \
        evolcg[15] = prevcg[14] - prevcg[15];                                  \
        diffcg = (stall) ? max_list(evolcg, 16) : 10.0f;                       \
      }                                                                        \
    } while (0)
    CSMPSP_PROJECT(1);
    s.err = sqrtf(errcg);
    w.prev[15] = s.err;
    iter++;  /* the initial projection counts as an iteration */
    int *bins_grad = w.bins_prev;
    while (keep_going(&s, iter, o->maxiter)) {
      gbo_AT(op, w.resid, w.grad);
      max_value = gbo_max_magnitude(w.grad, n);
      if (reset_min) bs.min_val = 0.0f;
      slope = ((float)(o->num_bins - 1) / max_value);
      int k_bin_x = bs.k_bin;
      bs.k_bin = k_bin_grad;
      gbo_find_support_set(w.grad, bins_grad, w.counters, slope, max_value, max_value, &bs, n, k);
      k_bin_grad = bs.k_bin;
      bs.k_bin = k_bin_x;
      /* joinSupports (GAGA/gaga/kernels.cu:162-172) */
      for (int i = 0; i < n; ++i)
        if (bins_grad[i] <= k_bin_grad && w.bins[i] > bs.k_bin) w.bins[i] = bs.k_bin;
      CSMPSP_PROJECT(loop_stall);
      max_value = gbo_max_magnitude(x, n);
      if (reset_min) bs.min_val = 0.0f;
      slope = ((float)(o->num_bins - 1) / max_value);
      gbo_find_support_set(x, w.bins, w.counters, slope, max_value, max_value, &bs, n, k);
      gbo_threshold(x, w.bins, bs.k_bin, n);
      residual(&w, x, w.resid, w.ru);
      s.err = nrm2f(w.resid, m);
      push16(w.prev, s.err);
      stop_update(&s, w.prev, iter, 125);
      iter++;
    }
#undef CSMPSP_PROJECT
  } else if (o->alg == GBO_HT_SD) {
    /* HT_SD_S_gen (GAGA/gaga/algorithms.cu:785-906): steepest descent on the fixed support */
    const float tol2 = (float)(0.1 * (double)s.tol);
    while ((s.err > s.tol) & (iter < o->maxiter) & (s.resid_diff > tol2)) {
      restricted_sd(&w, bs.k_bin);
      gbo_threshold(x, w.bins, bs.k_bin, n);
      s.err = w.prev[15];
      for (int j = 0; j < 15; ++j) s.evol[j] = s.evol[j + 1];
      s.evol[15] = w.prev[14] - w.prev[15];
      s.resid_diff = max_list(s.evol, 16);
      iter++;
    }
  } else if (o->alg == GBO_HT_CG) {
    /* HT_CG_S_gen (GAGA/gaga/algorithms.cu:1826-1990): CG on the fixed support, the
     * residual history in squared norms */
    const float tol_cg = s.tol * s.tol;
    const float tol2 = 10.0f * tol_cg;
    residual(&w, x, w.resid, w.ru);
    gbo_AT(op, w.resid, w.grad);
    gbo_threshold(w.grad, w.bins, bs.k_bin, n);
    memcpy(w.gp, w.grad, sizeof(float) * n);
    mu = dotf(w.gp, w.gp, n);
    s.err = dotf(w.resid, w.resid, m);
    w.prev[15] = s.err;
    while ((s.err > tol_cg) & (iter < o->maxiter) & (s.resid_diff > tol2)) {
      restricted_cg(&w, w.prev, &mu, bs.k_bin);
      s.err = w.prev[15];
      for (int j = 0; j < 15; ++j) s.evol[j] = s.evol[j + 1];
      s.evol[15] = w.prev[14] - w.prev[15];
      s.resid_diff = max_list(s.evol, 16);
      iter++;
    }
  } else if (o->alg == GBO_NIHT && timing) {
    /* NIHT_S_timings_gen (GAGA/gaga/algorithms_timings.cu:453-650; _dct 35-240, _smv 246-450) */
    float T = 0.0f;
    float *buf = (float *)malloc(sizeof(float) * (size_t)n);
    while (keep_going(&s, iter, o->maxiter)) {
      float max_change = restricted_sd(&w, bs.k_bin);
      timing_support_step(o, x, &w, &bs, max_change, &max_value, &slope, &T, buf, n, k);
      s.err = w.prev[15];
      stop_update_timing(&s, w.prev, iter, 749);
      iter++;
    }
    free(buf);
  } else if (o->alg == GBO_NIHT) {
    /* NIHT_S_gen (GAGA/gaga/algorithms.cu:1274-1441) */
    while (keep_going(&s, iter, o->maxiter)) {
      float max_change = restricted_sd(&w, bs.k_bin);
      if (bs.min_val <= max_change) {
        max_value = gbo_max_magnitude(x, n);
        slope = ((float)(o->num_bins - 1) / max_value);
      }
      gbo_find_support_set(x, w.bins, w.counters, slope, max_value, max_change, &bs, n, k);
      gbo_threshold(x, w.bins, bs.k_bin, n);
      s.err = w.prev[15];
      stop_update(&s, w.prev, iter, 749);
      iter++;
    }
  } else if (o->alg == GBO_HTP) {
    /* HTP_S_gen (GAGA/gaga/algorithms.cu:2491-2716); with timing on, HTP_S_timings_gen
     * (algorithms_timings.cu:1266-1560): the support step of supportFlag, no cycle test,
     * the rate test's 1/16-th root */
    float tol_cg = s.tol * s.tol;
    float tol2 = 10.0f * tol_cg;
    float T = 0.0f;
    float *buf = timing ? (float *)malloc(sizeof(float) * (size_t)n) : NULL;
    while (keep_going(&s, iter, o->maxiter)) {
      float max_change = restricted_sd(&w, bs.k_bin);
      if (timing) {
        timing_support_step(o, x, &w, &bs, max_change, &max_value, &slope, &T, buf, n, k);
      } else {
        if (bs.min_val <= max_change) {
          max_value = gbo_max_magnitude(x, n);
          slope = ((float)(o->num_bins - 1) / max_value);
        }
        gbo_find_support_set(x, w.bins, w.counters, slope, max_value, max_change, &bs, n, k);
        gbo_threshold(x, w.bins, bs.k_bin, n);
      }
      float prevcg[16], evolcg[16];
      for (int j = 0; j < 16; ++j) { prevcg[j] = 0.0f; evolcg[j] = 1.0f; }
      float diffcg = 1.0f;
      prevcg[15] = w.prev[15];
      residual(&w, x, w.resid, w.ru);
      gbo_AT(op, w.resid, w.grad);
      gbo_threshold(w.grad, w.bins, bs.k_bin, n);
      memcpy(w.gp, w.grad, sizeof(float) * n);
      mu = dotf(w.gp, w.gp, n);
      float errcg = dotf(w.resid, w.resid, m);
      prevcg[15] = errcg;
      int itcg = 0;
      while ((errcg > tol_cg) & (itcg < 15) & (diffcg > tol2)) {
        restricted_cg(&w, prevcg, &mu, bs.k_bin);
        errcg = prevcg[15];
        itcg++;
        for (int j = 0; j < 15; ++j) evolcg[j] = evolcg[j + 1];
        evolcg[15] = prevcg[14] - prevcg[15];
        diffcg = max_list(evolcg, 16);
      }
      s.err = sqrtf(errcg);
      push16(w.prev, s.err);
      if (timing) stop_update_timing(&s, w.prev, iter, 125);
      else stop_update(&s, w.prev, iter, 125);
      iter++;
    }
    free(buf);
  } else if (o->alg == GBO_CGIHT) {
    /* CGIHT_S_gen (GAGA/gaga/algorithms.cu:3689-3942) */
    residual(&w, x, w.resid, w.ru);
    s.err = nrm2f(w.resid, m);
    w.prev[15] = s.err;
    gbo_AT(op, w.resid, w.gp);
    masked_copy(w.gp, w.gpt, w.bins, bs.k_bin, n);
    for (int j = 0; j < 15; ++j) s.evol[j] = s.evol[j + 1];
    s.evol[15] = w.prev[14] - w.prev[15];
    int beta_to_zero = 1, supp_change = 1, k_bin_prev = 0;
    while (keep_going(&s, iter, o->maxiter)) {
      float max_change;
      const int ucg = !o->restart && supp_change;
      if (ucg) max_change = unrestricted_cg(&w, &mu, beta_to_zero, bs.k_bin);
      else max_change = rcg_support_evolution(&w, &mu, beta_to_zero, bs.k_bin);
      n_ucg += ucg;
      n_rcg += !ucg;
      beta_to_zero = 0;
      if (bs.min_val <= max_change) {
        max_value = gbo_max_magnitude(x, n);
        slope = ((float)(o->num_bins - 1) / max_value);
        memcpy(w.bins_prev, w.bins, sizeof(int) * n);
        k_bin_prev = bs.k_bin;
        gbo_find_support_set(x, w.bins, w.counters, slope, max_value, max_change, &bs, n, k);
        /* checkSupportEvolution (GAGA/gaga/kernels.cu:178-193), race-free form */
        int changed = 0;
        for (int i = 0; i < n; ++i)
          if (w.bins_prev[i] <= k_bin_prev && w.bins[i] > bs.k_bin) changed = 1;
        supp_change = changed;
        if (supp_change) {
          if (o->restart) beta_to_zero = 1;
          else masked_copy(w.gp, w.gpt, w.bins, bs.k_bin, n);
        }
      } else {
        supp_change = 0;
        bs.min_val = bs.min_val - max_change;
      }
      gbo_threshold(x, w.bins, bs.k_bin, n);
      s.err = w.prev[15];
      stop_update(&s, w.prev, iter, 749);
      iter++;
    }
  }

done:
  if (info) {
    info->iter = iter;
    info->sum = bs.sum;
    info->k_bin = bs.k_bin;
    info->ucg_steps = n_ucg;
    info->rcg_steps = n_rcg;
    memcpy(info->resid_prev, w.prev, sizeof(w.prev));
    /* given-data convRate (GAGA/gaga/gaga_gen.cu:733-741) */
    int temp = iter < 16 ? iter : 16;
    if (temp > 0) {
      float root = 1.0f / (float)temp;
      temp = 16 - temp;
      info->conv_rate = powf(w.prev[15] / w.prev[temp], root);
    } else {
      info->conv_rate = 0.0f;
    }
  }
  free(w.xt); free(w.grad); free(w.gp); free(w.gpt); free(w.resid); free(w.ru);
  free(w.bins); free(w.bins_prev); free(w.counters);
#ifdef _OPENMP
  omp_set_num_threads(saved_threads);
#endif
  return 0;
}

/* ------------------------------------------------------------------ */
/* Expander l0 decoding */

/* cuda_compute_scores_l0 (GAGA/gaga/expander/kernels.cu:353-388); the score is
 * kept as a float counter exactly as the reference kernel does. */
void gbo_l0_scores(const float *res, float *x, float *updates, const int *rows, int n, int d,
                   int thresh, int shift, int *found) {
  const float EPS = 0.000001f;
  for (int j = 0; j < n; ++j) {
    int idx = d * j;
    float score = 0.0f;
    float omega = res[rows[idx + shift]];
    updates[j] = 0.0f;
    if (fabsf(omega) > EPS) {
      for (int i = 0; i < d; ++i) {
        if (fabsf(res[rows[idx + i]] - omega) <= EPS) score += 1.0f;
        if (fabsf(res[rows[idx + i]]) <= EPS) score -= 1.0f;
      }
      if (score > (float)thresh) {
        *found = 1;
        x[j] = x[j] + omega;
        updates[j] = omega;
      }
    }
  }
}

/* cuda_update_residual (GAGA/gaga/expander/kernels.cu:3-14); updates applied in
 * column order */
void gbo_l0_update_residual(float *res, const int *rows, const float *updates, int n, int d) {
  for (int j = 0; j < n; ++j) {
    if (fabsf(updates[j]) > 0.0f) {
      float u = -updates[j];
      for (int i = 0; i < d; ++i) res[rows[j * d + i]] += u;
    }
  }
}

/* cuda_compute_scores_lddsr (GAGA/gaga/expander/kernels.cu:309-345): only matching rows
 * count, a candidate needs more than d/2 of them */
static void lddsr_scores(const float *res, float *x, float *updates, const int *rows, int n, int d, int shift,
                         int *found) {
  const float EPS = 0.000001f;
  const float thresh = ((float)d) / 2;
  for (int j = 0; j < n; ++j) {
    int idx = d * j;
    float score = 0.0f;
    float omega = res[rows[idx + shift]];
    updates[j] = 0.0f;
    if (fabsf(omega) > EPS) {
      for (int i = 0; i < d; ++i)
        if (fabsf(res[rows[idx + i]] - omega) <= EPS) score += 1.0f;
      if (score > thresh) {
        *found = 1;
        x[j] = x[j] + omega;
        updates[j] = omega;
      }
    }
  }
}

/* parallel_l0 (GAGA/gaga/expander/parallel_l0.cu:9-151); o->alg may also select
 * parallel_lddsr (parallel_lddsr.cu: lddsr scores) or parallel_l0_swipe
 * (parallel_l0_swipe.cu: the threshold starts at d - 1 and drops by one whenever no
 * column qualifies; such a pass leaves the residual history alone) */
int gbo_parallel_l0(const gbo_op *op, const float *y, const gbo_opts *o, float *x, float *res,
                    float *res_record, gbo_info *info) {
  int m = op->m, n = op->n, d = op->d;
  float *ax = (float *)malloc(sizeof(float) * m);
  float *upd = (float *)calloc((size_t)n, sizeof(float));
  gbo_A(op, x, ax);
  for (int i = 0; i < m; ++i) res[i] = fmaf(-1.0f, ax[i], y[i]);
  float norm = nrm2f(res, m), norm0 = norm;
  if (res_record) res_record[0] = norm;
  int L = 2 * d;
  float *cyc = (float *)calloc((size_t)L, sizeof(float));
  float *prev = (float *)calloc((size_t)L, sizeof(float));
  float *evol = (float *)malloc(sizeof(float) * L);
  for (int i = 0; i < L; ++i) evol[i] = 1.0f;
  float diff = 1.0f;
  int iter = 0, cycling = 0, found = 1;
  const int swipe = o->alg == GBO_PARALLEL_L0_SWIPE;
  int thresh = swipe ? d - 1 : o->l0_thresh;
  while ((iter < o->maxiter) & (norm > o->tol) & (norm < (100.0f * norm0)) & ((double)diff > 0.000001) &
         (cycling == 0) & (found == 1) & (!swipe || thresh > 0)) {
    int offset = iter % d;
    found = 0;
    if (o->alg == GBO_PARALLEL_LDDSR) lddsr_scores(res, x, upd, op->smv_rows, n, d, offset, &found);
    else gbo_l0_scores(res, x, upd, op->smv_rows, n, d, thresh, offset, &found);
    if (swipe && found == 0 && thresh > 0) {
      thresh--;
      found = 1;
      iter = iter + 1;
      if (res_record) res_record[iter] = norm;
      continue;
    }
    gbo_l0_update_residual(res, op->smv_rows, upd, n, d);
    norm = nrm2f(res, m);
    for (int i = 0; i < L - 1; ++i) prev[i] = prev[i + 1];
    prev[L - 1] = norm;
    for (int i = 0; i < L - 1; ++i) evol[i] = evol[i + 1];
    evol[L - 1] = prev[L - 2] - prev[L - 1];
    diff = max_list(evol, L);
    for (int i = 0; i < L - 1; ++i) cyc[i] = cyc[i + 1];
    cyc[L - 1] = norm;
    if (iter > L) {
      cycling = 1;
      for (int i = 3; i < L; i += 2) cycling = cycling * (cyc[i] == cyc[i - 2]);
    }
    iter = iter + 1;
    if (res_record) res_record[iter] = norm;
  }
  if (info) {
    memset(info, 0, sizeof(*info));
    info->iter = iter;
    /* gaga_smv.cu:1013-1020: the last <=16 records become residNorm_prev */
    if (res_record)
      for (int j = 0; j < (iter < 16 ? iter : 16); ++j) info->resid_prev[15 - j] = res_record[iter - j];
  }
  free(ax); free(upd); free(cyc); free(prev); free(evol);
  return 0;
}

/* H_k of the expander decoders (GAGA/gaga/expander/functions.cu:103-144): a fresh binning
 * (alpha 0.25, MaxBin = num_bins, minVal 0, maxChange = 2 max|v|), Threshold, then
 * ThresholdK trims the support to exactly K entries by zeroing entries of the k-th bin.
 * The reference picks those entries by atomic order; here they are the first ones in
 * index order. */
static int expander_hk(float *v, int K, int n, int num_bins, int *bins, int *counters) {
  float mx = gbo_max_magnitude(v, n);
  float slope = ((float)(num_bins - 1) / mx);
  gbo_bin_state bs;
  bs.num_bins = num_bins;
  bs.alpha = 0.25f;
  bs.max_bin = num_bins;
  bs.min_val = 0.0f;
  bs.k_bin = 0;
  bs.sum = 0;
  int sum = gbo_find_support_set(v, bins, counters, slope, mx, 2.0f * mx, &bs, n, K);
  gbo_threshold(v, bins, bs.k_bin, n);
  int supp = 0;
  for (int i = 0; i < n; ++i) supp += v[i] != 0.0f;
  int offset = supp - K;
  for (int i = 0; i < n && offset > 0; ++i)
    if (bins[i] == bs.k_bin) {
      v[i] = 0.0f;
      offset--;
    }
  return sum;
}

/* cuda_compute_scores_smp (GAGA/gaga/expander/kernels.cu:79-104): the median of the
 * residual over each column's d rows */
static void smp_scores(const float *res, const int *rows, int n, int d, float *u) {
  float buf[64];
  for (int j = 0; j < n; ++j) {
    for (int i = 0; i < d; ++i) buf[i] = res[rows[(size_t)j * d + i]];
    for (int i = 0; i < d; ++i)
      for (int q = 0; q < d - 1; ++q)
        if (buf[q] > buf[q + 1]) {
          float t = buf[q + 1];
          buf[q + 1] = buf[q];
          buf[q] = t;
        }
    u[j] = (d % 2) == 0 ? (buf[d / 2 - 1] + buf[d / 2]) / 2 : buf[(d - 1) / 2];
  }
}

int gbo_smp(const gbo_op *op, const float *y, int k, const gbo_opts *o, float *x, float *res, float *res_record,
            gbo_info *info) {
  int m = op->m, n = op->n, d = op->d;
  float *ax = (float *)malloc(sizeof(float) * m);
  float *u = (float *)calloc((size_t)n, sizeof(float));
  int *bins = (int *)calloc((size_t)n, sizeof(int));
  int *counters = (int *)calloc((size_t)o->num_bins, sizeof(int));
  gbo_A(op, x, ax);
  for (int i = 0; i < m; ++i) res[i] = fmaf(-1.0f, ax[i], y[i]);
  float err = nrm2f(res, m), err_start = err;
  if (res_record) res_record[0] = err;
  float prev[16], evol[16], diff = 1.0f;
  for (int i = 0; i < 16; ++i) { prev[i] = 0.0f; evol[i] = 1.0f; }
  int iter = 0, fail = 0;
  while ((iter < o->maxiter) & (err > o->tol) & (err < (100.0f * err_start)) & ((double)diff > 0.01 * (double)o->tol) &
         (fail == 0)) {
    smp_scores(res, op->smv_rows, n, d, u);
    expander_hk(u, 2 * k, n, o->num_bins, bins, counters);
    saxpy(n, 1.0f, u, x);
    expander_hk(x, k, n, o->num_bins, bins, counters);
    gbo_A(op, x, ax);
    for (int i = 0; i < m; ++i) res[i] = fmaf(-1.0f, ax[i], y[i]);
    err = nrm2f(res, m);
    push16(prev, err);
    for (int i = 0; i < 15; ++i) evol[i] = evol[i + 1];
    evol[15] = prev[14] - prev[15];
    diff = max_list(evol, 16);
    if (iter > ((int)(0.4 * o->maxiter))) {
      float rate = powf(prev[15] / prev[0], 1.0f / 15.0f);
      if (rate > 0.999f) fail = 1;
    }
    iter = iter + 1;
    if (res_record) res_record[iter] = err;
  }
  if (info) {
    memset(info, 0, sizeof(*info));
    info->iter = iter;
    memcpy(info->resid_prev, prev, sizeof(prev));
  }
  free(ax); free(u); free(bins); free(counters);
  return 0;
}

/* Node score of ssmp (median) or er (mode and its run length), cuda_compute_scores_ssmp /
 * cuda_compute_scores_er (GAGA/gaga/expander/kernels.cu:115-145, 195-245): bubble sort of
 * the node's d residual entries; ssmp: median, score |median|; er: the value before the first
 * longest run of neighbours within 1e-7, score its run length (0 if |mode| <= 1e-7). */
static void seq_score(int er, const float *res, const int *rows_j, int d, float *upd, float *score) {
  float b[64];
  for (int i = 0; i < d; ++i) b[i] = res[rows_j[i]];
  for (int i = 0; i < d; ++i)
    for (int q = 0; q < d - 1; ++q)
      if (b[q] > b[q + 1]) {
        float t = b[q + 1];
        b[q + 1] = b[q];
        b[q] = t;
      }
  if (!er) {
    float z = (d % 2) == 0 ? (b[d / 2 - 1] + b[d / 2]) / 2 : b[(d - 1) / 2];
    *upd = z;
    *score = fabsf(z);
  } else {
    const float eps = 0.0000001f;
    float mode = b[0], count = 1.0f, count_mode = 1.0f;
    for (int i = 1; i < d; ++i) {
      if (fabsf(b[i] - b[i - 1]) <= eps) {
        count = count + 1.0f;
        if (count > count_mode) {
          count_mode = count;
          mode = b[i - 1];
        }
      } else {
        count = 1.0f;
      }
    }
    *upd = mode;
    *score = fabsf(mode) > eps ? count_mode : 0.0f;
  }
}

/* ssmp and er, sequential: one node per iteration (GAGA/gaga/expander/ssmp.cu:9-160, er.cu:9-137;
 * variant 0 ssmp, 1 er, 2 ssmp_naive, 3 er_naive).  The node is the first of the largest
 * score (cublasIsamax), x_h += update_h, res -= update_h A_h (one fused multiply-add per row),
 * and the scores of the nodes sharing a row with h are recomputed (the naive forms recompute
 * all scores each iteration: the same values).  ssmp takes H_k(x) and a fresh residual every
 * k-th iteration and once after the loop; its loop stops on the residual history, er's on
 * a residual cycling between two values over the last 2d iterations (er_naive: no cycle test).
 * x and res: x^0 and scratch on entry. */
int gbo_seq_decode(const gbo_op *op, const float *y, int k, const gbo_opts *o, int variant, float *x, float *res,
                   float *res_record, gbo_info *info) {
  const int m = op->m, n = op->n, d = op->d;
  const int er = variant & 1, naive = variant >> 1;
  const int *rows = op->smv_rows;
  const float *vals = op->smv_vals;
  if (d < 1 || d > 64 || k < 1) return -1;
  /* row -> columns, ascending (create_row_index, kernels.cu:44-70) */
  int *ptr = (int *)calloc((size_t)m + 1, sizeof(int));
  int *col = (int *)malloc(sizeof(int) * (size_t)n * d);
  for (size_t e = 0; e < (size_t)n * d; ++e) ptr[rows[e] + 1]++;
  for (int i = 0; i < m; ++i) ptr[i + 1] += ptr[i];
  int *fill = (int *)malloc(sizeof(int) * (size_t)m);
  memcpy(fill, ptr, sizeof(int) * (size_t)m);
  for (int j = 0; j < n; ++j)
    for (int i = 0; i < d; ++i) col[fill[rows[(size_t)j * d + i]]++] = j;
  float *ax = (float *)malloc(sizeof(float) * m);
  float *upd = (float *)calloc((size_t)n, sizeof(float));
  float *score = (float *)calloc((size_t)n, sizeof(float));
  int *bins = (int *)calloc((size_t)n, sizeof(int));
  int *counters = (int *)calloc((size_t)o->num_bins, sizeof(int));
  gbo_A(op, x, ax);
  for (int i = 0; i < m; ++i) res[i] = fmaf(-1.0f, ax[i], y[i]);
  float err = nrm2f(res, m), err_start = err;
  if (res_record) res_record[0] = err;
  float prev[16], evol[16], diff = 1.0f, cyc[128];
  const int L = 2 * d;
  for (int i = 0; i < 16; ++i) { prev[i] = 0.0f; evol[i] = 1.0f; }
  for (int i = 0; i < L; ++i) cyc[i] = 0.0f;
  for (int j = 0; j < n; ++j) seq_score(er, res, rows + (size_t)j * d, d, &upd[j], &score[j]);
  int iter = 0, cycling = 0;
  while ((iter < o->maxiter) & (err > o->tol) & (err < (100.0f * err_start)) &
         (er ? (cycling == 0) : ((double)diff > 0.01 * (double)o->tol))) {
    if (naive)
      for (int j = 0; j < n; ++j) seq_score(er, res, rows + (size_t)j * d, d, &upd[j], &score[j]);
    int h = 0;
    float best = fabsf(score[0]);
    for (int j = 1; j < n; ++j)
      if (fabsf(score[j]) > best) {
        best = fabsf(score[j]);
        h = j;
      }
    const float u = upd[h];
    x[h] = x[h] + u;
    if (!er && (iter % k == 0) && (iter > 0)) {
      expander_hk(x, k, n, o->num_bins, bins, counters);
      gbo_A(op, x, ax);
      for (int i = 0; i < m; ++i) res[i] = fmaf(-1.0f, ax[i], y[i]);
      if (!naive)
        for (int j = 0; j < n; ++j) seq_score(er, res, rows + (size_t)j * d, d, &upd[j], &score[j]);
    } else {
      for (int i = 0; i < d; ++i) {
        const size_t e = (size_t)h * d + i;
        res[rows[e]] = fmaf(-u, vals[e], res[rows[e]]);
      }
      if (!naive)
        for (int i = 0; i < d; ++i) {
          const int r = rows[(size_t)h * d + i];
          for (int e = ptr[r]; e < ptr[r + 1]; ++e) {
            const int j = col[e];
            seq_score(er, res, rows + (size_t)j * d, d, &upd[j], &score[j]);
          }
        }
    }
    err = nrm2f(res, m);
    if (er) {
      iter++;
      for (int i = 0; i < L - 1; ++i) cyc[i] = cyc[i + 1];
      cyc[L - 1] = err;
      if (!naive && iter > L) {
        cycling = 1;
        for (int i = 3; i < L; i += 2) cycling = cycling * (cyc[i] == cyc[i - 2]);
      }
    } else {
      push16(prev, err);
      for (int i = 0; i < 15; ++i) evol[i] = evol[i + 1];
      evol[15] = prev[14] - prev[15];
      diff = max_list(evol, 16);
      iter++;
    }
    if (res_record) res_record[iter] = err;
  }
  if (!er) expander_hk(x, k, n, o->num_bins, bins, counters);
  if (info) {
    memset(info, 0, sizeof(*info));
    info->iter = iter;
    memcpy(info->resid_prev, prev, sizeof(prev));
  }
  free(ptr); free(col); free(fill); free(ax); free(upd); free(score); free(bins); free(counters);
  return 0;
}

/* serial_l0 (GAGA/gaga/expander/serial_l0.cu:16-161): Gauss-Seidel, the residual is
 * updated as soon as a column is accepted.  res must hold y - A x on entry. */
int gbo_serial_l0(const gbo_op *op, const float *y, const gbo_opts *o, float *x, float *res,
                  float *res_record, gbo_info *info) {
  (void)y;
  int m = op->m, n = op->n, d = op->d;
  const int *rows = op->smv_rows;
  float ss = 0.0f;
  for (int i = 0; i < m; ++i) ss = ss + res[i] * res[i];
  float norm = sqrtf(ss), norm0 = norm;
  if (res_record) res_record[0] = norm;
  int L = 2 * d;
  float *cyc = (float *)calloc((size_t)L, sizeof(float));
  float *prev = (float *)calloc((size_t)L, sizeof(float));
  float *evol = (float *)malloc(sizeof(float) * L);
  for (int i = 0; i < L; ++i) evol[i] = 1.0f;
  float diff = 1.0f;
  const float EPS = 0.000001f;
  int iter = 0, cycling = 0, nit = 0;
  while ((iter < o->maxiter) && (norm > o->tol) && (norm < (100.0f * norm0)) && (cycling == 0) &&
         ((double)diff > 0.000001)) {
    int shift = iter % d;
    for (int node = 0; node < n; ++node) {
      int idx = d * node;
      float omega = res[rows[idx + shift]];
      int score = 0;
      if (fabsf(omega) > EPS) {
        for (int i = 0; i < d; ++i) {
          if (fabsf(res[rows[idx + i]] - omega) <= EPS) score++;
          if (fabsf(res[rows[idx + i]]) <= EPS) score--;
        }
        if (score > o->l0_thresh) {
          x[node] = x[node] + omega;
          for (int i = 0; i < d; ++i) res[rows[idx + i]] = res[rows[idx + i]] - omega;
        }
      }
    }
    ss = 0.0f;
    for (int i = 0; i < m; ++i) ss = ss + res[i] * res[i];
    norm = sqrtf(ss);
    for (int i = 0; i < L - 1; ++i) prev[i] = prev[i + 1];
    prev[L - 1] = norm;
    for (int i = 0; i < L - 1; ++i) evol[i] = evol[i + 1];
    evol[L - 1] = prev[L - 2] - prev[L - 1];
    diff = evol[0];
    for (int i = 0; i < L; ++i) diff = diff > evol[i] ? diff : evol[i];
    for (int i = 0; i < L - 1; ++i) cyc[i] = cyc[i + 1];
    cyc[L - 1] = norm;
    if (iter > L) {
      cycling = 1;
      for (int i = 3; i < L; i += 2) cycling = cycling * (cyc[i] == cyc[i - 2]);
    }
    /* the reference writes resRecord[nIters] starting at 0 (overwriting the
     * initial norm), serial_l0.cu:146-148 */
    if (res_record) res_record[nit] = norm;
    nit++;
    iter = iter + 1;
  }
  if (info) {
    memset(info, 0, sizeof(*info));
    info->iter = iter;
  }
  free(cyc); free(prev); free(evol);
  return 0;
}

/* ------------------------------------------------------------------ */
void gbo_results(const float *x, const float *x_true, int n, int k, float norms[3], int supp[4]) {
  int tp = 0, tn = 0;
  double l1 = 0, l2 = 0, li = 0, e1 = 0, e2 = 0, ei = 0;
  for (int i = 0; i < n; ++i) {
    if (x_true[i] != 0.0f) { if (x[i] != 0.0f) tp++; }
    else if (x[i] == 0.0f) tn++;
    double a = fabs((double)x_true[i]), e = fabs((double)x_true[i] - (double)x[i]);
    l1 += a; l2 += a * a; if (a > li) li = a;
    e1 += e; e2 += e * e; if (e > ei) ei = e;
  }
  norms[0] = (float)(e1 / l1);
  norms[1] = (float)(sqrt(e2) / sqrt(l2));
  norms[2] = (float)(ei / li);
  supp[0] = tp; supp[1] = k - tp; supp[2] = tn; supp[3] = n - k - tn;
}

/* ------------------------------------------------------------------ */
int gbo_solve_dense_trials(int ntrials, const int *nn, const int *mm, const int *kk, uint32_t seed,
                           const uint32_t *trial_ids, int alg, float tol_rel, int maxiter,
                           int threads, int *iters, float *rel_err) {
  /* trials one after another; generation and operators use all `threads` inside a trial */
  int ok = 0;
#ifdef _OPENMP
  if (threads > 0) omp_set_num_threads(threads);
#endif
  for (int t = 0; t < ntrials; ++t) {
    int n = nn[t], m = mm[t], k = kk[t];
    uint32_t tid = trial_ids ? trial_ids[t] : (uint32_t)t;
    /* trial tid of a sweep is the problem drawn with seed + tid (the device's keying) */
    const uint32_t key = seed + tid;
    float *A = (float *)malloc(sizeof(float) * (size_t)m * n);
    float *xt = (float *)malloc(sizeof(float) * n);
    float *x = (float *)calloc((size_t)n, sizeof(float));
    float *y = (float *)malloc(sizeof(float) * m);
    gbo_gen_dense(m, n, m, 1, key, 0, A);
    int ksupp = gbo_gen_vector(n, k, 1, key, 0, xt);
    gbo_op op = {GBO_OP_DENSE, m, n, A, m, 0, 0, 0, 0};
    gbo_A(&op, xt, y);
    gbo_opts o = {alg, tol_rel * nrm2f(y, m), maxiter, n / 20 > 1000 ? n / 20 : 1000, 0, 1, threads, 3.0f};
    gbo_info info;
    gbo_solve(&op, y, ksupp, &o, x, &info);
    float norms[3];
    int supp[4];
    gbo_results(x, xt, n, ksupp, norms, supp);
    if (iters) iters[t] = info.iter;
    if (rel_err) rel_err[t] = norms[1];
    if (norms[1] <= 1e-3f) ok += 1;
    free(A); free(xt); free(x); free(y);
  }
  return ok;
}
