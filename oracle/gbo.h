/*
 * gbo.h -- CPU oracle for the greedy sparse-recovery hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker for the CUDA
 * product (gaga_gb300/csrc) and the timed CPU baseline of bench.py; the
 * product never links, loads or calls it.
 *
 * It restates, in plain C (FP32 vectors, FP64 accumulation of scalar
 * reductions), the reference algorithms of GAGA:
 *   - LinearBinning / FindSupportSet / Threshold      (GAGA/gaga/kernels.cu:64-81,135-146,
 *                                                      GAGA/gaga/functions.cu:374-436)
 *   - RestrictedSD / RestrictedCG / RestrictedCGwithSupportEvolution /
 *     UnrestrictedCG                                  (GAGA/gaga/functions.cu:659-745,922-1220)
 *   - NIHT / HTP / CGIHT loops                        (GAGA/gaga/algorithms.cu:1274-1441,
 *                                                      2491-2716, 3689-3942)
 *   - parallel_l0 (+ its kernels)                     (GAGA/gaga/expander/parallel_l0.cu:9-151,
 *                                                      GAGA/gaga/expander/kernels.cu:3-14,353-388)
 *   - serial_l0                                       (GAGA/gaga/expander/serial_l0.cu:16-161)
 *   - dense / DCT / expander operators                (GAGA/Matrices/gen_gpu.cu:141-171,
 *                                                      GAGA/Matrices/dct_gpu.cu:121-353,
 *                                                      GAGA/Matrices/smv_gpu.cu:29-47,108-135)
 *   - results norms                                   (GAGA/gaga/results.cu:363-487)
 *
 * Parity pins: the integer kernels (LinearBinning, threshold, checkSupportEvolution,
 * cuda_compute_scores_l0, cuda_update_residual, sparse_matvec(T)) and serial_l0 are
 * pinned against the reference's own source executed on the CPU (oracle/_ref, golden
 * fixtures in tests/golden).  The DCT is pinned against scipy's orthonormal DCT-II.
 * The algorithm loops are restated line by line; the reference has no CPU build of
 * them (its loops call cuBLAS/cuFFT), so those loops are pinned by reading only.
 */
#ifndef GBO_H
#define GBO_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* algorithm ids (reference alg switch, GAGA/gaga/gaga_gen.cu:619-631, gaga_smv.cu:841-857) */
enum { GBO_NIHT = 0, GBO_HTP = 1, GBO_IHT = 2, GBO_HT_SD = 3, GBO_HT_CG = 4, GBO_CSMPSP = 5, GBO_CGIHT = 6,
       GBO_FIHT = 7, GBO_ALPS = 8, GBO_CGIHT_PROJ = 9, GBO_SMP = 10, GBO_PARALLEL_LDDSR = 13, GBO_PARALLEL_L0 = 14,
       GBO_SERIAL_L0 = 15, GBO_PARALLEL_L0_SWIPE = 18 };
/* operator kinds */
enum { GBO_OP_DENSE = 0, GBO_OP_DCT = 1, GBO_OP_SMV = 2 };

typedef struct {
  int kind;
  int m, n;
  /* dense: column-major m x n with leading dimension lda >= m */
  const float *A;
  int lda;
  /* dct: m sampled rows, 0-based */
  const int *dct_rows;
  /* smv: d nonzeros per column, column j owns entries [j*d, (j+1)*d), 0-based rows */
  const int *smv_rows;
  const float *smv_vals;
  int d;
} gbo_op;

typedef struct {
  int alg;
  float tol;         /* absolute tolerance on ||y - Ax|| (reference semantics) */
  int maxiter;
  int num_bins;
  int restart;       /* CGIHT restartFlag */
  int l0_thresh;     /* parallel_l0 / serial_l0 alpha */
  int threads;       /* OpenMP threads for operators (0 = runtime default) */
  float proj_frac_tol; /* CGIHTprojected projFracTol (gaga_gen.cu:190: 3) */
  int timing;        /* 'timing' on: NIHT / HTP run as their timing variants
                        (GAGA/gaga/algorithms_timings.cu); other algorithms ignore it */
  int supp_flag;     /* 'supportFlag' of the timing variants: 0 adaptive binning, 1 binning every
                        iteration, 2 sort with a dynamic threshold, 3 sort every iteration */
  float alpha;       /* 'alpha' of the timing variants: initial MaxBin = num_bins (1 - alpha) */
} gbo_opts;

typedef struct {
  int iter;
  int sum;              /* last FindSupportSet sum */
  float conv_rate;      /* given-data convRate (GAGA/gaga/gaga_gen.cu:730-743) */
  float resid_prev[16]; /* residNorm_prev at exit */
  int k_bin;
  int ucg_steps, rcg_steps; /* CGIHT: UnrestrictedCG / RestrictedCGwithSupportEvolution steps */
} gbo_info;

/* ---------------- random numbers and problem generation ---------------- */
void gbo_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);
float gbo_u01(uint32_t x);
/* dense A (N(0,1)/sqrt(m) for ens 1, +-1/sqrt(m) for ens 2), column-major with lda */
void gbo_gen_dense(int m, int n, int lda, int ens, uint32_t seed, uint32_t trial, float *A);
/* sparse vector via the reference's support binning (GAGA/gaga/createVector.cu:207-300):
 * returns the support size (>= k). vec_dist 0 uniform, 1 +-1, 2 gaussian. */
int gbo_gen_vector(int n, int k, int vec_dist, uint32_t seed, uint32_t trial, float *x);
/* m of n DCT rows without replacement, partial Fisher-Yates as MRandShuffle
 * (GAGA/gaga/createProblem_kernels.cu:65-75, createMeasurements_dct.cu:85-89) */
void gbo_gen_dct_rows(int n, int m, uint32_t seed, uint32_t trial, int *rows);
/* expander rows: d distinct uniform rows per column (GAGA/gaga/createMeasurements_smv.cu:178-233);
 * vals: ens 1 -> 1/sqrt(d), 2 -> +-1/sqrt(d), 3 -> 1 */
void gbo_gen_smv(int m, int n, int d, int ens, uint32_t seed, uint32_t trial, int *rows, float *vals);

/* ---------------- operators ---------------- */
void gbo_A(const gbo_op *op, const float *x, float *y);   /* y = A x, length m */
void gbo_AT(const gbo_op *op, const float *r, float *g);  /* g = A^T r, length n */
void gbo_dct2(int N, const float *x, float *out);         /* orthonormal DCT-II */
void gbo_dct3(int N, const float *x, float *out);         /* its transpose (DCT-III) */

/* ---------------- support selection ---------------- */
int gbo_f2i_rz(float v);
void gbo_linear_binning(const float *v, int n, int num_bins, int max_bin, float slope,
                        float intercept, int *bins, int *counters);
typedef struct {
  int num_bins, max_bin, k_bin, sum;
  float alpha, min_val;
} gbo_bin_state;
int gbo_find_support_set(const float *v, int *bins, int *counters, float slope, float intercept,
                         float max_change, gbo_bin_state *st, int n, int k);
void gbo_threshold(float *v, const int *bins, int k_bin, int n);
/* FindSupportSet_sort (GAGA/gaga/functions.cu:446-465); buf: n floats of scratch; returns T */
float gbo_find_support_set_sort(float *v, int *bins, float T, float max_change, float *buf, int n, int k);
float gbo_max_magnitude(const float *v, int n);

/* ---------------- solvers ---------------- */
/* smp (GAGA/gaga/expander/smp.cu); res_record as for parallel_l0 */
int gbo_smp(const gbo_op *op, const float *y, int k, const gbo_opts *o, float *x, float *res, float *res_record,
            gbo_info *info);
/* ssmp / er and their naive forms (variant 0 ssmp, 1 er, 2 ssmp_naive, 3 er_naive) */
int gbo_seq_decode(const gbo_op *op, const float *y, int k, const gbo_opts *o, int variant, float *x, float *res,
                   float *res_record, gbo_info *info);
int gbo_solve(const gbo_op *op, const float *y, int k, const gbo_opts *o, float *x, gbo_info *info);
/* parallel_l0 / serial_l0 write res_record (maxiter+1 entries, may be NULL) */
int gbo_parallel_l0(const gbo_op *op, const float *y, const gbo_opts *o, float *x, float *res,
                    float *res_record, gbo_info *info);
int gbo_serial_l0(const gbo_op *op, const float *y, const gbo_opts *o, float *x, float *res,
                  float *res_record, gbo_info *info);
/* l0 step kernels, for per-step parity */
void gbo_l0_scores(const float *res, float *x, float *updates, const int *rows, int n, int d,
                   int thresh, int shift, int *found);
void gbo_l0_update_residual(float *res, const int *rows, const float *updates, int n, int d);

/* relative l1 / l2 / linf errors and TP/FP/TN/FN (GAGA/gaga/results.cu:408-487) */
void gbo_results(const float *x, const float *x_true, int n, int k, float norms[3], int supp[4]);

/* CPU baseline: independent dense trials generated from (seed, trial), solved with
 * OpenMP over trials.  Returns the number of trials with rel l2 error <= 1e-3. */
int gbo_solve_dense_trials(int ntrials, const int *n, const int *m, const int *k, uint32_t seed,
                           const uint32_t *trial_ids, int alg, float tol_rel, int maxiter,
                           int threads, int *iters, float *rel_err);

#ifdef __cplusplus
}
#endif
#endif
