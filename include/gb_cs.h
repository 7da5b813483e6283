/*
 * gb_cs.h -- C ABI of the GB300-native greedy sparse-recovery library (libgb_cs.so).
 *
 * The drop-in boundary for GAGA's recovery path.  GAGA exposes it as three MATLAB
 * MEX gateways reached through gaga_cs.m:
 *     gaga_gen  GAGA/gaga/gaga_gen.cu:41-848   dense Gaussian / Bernoulli matrices
 *     gaga_dct  GAGA/gaga/gaga_dct.cu:40-831   row-subsampled orthonormal DCT
 *     gaga_smv  GAGA/gaga/gaga_smv.cu:39-1198  sparse expander (d nonzeros per column)
 * each with a "generate and solve" usage and a "solve given data" usage
 * (GAGA/gaga/gaga_cs.m:7-64).  This header exports both usages as plain C calls on
 * host or device pointers.  A MEX shim maps MATLAB arrays onto these calls one to one
 * (1-based indices become 0-based there).  Names use the gb_cs_ prefix; the GAGA licence
 * (GAGA/GAGA_license:5) reserves the gaga_* function names.
 *
 * Semantics kept from the reference:
 *   - algorithms NIHT, HTP, CGIHT (restartFlag) on all operators; parallel_l0 on smv
 *   - option names/meaning/defaults of gagaOptions.m, including tol compared with the
 *     ABSOLUTE residual norm ||y - A x||_2 and the default tol of 10^(-4) evaluated
 *     as C's XOR (= -10), which disables the residual test (GAGA/gaga/gaga_gen.cu:183)
 *   - support selection by linear binning, bit-exact to the reference kernel
 *   - outputs: x, iterations, convergence rate; norms / times / support counts in
 *     generate mode; residual record for parallel_l0
 * Additions: integer status codes, an explicit CUDA stream, host or device buffers,
 * tol_is_relative (tol * ||y||), re-entrant calls (no globals on the solve path).
 */
#ifndef GB_CS_H
#define GB_CS_H

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
  GB_OK = 0,
  GB_BAD_ARG = 1,      /* invalid algorithm / size / option (reference: printf + return) */
  GB_OOM = 2,          /* device allocation failed */
  GB_WATCHDOG = 3,     /* a device-side iteration bound was hit before the stopping rules */
  GB_CUDA_ERROR = 4,   /* CUDA runtime error; text in gb_cs_last_error() */
  GB_UNSUPPORTED = 5,  /* valid reference input outside this build (e.g. DCT length not 2^p) */
  GB_NO_DEVICE = 6
} gb_status;

enum { GB_OP_DENSE = 0, GB_OP_DCT = 1, GB_OP_SMV = 2 };
enum { GB_HOST = 0, GB_DEVICE = 1 };

/* Reference algorithm numbers (GAGA/gaga/gaga_gen.cu:619-631, gaga_smv.cu:841-857):
 * "NIHT", "HTP", "IHT", "ThresholdSD", "ThresholdCG", "CSMPSP", "CGIHT", "FIHT", "ALPS",
 * "CGIHTprojected"; expander decoders "smp", "ssmp", "er", "parallel_lddsr", "parallel_l0",
 * "er_naive", "ssmp_naive", "parallel_l0_swipe". */
enum { GB_ALG_NIHT = 0, GB_ALG_HTP = 1, GB_ALG_IHT = 2, GB_ALG_HT_SD = 3, GB_ALG_HT_CG = 4, GB_ALG_CSMPSP = 5,
       GB_ALG_CGIHT = 6, GB_ALG_FIHT = 7, GB_ALG_ALPS = 8, GB_ALG_CGIHT_PROJ = 9, GB_ALG_SMP = 10,
       GB_ALG_SSMP = 11, GB_ALG_ER = 12, GB_ALG_PARALLEL_LDDSR = 13,
       GB_ALG_PARALLEL_L0 = 14, GB_ALG_ER_NAIVE = 16, GB_ALG_SSMP_NAIVE = 17, GB_ALG_PARALLEL_L0_SWIPE = 18 };

/* Options: the gagaOptions name/value list (GAGA/gaga/gagaOptions.m:8-58) as a struct. */
typedef struct {
  float tol;            /* 'tol'            default 10^(-4) == -10 (reference XOR) */
  int tol_is_relative;  /* extension: tol * ||y||_2 becomes the absolute tolerance */
  int maxiter;          /* 'maxiter'        300 for HTP, 5000 otherwise */
  int num_bins;         /* 'numBins'        max(n/20, 1000) */
  int restart_flag;     /* 'restartFlag'    0 */
  int l0_thresh;        /* 'l0_thresh'      1, clamped to [1, d] (gaga_smv.cu:310-313) */
  int vec_distribution; /* 'vecDistribution' 0 uniform, 1 binary (default), 2 gaussian */
  int matrix_ensemble;  /* 'matrixEnsemble' gen: 1 gaussian / 2 binary; smv: 1 ones/sqrt(d),
                           2 +-1/sqrt(d), 3 expander ones (default; forced for l0) */
  int k_fixed;          /* 'kFixed'         0 */
  unsigned int seed;    /* 'seed'           0 here (the reference uses clock()) */
  float noise;          /* 'noise'          0 */
  int gpu_number;       /* 'gpuNumber'      0 */
  int conv_rate_num;    /* 'convRateNum'    16 */
  float alpha;          /* 'alpha'          0.25: initial MaxBin = numBins (1 - alpha) of the timing variants */
  int support_flag;     /* 'supportFlag'    0 (timing variants only): 0 adaptive binning, 1 binning
                           every iteration, 2 sort-based threshold lowered while it can, 3 sort
                           every iteration (GAGA/gaga/algorithms_timings.cu:461-465) */
  int timing;           /* 'timing'         0; 1 ('on') runs NIHT and HTP as their timing variants
                           (algorithms_timings.cu; no cycle test, alpha and supportFlag used)
                           and records per-iteration times; other algorithms ignore it
                           (gaga_gen.cu:331-334) */
  const float *learned_params; /* extension: CGIHT only, device pointer to the warm-start
                           MLP's gb_cs_mlp_num_params() FP32 parameters; NULL = plain start */
  const char *results_dir;  /* extension: generate-and-solve appends the reference's result
                           line to the dated file in this directory ("" = current directory,
                           as the reference always does); NULL = no file */
  float proj_frac_tol;  /* 'projFracTol'    3 (CGIHTprojected, gaga_gen.cu:190) */
  int watchdog_passes;  /* extension: bound on the device-side passes of a solve's loop
                           (0: maxiter + 4); a loop still running past it stops with
                           GB_WATCHDOG.  The reference's host loop has no such bound. */
} gb_options;

/* A recovery problem in "given data" form. */
typedef struct {
  int kind;            /* GB_OP_DENSE / GB_OP_DCT / GB_OP_SMV */
  int m, n, k;
  const float *y;      /* m measurements */
  const float *A;      /* dense: column-major m x n, leading dimension lda (0 -> m) */
  int lda;
  const int *rows;     /* dct: m sampled rows; smv: n*d row indices, grouped by column */
  const int *cols;     /* smv: n*d column indices (each column's d entries contiguous) */
  const float *vals;   /* smv: n*d values */
  int d;               /* smv nonzeros per column (0: inferred from cols as the reference does) */
  int index_base;      /* 0, or 1 for MATLAB indices (the reference shifts down on the device) */
  int location;        /* GB_HOST or GB_DEVICE for every pointer above and x_out */
  void *stream;        /* cudaStream_t, NULL for the legacy default stream */
} gb_problem;

typedef struct {
  int iter;             /* iterations */
  float conv_rate;      /* convRate */
  float norms[3];       /* generate mode: relative l1, l2, linf error (results.cu:444-487) */
  float times[3];       /* ms: algorithm, average iteration, total incl. generation */
  int support[4];       /* generate mode: TP, FP, TN, FN */
  int k_used;           /* generate mode: support size actually drawn */
  float resid_prev[16]; /* residNorm_prev at exit */
  int stop_reason;      /* 1 tol, 2 maxiter, 3 divergence, 4 stall, 5 cycle, 6 slow rate, 7 no candidates */
  float *res_record;    /* parallel_l0: caller buffer of maxiter+1 floats or NULL (resRecord) */
  int warm_start;       /* learned warm start: 0 not used, 1 used, 2 abandoned after 10
                           iterations and solved again from zero (iter counts both runs) */
  /* timing variants (NIHT, HTP with timing on): caller buffers of maxiter floats or NULL,
   * filled for the first `iter` iterations from device timer stamps: time_per_iteration,
   * time_supp_set (support identification), and for HTP cg_per_iteration (CG steps) and
   * time_for_cg, in ms (algorithms_timings.cu:635-636, 1536-1539) */
  float *time_per_iteration;
  float *time_supp_set;
  float *cg_per_iteration;
  float *time_for_cg;
  float *time_record;   /* expander decoders: caller buffer of maxiter+1 floats or NULL
                           (timeRecord): ms from the loop start to the end of each iteration,
                           0 at entry 0, from device timer stamps */
} gb_result;

/* Support-selection state carried between FindSupportSet calls. */
typedef struct {
  int num_bins, max_bin, k_bin, sum;
  float alpha, min_val;
} gb_bin_state;

const char *gb_cs_version(void);
const char *gb_cs_last_error(void);

/* Reference defaults for `alg` and signal length n (GAGA/gaga/gaga_gen.cu:176-197,
 * gaga_smv.cu:239-258). */
void gb_cs_default_options(gb_options *o, const char *alg, int n);

/* Reference algorithm number for an algorithm string, or -1 (gaga_gen.cu:65, gaga_smv.cu:97-107). */
int gb_cs_alg_id(const char *alg);

/* "Solve given data": [x, iters, convRate] = gaga_gen(alg, y, A, k, opts)
 * (GAGA/gaga/gaga_gen.cu:115-134,560-563,730-743), gaga_dct(alg, y, rows, k, m, n, opts)
 * (gaga_dct.cu:88-127,540-544) and [x, iters, convRate, resRecord, timeRecord] =
 * gaga_smv(alg, y, rows, cols, vals, k, opts) (gaga_smv.cu:131-195,675-688).
 * x_out has n floats at p->location. */
gb_status gb_cs_solve(const char *alg, const gb_problem *p, const gb_options *o, float *x_out,
                      gb_result *r);

/* "Generate and solve": [norms, times, iters, support, convRate, xout] =
 * gaga_gen(alg, k, m, n, opts) (gaga_gen.cu:90-114,535-559), gaga_dct(alg, k, m, n, opts),
 * gaga_smv(alg, k, m, n, d, opts).  The problem is drawn on the device from o->seed
 * (Philox-4x32-10 instead of cuRAND).  x_out / x_true_out are host buffers of n floats
 * (x_true_out may be NULL). */
gb_status gb_cs_generate_and_solve(const char *alg, int kind, int k, int m, int n, int d,
                                   const gb_options *o, float *x_out, float *x_true_out,
                                   gb_result *r);

/* Append the result line of one generate-and-solve run to the reference's dated results file
 * in `dir` (NULL or "" = current directory): gpu_data_{gen,dct,smv}YYYYMMDD.txt, with
 * _noise%0.3f before .txt when o->noise > 0 (GAGA/gaga/results.cu:173,343,516,686,863,1032),
 * the line as File_output / File_output_smv / File_output_gen write it
 * (GAGA/gaga/functions.cu:34-80).  d is the expander's nonzeros per column (smv only).
 * The file's path is copied to path_out (path_len bytes) when not NULL. */
gb_status gb_cs_write_result(const char *dir, const char *alg, int kind, int k, int m, int n, int d,
                             const gb_options *o, const gb_result *r, char *path_out, int path_len);

/* ---- component entry points (device pointers; replace the reference's L1/L2 routines) ---- */

/* LinearBinning (GAGA/gaga/kernels.cu:135-146): bins[i] for every i; counters[b]
 * incremented for b < max_bin.  counters must hold num_bins ints and is NOT cleared. */
gb_status gb_cs_linear_binning(const float *d_v, int n, int num_bins, int max_bin, float slope,
                               float intercept, int *d_bins, int *d_counters, void *stream);

/* FindSupportSet (GAGA/gaga/functions.cu:397-436) followed by Threshold
 * (functions.cu:374-378) when threshold_v != 0.  `st` (host) is read and updated.
 * d_counters may be NULL. */
gb_status gb_cs_find_support_set(float *d_v, int n, int k, float slope, float intercept,
                                 float max_change, gb_bin_state *st, int *d_bins,
                                 int *d_counters, int threshold_v, void *stream);

/* A_gen/AT_gen (GAGA/Matrices/gen_gpu.cu:141-171), A_dct/AT_dct (dct_gpu.cu:328-353),
 * A_smv/AT_smv (smv_gpu.cu:108-135): out = A in (transpose 0) or A^T in (transpose 1).
 * p->location must be GB_DEVICE; y/k are ignored. */
gb_status gb_cs_operator_apply(const gb_problem *p, int transpose, const float *d_in, float *d_out);

/* Measurement helper (no reference counterpart): the device time of gb_cs_operator_apply's
 * kernels, set up once, CUDA events around each of `reps` applications after `warmup`
 * untimed ones; a non-NULL d_flush of flush_bytes is overwritten before each application
 * (outside the events) so operands come from HBM.  *ms_out = mean ms per application.
 * transpose 2 / 3 (dense, lda % 8 == 0): A^T in with the batched form's compact operand,
 * A rounded to 24 bits / to BF16 (gb_batch.grad_format), split from A before the timing. */
gb_status gb_cs_operator_time(const gb_problem *p, int transpose, const float *d_in, float *d_out, int warmup,
                              int reps, void *d_flush, size_t flush_bytes, float *ms_out);

/* FindSupportSet_sort (GAGA/gaga/functions.cu:446-465), the sort-based support of the timing
 * variants (supportFlag 2/3): if T > max_change, T -= max_change; otherwise T = the k-th
 * largest |v| (element n-k of |v| sorted ascending, exact) and every bin becomes 1; then
 * entries with |v| < T are zeroed and their bin set to 2.  The new T goes to *T_out.  Device
 * pointers, 1 <= k <= n; synchronises `stream`. */
gb_status gb_cs_find_support_set_sort(float *d_v, int *d_bins, int n, int k, float T, float max_change,
                                      float *T_out, void *stream);

/* Dense operator apply that allocates nothing (no counterpart in the reference): out = A in
 * (transpose 0, in has n entries, out m) or A^T in (transpose 1), A column-major m x n with
 * leading dimension lda, every pointer on the device; asynchronous on `stream`.  For
 * callers that cannot allocate device memory during the call: code inside a CUDA stream
 * capture, services that budget every allocation up front, embedders with their own
 * allocator.  Its scratch is one fixed 1 MiB device array per GPU held until the process
 * exits; m and n must be <= 65536 (GB_BAD_ARG otherwise).  The first call on a device
 * resolves the array's address and must happen outside a stream capture.  All calls share
 * the array: calls that overlap on the GPU race and must be serialised by the caller.
 * transpose 2 is A in on the support (nonzero pattern) found by the previous transpose 0
 * call on this device, skipping the support scan: repeated applications with a fixed
 * support, as in a CG solve on the support.  That call must have had the same d_A, lda, m
 * and n, with no transpose 1 call since (GB_BAD_ARG otherwise). */
gb_status gb_cs_dense_apply_noalloc(const float *d_A, int lda, int m, int n, int transpose,
                                    const float *d_in, float *d_out, void *stream);

/* One parallel_l0 iteration body (cuda_compute_scores_l0 + cuda_update_residual,
 * GAGA/gaga/expander/kernels.cu:3-14,353-388) on column-grouped 0-based rows.
 * Returns the candidate flag in *found. */
gb_status gb_cs_l0_step(float *d_res, float *d_x, float *d_updates, const int *d_rows, int m, int n,
                        int d, int thresh, int shift, int *found, void *stream);

/* ---- batched form (no reference counterpart: the reference solves one trial per call) ----
 * Thousands of independent dense Gaussian trials, each with its own (n, m, k) and its own
 * problem drawn on the device exactly as gb_cs_generate_and_solve draws it with seed
 * `seed + trial_id` (Gaussian A, +-1 signal), solved by NIHT, HTP or CGIHT: trials with
 * n <= resident_n by one thread-block cluster each in one persistent launch, the others by
 * slot graphs over a device trial queue, both at once.  Per-trial outputs (host or device arrays of ntrials entries, any may be NULL):
 * iterations, relative l2 error against the generated x, and a verdict flag
 * (rel l2 <= 1e-3).  tol_rel is relative to ||y||. */
typedef struct {
  int ntrials;
  const int *n, *m, *k;          /* host arrays */
  const unsigned int *trial_id;  /* host array (NULL: 0..ntrials-1) */
  unsigned int seed;
  int alg;                       /* GB_ALG_NIHT, GB_ALG_HTP or GB_ALG_CGIHT */
  float tol_rel;
  int maxiter;
  int use_learned;               /* CGIHT only: learned warm start, falling back to a plain
                                    solve for trials whose residual does not drop in 10 iterations */
  const float *learned_params;   /* device pointer to the MLP parameters when use_learned */
  int slots;                     /* schedule: concurrent trial slots (0: 16, fewer if memory is short) */
  int sm_share;                  /* schedule: SMs each slot's kernels are shaped for (0: half the GPU) */
  void *stream;
  int resident_n;                /* trials with n <= resident_n are solved by the cluster-resident
                                    kernel, one thread-block cluster per trial, while the slots take
                                    the others (0: 8192; < 0: slots only) */
  int cluster;                   /* CTAs per cluster of the resident kernel (0: 4, more if the
                                    trial sizes need more shared memory than 4 CTAs have) */
  int grad_format;               /* the operand of A^T r (GB_GRAD_*): FP32 A (0, the default),
                                    or a compact copy of A written beside it when the trial is
                                    drawn -- each entry rounded to 24 bits (3 bytes) or to BF16
                                    (2 bytes), FP32 accumulation.  A x_S, the residual and the
                                    stopping test keep FP32 A, so a solution of y = A x stays a
                                    fixed point; only the gradient directions change. */
  const unsigned char *grad_formats; /* host array of ntrials entries GB_GRAD_A24 / GB_GRAD_BF16: the
                                    operand per trial (NULL: grad_format for every trial) */
  int av_rows;                   /* schedule: row tile of the slot graphs' A x_S kernel, 128 or 256
                                    rows (0: 128) */
  int residual_refresh;          /* CGIHT: 0 (the default) computes y - A x at every step, as the
                                    reference does; N > 0 lets a restricted step that follows a
                                    restricted step on the same support update the residual as
                                    r - alpha A p (the product the previous step made, one pass
                                    over A_S fewer), recomputing y - A x every N-th iteration */
} gb_batch;

enum { GB_GRAD_FP32 = 0, GB_GRAD_A24 = 1, GB_GRAD_BF16 = 2 };

/* Calls from several host threads run one at a time (the batched form's engines are
 * shared per device). */
gb_status gb_cs_solve_batch(const gb_batch *b, int *iters_out, float *rel_err_out,
                            int *success_out, int *num_success);

/* Algorithmic matvec bytes (per-iteration operator traffic summed over all trials) and the
 * device time in ms of the last gb_cs_solve_batch call on this thread (no reference
 * counterpart; used for roofline reporting). */
void gb_cs_batch_last_stats(double *bytes, float *kernel_ms);

/* CTAs per cluster of the last cluster-resident launch of gb_cs_solve_batch on the current
 * device (0: none yet). */
int gb_cs_batch_last_cluster(void);

/* ---- shared-matrix batched form (no reference counterpart) ----
 * ntrials NIHT or CGIHT trials y_t = A x0_t that share one dense Gaussian A (drawn from `seed` as
 * gb_cs_generate_and_solve draws it; trial t's +-1 signal x0_t with k[t] nonzeros uses the
 * key seed + 1 + first_trial + t).  The operator applications of all trials run as BF16 tensor-core
 * GEMMs with FP32 accumulation; the residual keeps ~FP32 accuracy by splitting A and x
 * into BF16 high and low parts; trials that stop with ||y - A x|| <= tol_rel ||y|| are
 * debiased by least squares on their support (CG on the normal equations, FP64 scalars,
 * split-precision GEMM products).  m, n multiples of 128 with
 * 128 <= m <= n <= 32768.  Per-trial outputs as for gb_cs_solve_batch (host arrays).
 * d_A_out (m*n, column-major), d_Y_out (ntrials*m), d_X0_out (ntrials*n) are optional
 * device copies of the generated problem. */
typedef struct {
  int ntrials, m, n;
  const int *k;                  /* host array of ntrials sparsities */
  unsigned int seed;
  unsigned int first_trial;      /* trial t's signal uses the key seed + 1 + first_trial + t */
  float tol_rel;
  int maxiter;
  int precision;                 /* bit 0: split-BF16 A^T r, bit 1: split-BF16 A x_thres (0: plain BF16) */
  float *d_A_out, *d_Y_out, *d_X0_out;
  void *stream;
  int alg;                       /* GB_ALG_NIHT (0, the default) or GB_ALG_CGIHT (restartFlag off) */
  const float *learned_params;   /* CGIHT: device pointer to the warm-start MLP's parameters, or
                                    NULL for the plain start; a trial whose residual has not
                                    dropped below the warm start's within 10 iterations is
                                    solved again from the plain start, iterations added */
  float *d_X_out;                /* optional device copy of the final x of every trial (ntrials*n) */
} gb_shared_batch;

gb_status gb_cs_solve_shared_batch(const gb_shared_batch *b, int *iters_out, float *rel_err_out,
                                   int *success_out, int *num_success);

/* Trials of the last gb_cs_solve_shared_batch call on this thread whose learned warm start
 * was abandoned after 10 iterations and solved again from the plain start (no reference
 * counterpart). */
int gb_cs_shared_last_fallbacks(void);

/* ---- learned warm start (no reference counterpart) ----
 * A per-coordinate MLP 4 -> 64 -> 64 -> 1 (GELU; weights rounded to BF16 at use, FP32
 * accumulation) maps the features of coordinate i of a problem, g = A^T y:
 *   |g_i| / max|g|, rank fraction of |g_i| (0 = largest), delta = m/n, rho = k/m
 * to w_i ~ x_i / g_i of the final solution; CGIHT then starts from H_k(w . g).
 * Parameters are FP32 on the device in the order W1[64][4] b1[64] W2[64][64] b2[64] W3[64] b3. */
int gb_cs_mlp_num_params(void);
/* features (n x 4 row-major, device) of g (device, n); synchronous */
gb_status gb_cs_mlp_features(const float *d_g, int n, int m, int k, float *d_feat, void *stream);
/* network outputs for ns feature rows */
gb_status gb_cs_mlp_forward(const float *d_params, const float *d_feat, int ns, float *d_out, void *stream);
/* gradient of the mean squared error against d_tgt over all ns rows (and the loss); synchronous */
gb_status gb_cs_mlp_grad(const float *d_params, const float *d_feat, const float *d_tgt, int ns, float *d_grad,
                         float *d_loss, void *stream);
/* Adam training in place (minibatches of `batch` rows, `epochs` shuffled passes); the mean
 * minibatch loss of each epoch goes to h_epoch_loss (host, epochs floats) if not NULL */
gb_status gb_cs_mlp_train(float *d_params, const float *d_feat, const float *d_tgt, int ns, int batch, int epochs,
                          float lr, unsigned int seed, float *h_epoch_loss, void *stream);

/* GEMM FLOPs issued and device time in ms of the last gb_cs_solve_shared_batch call on this
 * thread (no reference counterpart; used for roofline reporting). */
void gb_cs_shared_last_stats(double *gemm_flops, float *kernel_ms);

/* BF16 tensor-core GEMM with FP32 accumulation (no reference counterpart; the building
 * block of the shared-matrix form):  Ct[N x M] = [Y -] (A[M x K] . B[N x K]^T)^T with A, B
 * row-major BF16 (K contiguous), Ct and Y FP32 with M contiguous per column, d_Cb an
 * optional BF16 copy of Ct.  M, N multiples of 128, K a multiple of 32. */
gb_status gb_cs_gemm_bf16_tn(const void *d_A, const void *d_B, float *d_Ct, int M, int N, int K,
                             const float *d_Y, void *d_Cb, void *stream);

#ifdef __cplusplus
}
#endif
#endif
