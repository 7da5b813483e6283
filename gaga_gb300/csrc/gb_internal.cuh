// gb_internal.cuh -- shared definitions of the GB300 greedy sparse-recovery library.
//
// Layout in HBM (per solve workspace):
//   dense A   column-major, leading dimension lda (a multiple of 4 floats when the library
//             owns the copy, so every column starts 16-byte aligned for float4 streams)
//   vectors   x, x_thres, grad, grad_prev, grad_prev_thres (n); y, resid, resid_update (m,
//             padded to lda with zeros); bins, bins_prev (n int32); counters (num_bins int32)
//   support   S = ascending list of indices with bin <= k_bin (rebuilt at each binning)
//   state     one GbState struct: every scalar of the reference's host loop lives here,
//             so an iteration never returns to the host
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>

#include <atomic>

#include "../../include/gb_cs.h"

#define GB_NSLOT 16     // reduction result slots
#define GB_MAXRB 1024   // max blocks of a reducing kernel
#define GB_NFLAG 10     // predicate flags
#define GB_TILE 2048    // elements per block in the ordered compaction
#define GB_SMV_BM_MAX_N (1 << 19)  // expander A v: largest n whose support bitmap is staged
#define GB_SEL_BINS 2048  // radix-select digits per pass (11 bits)
#define GB_NSTAMP 6       // timing variants: stamps per iteration (see k_stamp)

// predicate flags (GbState::flags)
enum {
  F_ALWAYS = 0,  // constant 1
  F_DOBIN = 1,   // binning happens this iteration (minVal <= maxChange)
  F_UCG = 2,     // CGIHT: unrestricted CG step this iteration
  F_RCG = 3,     // CGIHT: restricted CG step this iteration
  F_CG = 4,      // HTP: inner CG loop running
  F_REMASK = 5,  // CGIHT: support changed, re-restrict the search direction
  F_KBIN_ALT = 6, // CSMPSP: the k-th bin scan is for the gradient (k_bin_prev), not x
  F_SORT = 7,     // timing variants, supportFlag 2/3: a new k-th largest |x| this iteration
  F_RESX = 8,     // CGIHT restricted step: the residual y - A x computed from x
  F_RESR = 9      // CGIHT restricted step: the residual by r -= alpha A p (batched, rec_every > 0)
};

// reduction slots
enum {
  R_RES = 0,   // ||resid||^2
  R_XT = 1,    // ||x_thres||^2
  R_GMAX = 2,  // max |grad| (or |grad_prev|)
  R_AXT = 3,   // ||A x_thres||^2
  R_XMAX = 4,  // max |x|
  R_DOT1 = 5,
  R_DOT2 = 6,
  R_DOT3 = 7,
  R_DOT4 = 8,
  R_CG = 9,    // HTP inner CG: ||A grad||^2
  R_SEQ_VAL = 12,  // ssmp / er argmax: block partials of the best score (ticket 12)
  R_SEQ_IDX = 13   // and of its index
};

struct GbState {
  // configuration
  int m, n, k, lda, num_bins, maxiter, alg, restart, l0_thresh, d;
  float tol;
  // loop bookkeeping (GAGA/gaga/algorithms.cu:1285-1330)
  int iter, active, fail, cycle, passes, pass_limit, status, stop_reason;
  float err, err_start, resid_diff;
  float prev[16], evol[16];
  // support selection (GAGA/gaga/functions.cu:397-436)
  int max_bin, k_bin, sum, k_bin_prev;  // k_bin_prev: CGIHT's previous k_bin, CSMPSP's gradient k_bin
  float alpha_bin, min_val, slope, max_value, max_change;
  int s_cnt;
  // CG scalars
  float mu, cg_alpha, cg_beta;
  int beta_to_zero, supp_change;
  // HTP inner CG (GAGA/gaga/algorithms.cu:2531-2540,2617-2669)
  int it_cg;
  float err_cg, tol_cg, tol2, diff_cg, prev_cg[16], evol_cg[16];
  // l0 decoding bookkeeping (GAGA/gaga/expander/parallel_l0.cu:36-60)
  int found, l0_len, l0_offset, l0_mode;  // l0_mode: 0 parallel_l0, 1 parallel_lddsr, 2 parallel_l0_swipe
  float norm, norm0, l0_diff, l0_prev[64], l0_evol[64], l0_cyc[64];
  // predicates and reduction results
  int flags[GB_NFLAG];
  double red[GB_NSLOT];
  // CGIHT support-change detection
  int changed;
  // batched form: current trial index and algorithmic operator bytes of this trial; the
  // format of the A^T r operand (GB_GRAD_*)
  int trial, op_kind;
  double bytes;
  int gfmt;
  // batched CGIHT: a restricted step whose predecessor was a restricted step on the same
  // support updates the residual as r - alpha A p (the product that step already made)
  // instead of y - A x, except every rec_every-th iteration (0: never); the support count
  // before the last binning and whether the support set is unchanged since the last step
  int rec_every, s_cnt_prev, supp_same;
  // learned warm start (CGIHT): on, gave up after 10 iterations, residual at the warm x0
  int learned, fell_back;
  float err_warm0;
  // shared-matrix CGIHT: iterations of an abandoned warm start (counted with the plain
  // restart's), a pass that only ran the restart's prologue, GEMM flops of this trial
  int warm_iters, sh_prologue;
  double sh_flops;
  // CGIHTprojected projFracTol; ALPS: the outer bin state kept across its local binning
  float proj_frac_tol, sv_alpha, sv_min_val;
  int sv_max_bin, sv_k_bin;
  // NIHT / HTP timing variants (GAGA/gaga/algorithms_timings.cu): supportFlag, whether this
  // iteration takes a new max for the bins (supportFlag 1), the sort threshold T and the
  // radix-select state of the k-th largest |x| (supportFlag 2/3)
  int timing, supp_flag, newmax, sel_need;
  unsigned int sel_prefix;
  float sort_T;
  // sequential decoders: the node picked this iteration, whether ssmp takes its periodic
  // H_k step this iteration
  int h_node, periodic;
  // expander decoders: global-timer stamp at the loop start (entry 0) and at the end of each
  // iteration (entry iter), for their cumulative time record; null when not recorded
  unsigned long long *tlog;
};

// Operator description on the device.
struct GbOp {
  int kind;  // GB_OP_DENSE / GB_OP_DCT / GB_OP_SMV
  int m, n, lda;
  const float *A;
  int vec4;  // dense: lda % 4 == 0 and A 16-byte aligned
  // dct: n = 2^logn = 2^log1 * 2^log2
  const int *rows;
  int logn, log1, log2;
  float2 *cbuf0, *cbuf1;  // complex work buffers (n)
  float *freq;            // frequency image for A^T (zero except at rows)
  // smv: column-grouped rows/vals (n*d) and a row-major (CSR) copy, columns ascending
  const int *smv_rows;
  const float *smv_vals;
  int d;
  const int *csr_ptr, *csr_col;
  const float *csr_val;
  // the operator kernels' compact copies: the column-grouped rows as 16-bit indices when
  // m <= 65536 (null otherwise), and whether every value is the one float smv_cval (then
  // neither value stream is read)
  const unsigned short *smv_r16;
  int smv_cv;
  float smv_cval;
  // dense, batched form: the A^T r operand in a compact format (gfmt != GB_GRAD_FP32): the
  // top 16 bits of each entry of A rounded to 24 (A24) or 16 (BF16) bits, and for A24 the
  // next 8 bits, both indexed like A (column j at j * lda)
  const unsigned short *A_hi;
  const unsigned char *A_lo;
  int gfmt;
};

struct GbWork {
  GbState *st;            // device state
  float *red_part;        // [GB_NSLOT][GB_MAXRB]
  unsigned int *tickets;  // [GB_NSLOT]
  float *x, *xt, *grad, *gp, *gpt;
  float *y, *resid, *ru;
  float *am1, *am2;  // FIHT / ALPS / CGIHTprojected: A x_prev, A v (or A p)
  int *bins, *bins_prev, *counters;
  int *S;        // support list (n)
  // expander, n <= GB_SMV_BM_MAX_N: bitmap of the same support (bit i % 32 of word i / 32),
  // written with S by k_compact; A v reads it when smv_bm_ok (v supported on S: every
  // gen / dct / smv algorithm's products, not the expander decoders')
  unsigned *smv_bm;
  int smv_bm_ok;
  int *tile_cnt; // per-tile counts for ordered compaction
  float *part;   // dense A x_S partial tiles (av_ntile * av_nsplit * av_rows floats)
  size_t part_cap;
  int part_two;  // part holds 2 * part_cap floats: the two-product A x_S (enq_A2) may run
  unsigned int *av_tickets;  // per row tile arrival counters
  int av_ntile, av_nsplit, av_rows;   // A x_S launch shape (row tiles of 128 or 256 rows)
  float *upd;    // l0 updates (n)
  float *rec;    // l0 residual record (maxiter + 1)
  unsigned int *sel_hist;    // timing variants: radix-select histograms (3 x GB_SEL_BINS, kept zero)
  unsigned long long *tstamp;  // timing variants: GB_NSTAMP global-timer stamps per iteration (or null)
  int *tcg;                  // timing variants: CG steps per iteration (HTP)
  unsigned long long *tlog;  // expander decoders: loop start + per-iteration end stamps (maxiter + 1)
  GbOp op;          // dimensions here are capacities when dyn is set
  int dyn;          // 1: kernels read m, n, lda, num_bins, k of the current trial from GbState
  const float *ml_params;    // learned warm start: MLP parameters (null: plain start)
  int *ml_counts, *ml_cum;   // its rank histogram (4096 bins) and prefix
  int *nonfinite;   // set when the caller's A or y holds NaN / Inf (gb_cs_solve)
  int num_sms;
  int red_blocks;   // grid of reducing kernels (fixed -> deterministic reductions)
  int wide_blocks;  // grid of the dense streaming kernels
};

void gb_set_error_message(const char *msg, const char *file, int line);

// Runs `f` (a one-time setup such as a kernel attribute, which CUDA keeps per device) once
// for the current device, from any thread; a repeat from a racing thread is harmless.
template <class F>
gb_status gb_once_per_device(std::atomic<unsigned long long> &done, F f) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) {
    gb_set_error_message("cudaGetDevice failed", __FILE__, __LINE__);
    return GB_CUDA_ERROR;
  }
  const unsigned long long bit = 1ull << (dev & 63);
  if (done.load(std::memory_order_acquire) & bit) return GB_OK;
  const gb_status rc = f();
  if (rc == GB_OK) done.fetch_or(bit, std::memory_order_release);
  return rc;
}

#define GB_CUDA_TRY(call)                                               \
  do {                                                                  \
    cudaError_t e_ = (call);                                            \
    if (e_ != cudaSuccess) {                                            \
      gb_set_error_message(cudaGetErrorString(e_), __FILE__, __LINE__); \
      return e_ == cudaErrorMemoryAllocation ? GB_OOM : GB_CUDA_ERROR;  \
    }                                                                   \
  } while (0)

#define GB_TRY(call)            \
  do {                          \
    gb_status s_ = (call);      \
    if (s_ != GB_OK) return s_; \
  } while (0)

// the expander decoders that share parallel_l0's kernels
inline bool gb_is_l0(int alg) {
  return alg == GB_ALG_PARALLEL_L0 || alg == GB_ALG_PARALLEL_LDDSR || alg == GB_ALG_PARALLEL_L0_SWIPE;
}
// the expander (CCS) decoders: smv only, unit values, a residual record
// the sequential decoders: one node per iteration (ssmp, er and their naive forms)
inline bool gb_is_seq(int alg) {
  return alg == GB_ALG_SSMP || alg == GB_ALG_ER || alg == GB_ALG_SSMP_NAIVE || alg == GB_ALG_ER_NAIVE;
}
inline bool gb_is_ccs(int alg) { return gb_is_l0(alg) || alg == GB_ALG_SMP || gb_is_seq(alg); }

// ---------------------------------------------------------------- device helpers
// Dimension arguments of the solver kernels: a value >= 0 is used as is; a negative code
// reads the current trial's dimension from GbState (the batched form reuses one captured
// graph for trials of different sizes).
enum { D_N = -1, D_M = -2, D_LDA = -3, D_NBINS = -4, D_K = -5 };
__device__ __forceinline__ int dimv(const GbState *st, int v) {
  if (v >= 0) return v;
  switch (v) {
    case D_N: return st->n;
    case D_M: return st->m;
    case D_LDA: return st->lda;
    case D_NBINS: return st->num_bins;
    default: return st->k;
  }
}

__device__ __forceinline__ bool gb_pred(const GbState *st, int flag) {
  return st->active != 0 && st->flags[flag] != 0;
}

__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ float warp_max(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

// Block reduction (OP 0 sum, 1 max); the result is valid in thread 0.
template <int OP>
__device__ __forceinline__ float block_reduce(float v, float *smem32) {
  v = OP == 0 ? warp_sum(v) : warp_max(v);
  int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) smem32[wid] = v;
  __syncthreads();
  int nw = blockDim.x >> 5;
  v = (threadIdx.x < nw) ? smem32[threadIdx.x] : 0.0f;
  if (wid == 0) v = OP == 0 ? warp_sum(v) : warp_max(v);
  return v;
}

// Grid reduction in a fixed order: every block publishes its partial, the last block to
// arrive combines the partials (sums in double) and writes st->red[slot].  All threads
// of every block must call it; the grid size must not exceed GB_MAXRB.
template <int OP>
__device__ void grid_reduce_publish(float v, int slot, GbState *st, float *parts, unsigned int *tickets) {
  __shared__ float sm[32];
  __shared__ int last;
  float b = block_reduce<OP>(v, sm);
  if (threadIdx.x == 0) {
    parts[slot * GB_MAXRB + blockIdx.x] = b;
    __threadfence();
    unsigned int t = atomicAdd(&tickets[slot], 1u);
    last = (t == gridDim.x - 1);
  }
  __syncthreads();
  if (last && threadIdx.x < 32) {
    __threadfence();
    double acc = 0.0;
    float mx = 0.0f;
    for (int i = threadIdx.x; i < (int)gridDim.x; i += 32) {
      float p = __ldcg(&parts[slot * GB_MAXRB + i]);
      if (OP == 0) acc += (double)p;
      else mx = fmaxf(mx, p);
    }
    if (OP == 0) {
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    } else {
      mx = warp_max(mx);
    }
    if (threadIdx.x == 0) {
      st->red[slot] = OP == 0 ? acc : (double)mx;
      tickets[slot] = 0u;
    }
  }
}

// host-side dimension arguments (codes when the workspace is dynamic)
inline int argN(const GbWork &w) { return w.dyn ? D_N : w.op.n; }
inline int argM(const GbWork &w) { return w.dyn ? D_M : w.op.m; }
inline int argLDA(const GbWork &w) { return w.dyn ? D_LDA : w.op.lda; }

// ---------------------------------------------------------------- host-side pieces
// operators (gb_ops.cu)
// out = A v (v must vanish outside S for the dense operator); with y, out = y - A v;
// with slot >= 0, st->red[slot] = ||out||^2.  Runs only while flag `pf` is set.
void enq_A(GbWork &w, cudaStream_t s, const float *v, float *out, const float *y, int slot, int pf);
void enq_A2(GbWork &w, cudaStream_t s, const float *v, float *out, const float *y, int slot, const float *v2,
            float *out2, int pf);
// g = A^T r
void enq_AT(GbWork &w, cudaStream_t s, const float *r, float *g, int pf);
// dense only: g = A^T r fused with xt = g on the support, ||xt||^2 and max|g|
void enq_AT_mask(GbWork &w, cudaStream_t s, const float *r, float *g, float *xt, int slot_sq, int slot_max, int pf);
// batched form: the compact A^T r operand (op.gfmt) of the current trial from op.A
void enq_split_a(GbWork &w, cudaStream_t s);
// dense A x_S launch shape for (capacity) m and its partial buffer size in floats
// rows_req 128 / 256 picks the row tile (0: 256 for a whole-GPU launch, 128 on a share of the SMs)
void gb_dense_av_shape(int m, int num_sms, bool share, int *ntile, int *nsplit, int *rows, int rows_req = 0);
size_t gb_dense_part_floats_av(int ntile, int nsplit, int rows);

// BF16 TN GEMM with FP32 accumulation (gb_gemm.cu):
//   Ct[N x M] = [Y -] (A[M x K] . B[N x K]^T)^T,  A, B row-major with row strides lda, ldb,
// optional BF16 copy Cb of Ct, or with cb_split its split [hi ; hi ; lo] (3M per column).
// With a device column map only columns c < *ncount are computed and column c stands for
// B row / Ct column nmap[c] (the batched form passes its list of active trials).  With a
// workspace, K is split over CTAs when the live tiles would leave SMs idle.
#define GB_GEMM_SPLIT_MAX 8
struct GbGemmWs {
  float *part;            // partial tiles, part_tiles units of 128 x 128 floats
  unsigned int *tickets;  // one per output tile, zero between launches
  int part_tiles, ticket_count, num_sms;
  void *gather;           // tcgen05 path with a column map: the live B rows, contiguous
  size_t gather_elems;
};
struct GbGemm {
  const void *A, *B;
  float *Ct;
  int M, N, K, lda, ldb;
  const float *Y;
  void *Cb;
  int cb_split;
  const int *nmap, *ncount;
  const GbGemmWs *ws;
  int split_rows;  // tcgen05 kernel: the split-K count from the row tiles alone, so that every
                   // 256-column block of the call is summed as a one-block call would sum it
};
gb_status gb_gemm(const GbGemm &g, cudaStream_t s);
// tcgen05 + TMA kernel (gb_gemm_tc.cu): M % 128, N % 256, K % 64; and its error word
gb_status gb_gemm_tc(const GbGemm &g, cudaStream_t s);
gb_status gb_gemm_tc_check();
// which kernel gb_gemm uses: 1 tcgen05 (default), 0 the mma.sync kernel (GB_CS_GEMM=mma)
int gb_gemm_use_tc();

// learned warm start (gb_learned.cu): x = g . net(features) for g = A^T y held in x
void enq_learned_warm(GbWork &w, cudaStream_t s, int pf);
int gb_ml_num_params();
int gb_ml_rank_bins();

// solver (gb_solver.cu)
enum { GB_RUN_SOLVE = 0, GB_RUN_L0 = 1 };
gb_status gb_run_solver(GbWork &w, int alg, const gb_options &o, int k, cudaStream_t s, float tol_abs);
// support list S := { j : v_j != 0 } (used by the component operator entry point)
void enq_support_of_nonzeros(GbWork &w, cudaStream_t s, const float *v, int n);

// pieces of a solve (gb_solver.cu), composed into larger graphs by the batched form
struct SolvePlan {
  GbWork *w;
  int alg, k, num_bins;
  int supp_flag = 0;  // NIHT / HTP timing variants: supportFlag (2, 3: sort-based support)
};
void enq_prologue(SolvePlan &P, cudaStream_t s0, cudaGraphConditionalHandle h_outer);
void enq_body(SolvePlan &P, cudaStream_t s1, cudaGraphConditionalHandle h_outer);
void enq_cg_body(SolvePlan &P, cudaStream_t s2, cudaGraphConditionalHandle h_inner, int stop_phase = -1);
void enq_ctrl_phase(GbWork &w, cudaStream_t s, int phase, cudaGraphConditionalHandle h);
void enq_stamp(GbWork &w, cudaStream_t s, int which, int which2 = -1);
gb_status gb_make_handle(cudaStream_t parent, cudaGraphConditionalHandle *h);
gb_status gb_open_while(cudaStream_t parent, cudaStream_t body, cudaGraphConditionalHandle h);
gb_status gb_close_while(cudaStream_t body);
enum { GB_PHASE_HTP_CGINIT = 1000, GB_PHASE_HTP_STOP = 1001 };
// the compact A^T r operand (GB_GRAD_A24 / GB_GRAD_BF16): b rounded to nearest even at bit
// `drop` (8: 24-bit entries, 16: BF16), the dropped bits zero
__device__ __forceinline__ uint32_t round_top_bits(uint32_t b, int drop) {
  const uint32_t half = (1u << (drop - 1)) - 1u;
  return (b + half + ((b >> drop) & 1u)) & ~((1u << drop) - 1u);
}

// entry pair (2q, 2q+1) of a 32-bit word of high parts and the low bytes l0, l1
__device__ __forceinline__ float dec_lo(uint32_t w, uint32_t l) { return __uint_as_float((w << 16) | (l << 8)); }
__device__ __forceinline__ float dec_hi(uint32_t w, uint32_t l) {
  return __uint_as_float((w & 0xffff0000u) | (l << 8));
}

// 8 consecutive rows of one column: hi (16 bytes) and lo (8 bytes, LO only) decoded into a
__device__ __forceinline__ void dec8(const uint4 h, const uint2 l, float (&a)[8], bool lo) {
  const uint32_t l0 = lo ? l.x : 0u, l1 = lo ? l.y : 0u;
  a[0] = dec_lo(h.x, l0 & 0xffu);
  a[1] = dec_hi(h.x, (l0 >> 8) & 0xffu);
  a[2] = dec_lo(h.y, (l0 >> 16) & 0xffu);
  a[3] = dec_hi(h.y, l0 >> 24);
  a[4] = dec_lo(h.z, l1 & 0xffu);
  a[5] = dec_hi(h.z, (l1 >> 8) & 0xffu);
  a[6] = dec_lo(h.w, (l1 >> 16) & 0xffu);
  a[7] = dec_hi(h.w, l1 >> 24);
}

__device__ __forceinline__ float dec1(const unsigned short *hi, const unsigned char *lo, size_t e, bool has_lo) {
  return __uint_as_float(((uint32_t)hi[e] << 16) | (has_lo ? (uint32_t)lo[e] << 8 : 0u));
}

// per-iteration algorithmic operator bytes of the dense operator (survey formula):
// A^T r: b mn + 4m + 4n (b = 4 bytes per entry of A, 3 or 2 in the compact A^T formats) ;
// A x_S: 4 m s + 8 s + 4 m
__device__ __forceinline__ double dense_bytes(const GbState *st, int n_at, int n_a) {
  const double m = st->m, n = st->n, s = st->s_cnt;
  const double b = st->gfmt == GB_GRAD_A24 ? 3.0 : st->gfmt == GB_GRAD_BF16 ? 2.0 : 4.0;
  return n_at * (b * m * n + 4.0 * m + 4.0 * n) + n_a * (4.0 * m * s + 8.0 * s + 4.0 * m);
}
