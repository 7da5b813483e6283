// gb_solver.cu -- NIHT / HTP / CGIHT and parallel_l0 as one CUDA graph per solve.
//
// The reference runs each algorithm as a host loop that returns to the host several
// times per iteration (cuBLAS v1 scalars, bin counters, flags).  Here every scalar of
// that loop lives in a device-resident GbState; small single-thread "control" kernels
// execute the reference's scalar logic; every other kernel is predicated on
// GbState::active and a flag.  One iteration is captured into the body of a CUDA graph
// WHILE node whose condition the last control kernel sets from the stopping rules, so
// a whole solve is a single graph launch.
#include <stdlib.h>
#include <string.h>

#include "gb_internal.cuh"
#include "gb_resident.h"

#include "gb_ctrl.cuh"

__global__ void k_ctrl(GbState *st, int phase, cudaGraphConditionalHandle h) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  ctrl_phase(st, phase, h);
}

// ------------------------------------------------------------------ l0 control
// the time record of the expander decoders (timeRecord of GAGA/gaga/expander/*.cu): the
// global timer when the loop starts and as each iteration ends
__device__ __forceinline__ void tlog_mark(GbState *st) {
  if (st->tlog && st->iter >= 0 && st->iter <= st->maxiter) {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    st->tlog[st->iter] = t;
  }
}

__global__ void k_ctrl_l0(GbState *st, int phase, float *rec, cudaGraphConditionalHandle h) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  const int L = st->l0_len;
  const int iter0 = st->iter;
  switch (phase) {
    case C_L0_INIT:
      // parallel_l0 (GAGA/gaga/expander/parallel_l0.cu:31-60)
      st->norm = sqrt_red(st, R_RES);
      st->norm0 = st->norm;
      if (rec) rec[0] = st->norm;
      for (int i = 0; i < L; ++i) { st->l0_cyc[i] = 0.0f; st->l0_prev[i] = 0.0f; st->l0_evol[i] = 1.0f; }
      st->l0_diff = 1.0f;
      st->found = 1;
      if (st->l0_mode == 2) st->l0_thresh = st->d - 1;  // parallel_l0_swipe.cu:11
      st->active = (st->iter < st->maxiter) & (st->norm > st->tol) & (st->norm < (100.0f * st->norm0)) &
                   ((double)st->l0_diff > 0.000001) & (st->cycle != 0) & (st->found == 1) &
                   (st->l0_mode != 2 || st->l0_thresh > 0);
      set_cond(h, st->active ? 1u : 0u);
      break;
    case C_SMP_INIT:
      // smp.cu:45-66: res = y - A x^0, err, records
      st->err = sqrt_red(st, R_RES);
      st->err_start = st->err;
      if (rec) rec[0] = st->err;
      for (int j = 0; j < 16; ++j) { st->prev[j] = 0.0f; st->evol[j] = 1.0f; }
      st->resid_diff = 1.0f;
      st->active = (st->iter < st->maxiter) & (st->err > st->tol) & (st->err < 100.0f * st->err_start) &
                   ((double)st->resid_diff > 0.01 * (double)st->tol) & (st->fail == 0);
      set_cond(h, st->active ? 1u : 0u);
      break;
    case C_SMP_HK:
      if (!st->active) break;
      // H_k (expander/functions.cu:125-144): maxChange = 2 max, minVal 0, alpha 0.25,
      // MaxBin = num_bins, a forced binning
      st->max_value = (float)st->red[R_XMAX];
      st->max_change = 2.0f * st->max_value;
      st->slope = ((float)(st->num_bins - 1) / st->max_value);
      st->min_val = 0.0f;
      st->alpha_bin = 0.25f;
      st->max_bin = st->num_bins;
      st->flags[F_DOBIN] = 1;
      break;
    case C_SMP_STOP:
      if (st->active) {
        st->err = sqrt_red(st, R_RES);
        for (int j = 0; j < 15; ++j) { st->prev[j] = st->prev[j + 1]; st->evol[j] = st->evol[j + 1]; }
        st->prev[15] = st->err;
        st->evol[15] = st->prev[14] - st->prev[15];
        st->resid_diff = max_list(st->evol, 16);
        if (st->iter > (int)(0.4 * st->maxiter)) {
          float rate = powf(st->prev[15] / st->prev[0], 1.0f / 15.0f);
          if (rate > 0.999f) st->fail = 1;
        }
        st->iter++;
        st->passes++;
        if (rec) rec[st->iter] = st->err;
        const int go = (st->iter < st->maxiter) & (st->err > st->tol) & (st->err < 100.0f * st->err_start) &
                       ((double)st->resid_diff > 0.01 * (double)st->tol) & (st->fail == 0);
        if (!go) {
          if (!(st->err > st->tol)) st->stop_reason = 1;
          else if (!(st->iter < st->maxiter)) st->stop_reason = 2;
          else if (!(st->err < 100.0f * st->err_start)) st->stop_reason = 3;
          else if (!((double)st->resid_diff > 0.01 * (double)st->tol)) st->stop_reason = 4;
          else st->stop_reason = 6;
        }
        st->active = go;
        if (st->passes > st->pass_limit && st->active) {
          st->active = 0;
          st->status = GB_WATCHDOG;
        }
      }
      set_cond(h, st->active ? 1u : 0u);
      break;
    case C_SEQ_INIT: {
      // ssmp.cu:56-81 / er.cu:43-68: res = y - A x^0, err, records
      st->err = sqrt_red(st, R_RES);
      st->err_start = st->err;
      if (rec) rec[0] = st->err;
      for (int j = 0; j < 16; ++j) { st->prev[j] = 0.0f; st->evol[j] = 1.0f; }
      for (int i = 0; i < L; ++i) st->l0_cyc[i] = 0.0f;
      st->resid_diff = 1.0f;
      st->cycle = 1;
      const bool er = st->alg == GB_ALG_ER || st->alg == GB_ALG_ER_NAIVE;
      st->active = (st->iter < st->maxiter) & (st->err > st->tol) & (st->err < 100.0f * st->err_start) &
                   (er ? 1 : ((double)st->resid_diff > 0.01 * (double)st->tol));
      set_cond(h, st->active ? 1u : 0u);
      break;
    }
    case C_SEQ_STOP:
      if (st->active) {
        const bool er = st->alg == GB_ALG_ER || st->alg == GB_ALG_ER_NAIVE;
        st->err = sqrt_red(st, R_RES);
        int cycling = 0;
        if (er) {
          // er.cu:97-110: the last 2p residuals alternate between two values (er only)
          st->iter++;
          for (int i = 0; i < L - 1; ++i) st->l0_cyc[i] = st->l0_cyc[i + 1];
          st->l0_cyc[L - 1] = st->err;
          if (st->alg == GB_ALG_ER && st->iter > L) {
            cycling = 1;
            for (int i = 3; i < L; i += 2) cycling = cycling * (st->l0_cyc[i] == st->l0_cyc[i - 2]);
          }
          st->cycle = cycling ? 0 : 1;
        } else {
          // ssmp.cu:124-131: residual history
          for (int j = 0; j < 15; ++j) { st->prev[j] = st->prev[j + 1]; st->evol[j] = st->evol[j + 1]; }
          st->prev[15] = st->err;
          st->evol[15] = st->prev[14] - st->prev[15];
          st->resid_diff = max_list(st->evol, 16);
          st->iter++;
        }
        st->passes++;
        if (rec) rec[st->iter] = st->err;
        const int go = (st->iter < st->maxiter) & (st->err > st->tol) & (st->err < 100.0f * st->err_start) &
                       (er ? (cycling == 0) : ((double)st->resid_diff > 0.01 * (double)st->tol));
        if (!go) {
          if (!(st->err > st->tol)) st->stop_reason = 1;
          else if (!(st->iter < st->maxiter)) st->stop_reason = 2;
          else if (!(st->err < 100.0f * st->err_start)) st->stop_reason = 3;
          else if (er) st->stop_reason = 5;
          else st->stop_reason = 4;
        }
        st->active = go;
        if (st->passes > st->pass_limit && st->active) {
          st->active = 0;
          st->status = GB_WATCHDOG;
        }
      }
      set_cond(h, st->active ? 1u : 0u);
      break;
    case C_SEQ_END1:
      st->active = 1;
      break;
    case C_SEQ_END2:
      st->active = 0;
      break;
    case C_L0_PRE:
      if (!st->active) break;
      st->l0_offset = st->iter % st->d;
      st->found = 0;
      break;
    case C_L0_STOP:
      if (st->active && st->l0_mode == 2 && st->found == 0 && st->l0_thresh > 0) {
        // parallel_l0_swipe: no column qualified; lower the threshold, keep the residual
        // history (parallel_l0_swipe.cu:82-85)
        st->l0_thresh--;
        st->found = 1;
        st->iter++;
        st->passes++;
        if (rec) rec[st->iter] = st->norm;
        const int go = (st->iter < st->maxiter) & (st->norm > st->tol) & (st->norm < (100.0f * st->norm0)) &
                       ((double)st->l0_diff > 0.000001) & (st->cycle != 0) & (st->l0_thresh > 0);
        if (!go) st->stop_reason = !(st->iter < st->maxiter) ? 2 : 7;
        st->active = go;
        if (st->passes > st->pass_limit && st->active) {
          st->active = 0;
          st->status = GB_WATCHDOG;
        }
      } else if (st->active) {
        st->norm = sqrt_red(st, R_RES);
        for (int i = 0; i < L - 1; ++i) st->l0_prev[i] = st->l0_prev[i + 1];
        st->l0_prev[L - 1] = st->norm;
        for (int i = 0; i < L - 1; ++i) st->l0_evol[i] = st->l0_evol[i + 1];
        st->l0_evol[L - 1] = st->l0_prev[L - 2] - st->l0_prev[L - 1];
        st->l0_diff = max_list(st->l0_evol, L);
        for (int i = 0; i < L - 1; ++i) st->l0_cyc[i] = st->l0_cyc[i + 1];
        st->l0_cyc[L - 1] = st->norm;
        int cycling = 0;
        if (st->iter > L) {
          cycling = 1;
          for (int i = 3; i < L; i += 2) cycling = cycling * (st->l0_cyc[i] == st->l0_cyc[i - 2]);
        }
        st->cycle = cycling ? 0 : 1;
        st->iter++;
        st->passes++;
        if (rec) rec[st->iter] = st->norm;
        int go = (st->iter < st->maxiter) & (st->norm > st->tol) & (st->norm < (100.0f * st->norm0)) &
                 ((double)st->l0_diff > 0.000001) & (cycling == 0) & (st->found == 1) &
                 (st->l0_mode != 2 || st->l0_thresh > 0);
        if (!go) {
          if (!(st->norm > st->tol)) st->stop_reason = 1;
          else if (!(st->iter < st->maxiter)) st->stop_reason = 2;
          else if (!(st->norm < 100.0f * st->norm0)) st->stop_reason = 3;
          else if (!((double)st->l0_diff > 0.000001)) st->stop_reason = 4;
          else if (cycling) st->stop_reason = 5;
          else st->stop_reason = 7;
        }
        st->active = go;
        if (st->passes > st->pass_limit && st->active) {
          st->active = 0;
          st->status = GB_WATCHDOG;
        }
      }
      set_cond(h, st->active ? 1u : 0u);
      break;
  }
  // the loop start, and each finished iteration
  if (phase == C_L0_INIT || phase == C_SMP_INIT || phase == C_SEQ_INIT || st->iter != iter0) tlog_mark(st);
}

// ------------------------------------------------------------------ vector kernels
// dst_i = src_i if bin_i <= k_bin else 0 (zero_vector_float + threshold_one,
// GAGA/gaga/kernels.cu:64-71); optional ||dst||^2 and max|src|
__global__ void k_mask(GbState *st, int pf, const float *__restrict__ src, float *__restrict__ dst,
                       const int *__restrict__ bins, int n, int slot_sq, int slot_max, float *rp,
                       unsigned int *tk) {
  if (!gb_pred(st, pf)) return;
  n = dimv(st, n);
  const int kb = st->k_bin;
  float s2 = 0.0f, mx = 0.0f;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const float v = src[i];
    const float o = bins[i] <= kb ? v : 0.0f;
    dst[i] = o;
    s2 = fmaf(o, o, s2);
    mx = fmaxf(mx, fabsf(v));
  }
  if (slot_sq >= 0) grid_reduce_publish<0>(s2, slot_sq, st, rp, tk);
  if (slot_max >= 0) grid_reduce_publish<1>(mx, slot_max, st, rp, tk);
}

// v_i = 0 where bin_i > k_bin (threshold, GAGA/gaga/kernels.cu:74-81)
__global__ void k_threshold(const GbState *st, int pf, float *__restrict__ v, const int *__restrict__ bins, int n) {
  if (!gb_pred(st, pf)) return;
  n = dimv(st, n);
  const int kb = st->k_bin;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    if (bins[i] > kb) v[i] = 0.0f;
}

// scalar selector for the fused updates
enum { SC_MU = 0, SC_CG_ALPHA = 1, SC_NEG_CG_ALPHA = 2, SC_CG_BETA = 3, SC_ONE = 4, SC_NEG_ONE = 5 };
__device__ __forceinline__ float pick(const GbState *st, int which) {
  switch (which) {
    case SC_MU: return st->mu;
    case SC_CG_ALPHA: return st->cg_alpha;
    case SC_NEG_CG_ALPHA: return -st->cg_alpha;
    case SC_CG_BETA: return st->cg_beta;
    case SC_NEG_ONE: return -1.0f;
    default: return 1.0f;
  }
}

// y += a * x (cublasSaxpy); optional max|y| and ||y||^2; optionally clears the bin counters
__global__ void k_axpy(GbState *st, int pf, int which, const float *__restrict__ x, float *__restrict__ y, int n,
                       int slot_max, int slot_sq, int *counters, int ncount, float *rp, unsigned int *tk) {
  if (!gb_pred(st, pf)) return;
  n = dimv(st, n);
  ncount = dimv(st, ncount);
  const float a = pick(st, which);
  float mx = 0.0f, s2 = 0.0f;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const float o = fmaf(a, x[i], y[i]);
    y[i] = o;
    mx = fmaxf(mx, fabsf(o));
    s2 = fmaf(o, o, s2);
  }
  if (counters)
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < ncount; i += gridDim.x * blockDim.x) counters[i] = 0;
  if (slot_max >= 0) grid_reduce_publish<1>(mx, slot_max, st, rp, tk);
  if (slot_sq >= 0) grid_reduce_publish<0>(s2, slot_sq, st, rp, tk);
}

// out = a + c b (cublasSaxpy form: one fused multiply-add), or out = a without b; the
// optional reductions give sum(out * dv) and sum(out^2).  out may alias a or b.
__global__ void k_lin(GbState *st, int pf, float *out, const float *a, int which, const float *b, int n,
                      const float *dv, int slot_dot, int slot_sq, float *rp, unsigned int *tk) {
  if (!gb_pred(st, pf)) return;
  n = dimv(st, n);
  const float c = pick(st, which);
  float d = 0.0f, q = 0.0f;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const float o = b ? fmaf(c, b[i], a[i]) : a[i];
    out[i] = o;
    if (dv) d = fmaf(o, dv[i], d);
    q = fmaf(o, o, q);
  }
  if (slot_dot >= 0) grid_reduce_publish<0>(d, slot_dot, st, rp, tk);
  if (slot_sq >= 0) grid_reduce_publish<0>(q, slot_sq, st, rp, tk);
}

// The reference's flag thresholds (GAGA/gaga/kernels.cu:32-61): mode 0 out = flag != 0 ? in : 0
// (a copy then threshold_two), mode 1 out = flag == 0 ? in : 0 (zero then threshold_three),
// mode 2 out = flag != 0 ? in : out (threshold_four)
__global__ void k_flagmask(const GbState *st, int pf, float *out, const float *in, const float *flag, int mode, int n) {
  if (!gb_pred(st, pf)) return;
  n = dimv(st, n);
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const bool f = flag[i] != 0.0f;
    if (mode == 0) out[i] = f ? in[i] : 0.0f;
    else if (mode == 1) out[i] = f ? 0.0f : in[i];
    else if (f) out[i] = in[i];
  }
}

// a = beta * a + b (cublasSscal then cublasSaxpy with 1)
__global__ void k_scale_add(const GbState *st, int pf, int which, float *__restrict__ a, const float *__restrict__ b,
                            int n) {
  if (!gb_pred(st, pf)) return;
  n = dimv(st, n);
  const float beta = pick(st, which);
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const float t = beta * a[i];
    a[i] = fmaf(1.0f, b[i], t);
  }
}

// two dot products in one pass: red[s1] = a.b, red[s2] = c.d
__global__ void k_dot2(GbState *st, int pf, const float *__restrict__ a, const float *__restrict__ b, int s1, int n1,
                       const float *__restrict__ c, const float *__restrict__ d, int s2, int n2, float *rp,
                       unsigned int *tk) {
  if (!gb_pred(st, pf)) return;
  n1 = dimv(st, n1);
  n2 = dimv(st, n2);
  float p = 0.0f, q = 0.0f;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n1; i += gridDim.x * blockDim.x) p = fmaf(a[i], b[i], p);
  if (c)
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n2; i += gridDim.x * blockDim.x) q = fmaf(c[i], d[i], q);
  grid_reduce_publish<0>(p, s1, st, rp, tk);
  if (c) grid_reduce_publish<0>(q, s2, st, rp, tk);
}

// dst = src; red[slot] = ||src||^2 ; optional max|src|
__global__ void k_copy_norm(GbState *st, int pf, const float *__restrict__ src, float *__restrict__ dst, int n,
                            int slot_sq, int slot_max, float *rp, unsigned int *tk) {
  if (!gb_pred(st, pf)) return;
  n = dimv(st, n);
  float s2 = 0.0f, mx = 0.0f;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const float v = src[i];
    if (dst) dst[i] = v;
    s2 = fmaf(v, v, s2);
    mx = fmaxf(mx, fabsf(v));
  }
  if (slot_sq >= 0) grid_reduce_publish<0>(s2, slot_sq, st, rp, tk);
  if (slot_max >= 0) grid_reduce_publish<1>(mx, slot_max, st, rp, tk);
}

// ------------------------------------------------------------------ support selection
__global__ void k_hist(const GbState *st, int pf, const float *__restrict__ v, int *__restrict__ bins,
                       int *__restrict__ bins_prev, int *__restrict__ counters, int n) {
  if (!gb_pred(st, pf)) return;
  n = dimv(st, n);
  const float intercept = st->max_value;
  const float slope = st->slope;
  const float small_f = __double2float_rd((double)intercept * 0.000001);
  const int max_bin = st->max_bin;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    bool counted;
    const int b = lin_bin(v[i], slope, intercept, small_f, counted);
    if (bins_prev) bins_prev[i] = bins[i];
    bins[i] = b;
    if (counted && b < max_bin) {
      // warp-aggregated increment of equal bins
      const unsigned act = __activemask();
      const unsigned same = __match_any_sync(act, b);
      const int leader = __ffs(same) - 1;
      if ((int)(threadIdx.x & 31) == leader) atomicAdd(&counters[b], __popc(same));
    }
  }
}

// k-th largest bin: the reference copies the first MaxBin counters to the host and scans
// (GAGA/gaga/functions.cu:412-433).  One block of 1024 threads does the same scan: thread t
// sums a contiguous run of C bins (its loads issued KB_BATCH at a time, so a run costs a
// few memory trips, not C), a shuffle scan over the 1024 run sums finds the run where the
// count reaches k, and that run's thread walks it bin by bin (the same batches, now hitting
// L1).  Integer sums: the result is the sequential scan's.
#define KB_BATCH 16
__global__ void __launch_bounds__(1024) k_kbin(GbState *st, int pf, const int *__restrict__ counters, int k) {
  if (!gb_pred(st, pf)) return;
  k = dimv(st, k);
  __shared__ int wsum[32];
  __shared__ int res_kbin, res_sum, total;
  const int max_bin = st->max_bin;
  const int C = (max_bin + 1023) / 1024;
  const int t = threadIdx.x, lane = t & 31, wid = t >> 5;
  const int b0 = min(t * C, max_bin), b1 = min(b0 + C, max_bin);
  int csum = 0;
  for (int b = b0; b < b1; b += KB_BATCH) {
    int v[KB_BATCH];
#pragma unroll
    for (int u = 0; u < KB_BATCH; ++u) v[u] = b + u < b1 ? counters[b + u] : 0;
#pragma unroll
    for (int u = 0; u < KB_BATCH; ++u) csum += v[u];
  }
  if (t == 0) { res_kbin = -2; res_sum = 0; }
  // inclusive scan of csum over the block: in each warp, then over the warp totals
  int incl = csum;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += y;
  }
  if (lane == 31) wsum[wid] = incl;
  __syncthreads();
  if (wid == 0) {
    int ws = wsum[lane];
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, ws, o);
      if (lane >= o) ws += y;
    }
    wsum[lane] = ws;  // inclusive over warps
    if (lane == 31) total = ws;
  }
  __syncthreads();
  incl += wid > 0 ? wsum[wid - 1] : 0;
  const int excl = incl - csum;
  if (k > 0 && excl < k && incl >= k) {  // exactly one thread
    int s = excl;
    bool found = false;
    for (int b = b0; b < b1 && !found; b += KB_BATCH) {
      int v[KB_BATCH];
#pragma unroll
      for (int u = 0; u < KB_BATCH; ++u) v[u] = b + u < b1 ? counters[b + u] : 0;
#pragma unroll
      for (int u = 0; u < KB_BATCH; ++u) {
        if (!found && b + u < b1) {
          s += v[u];
          if (s >= k) { res_kbin = b + u; res_sum = s; found = true; }
        }
      }
    }
  }
  __syncthreads();
  if (t == 0) {
    int k_bin, sum;
    if (k <= 0) { k_bin = -1; sum = 0; }
    else if (res_kbin == -2) { k_bin = max_bin - 1; sum = total; }
    else { k_bin = res_kbin; sum = res_sum; }
    const float intercept = st->max_value;
    const float slope = st->slope;
    if (sum < k) {
      st->alpha_bin = st->alpha_bin * 0.5f;
      st->max_bin = (int)((float)st->num_bins * (1.0f - st->alpha_bin));
    }
    st->min_val = intercept - (float)(k_bin + 1) / slope;
    if (st->flags[F_KBIN_ALT]) st->k_bin_prev = k_bin;
    else st->k_bin = k_bin;
    st->sum = sum;
  }
}

// joinSupports (GAGA/gaga/kernels.cu:162-172): entries in the gradient's top bins join the
// support of x (their bin becomes k_bin)
__global__ void k_join(const GbState *st, int *__restrict__ bins, const int *__restrict__ bins_grad, int n) {
  if (!gb_pred(st, F_ALWAYS)) return;
  n = dimv(st, n);
  const int kb = st->k_bin, kbg = st->k_bin_prev;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    if (bins_grad[i] <= kbg && bins[i] > kb) bins[i] = kb;
}

// threshold v (always) and, when binning, count the tile's support entries and detect
// whether a previous support entry left the support (checkSupportEvolution,
// GAGA/gaga/kernels.cu:178-193, without its block-local flag reset race)
__global__ void __launch_bounds__(256) k_thresh_count(GbState *st, int pf, float *__restrict__ v,
                                                      const int *__restrict__ bins, const int *__restrict__ bins_prev,
                                                      int n, int *__restrict__ tile_cnt) {
  if (!gb_pred(st, pf)) return;
  n = dimv(st, n);
  const int kb = st->k_bin, kbp = st->k_bin_prev;
  const bool count = st->flags[F_DOBIN] != 0;
  const int base = blockIdx.x * GB_TILE;
  int cnt = 0, changed = 0;
  for (int q = threadIdx.x; q < GB_TILE; q += blockDim.x) {
    const int i = base + q;
    if (i < n) {
      const int b = bins[i];
      if (b > kb) {
        if (v) v[i] = 0.0f;
      } else {
        cnt++;
      }
      if (bins_prev && count && bins_prev[i] <= kbp && b > kb) changed = 1;
    }
  }
  if (!count) return;
  __shared__ float sm[32];
  const float tot = block_reduce<0>((float)cnt, sm);
  if (threadIdx.x == 0) tile_cnt[blockIdx.x] = (int)tot;
  if (bins_prev && __syncthreads_or(changed) && threadIdx.x == 0) atomicOr(&st->changed, 1);
}

// ordered compaction: S = ascending { i : bin_i <= k_bin }; with bm, the same set as a bitmap
__global__ void __launch_bounds__(256) k_compact(GbState *st, int pf, const int *__restrict__ bins, int n,
                                                 const int *__restrict__ tile_cnt, int *__restrict__ S,
                                                 unsigned *__restrict__ bm) {
  if (!gb_pred(st, pf)) return;
  n = dimv(st, n);
  __shared__ float sm[32];
  __shared__ int warp_base[8];
  const int kb = st->k_bin;
  // offset of this tile = sum of the previous tiles' counts
  float off = 0.0f;
  for (int t = threadIdx.x; t < (int)blockIdx.x; t += blockDim.x) off += (float)tile_cnt[t];
  int offset = (int)block_reduce<0>(off, sm);
  __shared__ int s_off;
  if (threadIdx.x == 0) s_off = offset;
  __syncthreads();
  int running = s_off;
  const int base = blockIdx.x * GB_TILE;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  for (int q0 = 0; q0 < GB_TILE; q0 += blockDim.x) {
    const int i = base + q0 + threadIdx.x;
    const bool in = i < n && bins[i] <= kb;
    const unsigned bal = __ballot_sync(0xffffffffu, in);
    if (lane == 0) warp_base[wid] = __popc(bal);
    if (bm && lane == 0) bm[i >> 5] = bal;  // i - lane is a multiple of 32
    __syncthreads();
    int wb = 0, tot = 0;
    for (int w2 = 0; w2 < 8; ++w2) {
      if (w2 < wid) wb += warp_base[w2];
      tot += warp_base[w2];
    }
    if (in) S[running + wb + __popc(bal & ((1u << lane) - 1u))] = i;
    running += tot;
    __syncthreads();
  }
  if (blockIdx.x == gridDim.x - 1 && threadIdx.x == 0) st->s_cnt = running;
}

// ------------------------------------------------------------------ sort-based support
// The timing variants' supportFlag 2/3 (FindSupportSet_sort, GAGA/gaga/functions.cu:446-465)
// threshold at T = the k-th largest |x|, which the reference reads from a full thrust::sort
// of |x| (element n-k of the ascending order).  Here T comes from a three-pass radix select
// over the bits of |x| (bit 31 is 0; digits of bits 30..21, 20..10, 9..0): each pass
// histograms the digit of the entries whose higher bits match the prefix chosen so far,
// then one block picks the digit where the count from the top reaches k.  Integer counts,
// so T is exactly the sorted element and the result does not depend on the grid.
__device__ __forceinline__ void sel_digit(int pass, int *shift, int *width) {
  *shift = pass == 0 ? 21 : pass == 1 ? 10 : 0;
  *width = pass == 1 ? 11 : 10;
}

__global__ void __launch_bounds__(256) k_sel_hist(const GbState *st, const float *__restrict__ v, int n,
                                                  unsigned int *__restrict__ hist, int pass) {
  if (!gb_pred(st, F_SORT)) return;
  __shared__ unsigned int h[GB_SEL_BINS];
  for (int i = threadIdx.x; i < GB_SEL_BINS; i += blockDim.x) h[i] = 0u;
  __syncthreads();
  int shift, width;
  sel_digit(pass, &shift, &width);
  const int hs = shift + width;  // the bits above this pass's digit
  const unsigned int prefix = st->sel_prefix >> hs, mask = (1u << width) - 1u;
  const int lane = threadIdx.x & 31;
  // i0 is uniform in the block, so every lane of a warp takes part in each match
  for (int i0 = blockIdx.x * blockDim.x; i0 < n; i0 += gridDim.x * blockDim.x) {
    const int i = i0 + threadIdx.x;
    unsigned int key = 0xffffffffu;
    if (i < n) {
      const unsigned int u = __float_as_uint(v[i]) & 0x7fffffffu;
      if (hs >= 31 || (u >> hs) == prefix) key = (u >> shift) & mask;
    }
    const unsigned int peers = __match_any_sync(0xffffffffu, key);
    if (key != 0xffffffffu && lane == __ffs(peers) - 1) atomicAdd(&h[key], (unsigned int)__popc(peers));
  }
  __syncthreads();
  for (int i = threadIdx.x; i < GB_SEL_BINS; i += blockDim.x)
    if (h[i]) atomicAdd(&hist[i], h[i]);
}

// one block of 1024 threads: thread t owns digits 2047-2t and 2046-2t (descending order);
// picks the digit, narrows the prefix and the remaining count, and zeroes its histogram
__global__ void __launch_bounds__(1024) k_sel_scan(GbState *st, unsigned int *__restrict__ hist, int pass) {
  if (!gb_pred(st, F_SORT)) return;
  int shift, width;
  sel_digit(pass, &shift, &width);
  const int t = threadIdx.x, lane = t & 31, wid = t >> 5;
  const int d0 = GB_SEL_BINS - 1 - 2 * t, d1 = d0 - 1;
  const unsigned int c0 = hist[d0], c1 = hist[d1];
  long long need;
  if (pass == 0) {
    const int n = st->n;
    need = st->k < 1 ? 1 : (st->k > n ? n : st->k);
  } else {
    need = st->sel_need;
  }
  const unsigned int prefix = pass == 0 ? 0u : st->sel_prefix;
  // exclusive scan of c0 + c1 over the threads
  unsigned long long x = (unsigned long long)c0 + c1, inc = x;
  for (int o = 1; o < 32; o <<= 1) {
    const unsigned long long y = __shfl_up_sync(0xffffffffu, inc, o);
    if (lane >= o) inc += y;
  }
  __shared__ unsigned long long wsum[32];
  if (lane == 31) wsum[wid] = inc;
  __syncthreads();
  if (wid == 0) {
    unsigned long long ws = wsum[lane], wi = ws;
    for (int o = 1; o < 32; o <<= 1) {
      const unsigned long long y = __shfl_up_sync(0xffffffffu, wi, o);
      if (lane >= o) wi += y;
    }
    wsum[lane] = wi - ws;  // exclusive over warps
  }
  __syncthreads();
  const long long before = (long long)(wsum[wid] + inc - x);
  int digit = -1;
  long long rest = 0;
  if (before < need && need <= before + (long long)c0) {
    digit = d0;
    rest = need - before;
  } else if (before + (long long)c0 < need && need <= before + (long long)c0 + (long long)c1) {
    digit = d1;
    rest = need - before - (long long)c0;
  }
  if (digit >= 0) {
    const unsigned int np = prefix | ((unsigned int)digit << shift);
    st->sel_prefix = np;
    st->sel_need = (int)rest;
    if (pass == 2) st->sort_T = __uint_as_float(np);
  }
  hist[d0] = 0u;
  hist[d1] = 0u;
}

// threshold_and_support (GAGA/gaga/kernels.cu:85-95) at T, after one_vector_int when a
// new T was selected: |x| < T -> x = 0, bin 2; else bin 1 on a new T (bins of survivors of a
// lowered T stay as they were).  Counts each tile's survivors for the support list.
__global__ void __launch_bounds__(256) k_sort_thresh(GbState *st, float *__restrict__ v, int *__restrict__ bins,
                                                     int n, int *__restrict__ tile_cnt) {
  if (!gb_pred(st, F_ALWAYS)) return;
  const bool reset = st->flags[F_SORT] != 0;
  const float T = st->sort_T;
  const int base = blockIdx.x * GB_TILE;
  int cnt = 0;
  for (int q = threadIdx.x; q < GB_TILE; q += blockDim.x) {
    const int i = base + q;
    if (i < n) {
      if (fabsf(v[i]) < T) {
        v[i] = 0.0f;
        bins[i] = 2;
      } else {
        if (reset) bins[i] = 1;
        cnt++;
      }
    }
  }
  __shared__ float sm[32];
  const float tot = block_reduce<0>((float)cnt, sm);
  if (threadIdx.x == 0) tile_cnt[blockIdx.x] = (int)tot;
}

// S = ascending { i : |x_i| >= T } after the threshold: every nonzero of x (which can lie
// outside bins <= 1 after a lowered T) and every entry of bins <= 1, for the dense A x_S
__global__ void __launch_bounds__(256) k_sort_compact(GbState *st, const float *__restrict__ v, int n,
                                                      const int *__restrict__ tile_cnt, int *__restrict__ S) {
  if (!gb_pred(st, F_ALWAYS)) return;
  const float T = st->sort_T;
  __shared__ float sm[32];
  __shared__ int warp_base[8];
  __shared__ int s_off;
  float off = 0.0f;
  for (int t = threadIdx.x; t < (int)blockIdx.x; t += blockDim.x) off += (float)tile_cnt[t];
  const int offset = (int)block_reduce<0>(off, sm);
  if (threadIdx.x == 0) s_off = offset;
  __syncthreads();
  int running = s_off;
  const int base = blockIdx.x * GB_TILE;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  for (int q0 = 0; q0 < GB_TILE; q0 += blockDim.x) {
    const int i = base + q0 + threadIdx.x;
    const bool in = i < n && !(fabsf(v[i]) < T);
    const unsigned bal = __ballot_sync(0xffffffffu, in);
    if (lane == 0) warp_base[wid] = __popc(bal);
    __syncthreads();
    int wb = 0, tot = 0;
    for (int w2 = 0; w2 < 8; ++w2) {
      if (w2 < wid) wb += warp_base[w2];
      tot += warp_base[w2];
    }
    if (in) S[running + wb + __popc(bal & ((1u << lane) - 1u))] = i;
    running += tot;
    __syncthreads();
  }
  if (blockIdx.x == gridDim.x - 1 && threadIdx.x == 0) st->s_cnt = running;
}

// Timing variants: the global timer (ns) at a point of the current iteration, into
// ts[iter * GB_NSTAMP + which] (and + which2).  Stamps: 0 iteration start, 1 support step
// start, 2 support step end, 3 CG start (HTP), 4 CG end, 5 iteration end; with the end
// stamp the HTP CG step count.  Kernels of one stream run in order, so a stamp kernel runs
// after the kernels before it have finished.
__global__ void k_stamp(const GbState *st, unsigned long long *ts, int *tcg, int which, int which2) {
  if (!st->active) return;
  const int it = st->iter;
  if (it < 0 || it >= st->maxiter) return;
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  ts[(size_t)it * GB_NSTAMP + which] = t;
  if (which2 >= 0) ts[(size_t)it * GB_NSTAMP + which2] = t;
  if (tcg && (which == GB_NSTAMP - 1 || which2 == GB_NSTAMP - 1)) tcg[it] = st->it_cg;
}

// ------------------------------------------------------------------ l0 kernels
// cuda_compute_scores_l0 (GAGA/gaga/expander/kernels.cu:353-388); the score stays a float
// counter as in the reference
__global__ void k_l0_scores(GbState *st, const float *__restrict__ res, float *__restrict__ x,
                            float *__restrict__ upd, const int *__restrict__ rows, int n, int d) {
  if (!st->active) return;
  const int thresh = st->l0_thresh;
  const int shift = st->l0_offset;
  const bool lddsr = st->l0_mode == 1;
  // cuda_compute_scores_lddsr (GAGA/gaga/expander/kernels.cu:309-345): matching rows only,
  // more than d/2 of them
  const float cut = lddsr ? ((float)d) / 2 : (float)thresh;
  const float EPS = 0.000001f;
  int found = 0;
  for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
    const size_t idx = (size_t)d * j;
    float score = 0.0f;
    const float omega = res[rows[idx + shift]];
    float u = 0.0f;
    if (fabsf(omega) > EPS) {
      for (int i = 0; i < d; ++i) {
        const float ri = res[rows[idx + i]];
        if (fabsf(__fsub_rn(ri, omega)) <= EPS) score += 1.0f;
        if (!lddsr && fabsf(ri) <= EPS) score -= 1.0f;
      }
      if (score > cut) {
        found = 1;
        x[j] = __fadd_rn(x[j], omega);
        u = omega;
      }
    }
    upd[j] = u;
  }
  if (__syncthreads_or(found) && threadIdx.x == 0) st->found = 1;
}

// cuda_compute_scores_smp (GAGA/gaga/expander/kernels.cu:79-104): u_j = median of the
// residual over column j's d rows (d <= 32)
__global__ void k_smp_scores(const GbState *st, const float *__restrict__ res, const int *__restrict__ rows, int n,
                             int d, float *__restrict__ u) {
  if (!st->active) return;
  for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
    float b[32];
    for (int i = 0; i < d; ++i) b[i] = res[rows[(size_t)j * d + i]];
    for (int i = 0; i < d; ++i)
      for (int q = 0; q < d - 1; ++q)
        if (b[q] > b[q + 1]) {
          const float t = b[q + 1];
          b[q + 1] = b[q];
          b[q] = t;
        }
    u[j] = (d % 2) == 0 ? (b[d / 2 - 1] + b[d / 2]) / 2 : b[(d - 1) / 2];
  }
}

// ------------------------------------------------------------------ sequential decoders
// Node scores of ssmp and er (GAGA/gaga/expander/kernels.cu:115-145, 195-245): the d residual
// entries of node j, bubble-sorted as the reference does; ssmp: the median and its
// magnitude; er: the mode (the value before the first longest run of entries within 1e-7 of
// their neighbour) and its run length as the score (0 when |mode| <= 1e-7).
__device__ __forceinline__ void seq_score(int er, const float *__restrict__ res, const int *__restrict__ rows_j,
                                          int d, float *upd, float *score) {
  float b[32];
  for (int i = 0; i < d; ++i) b[i] = res[rows_j[i]];
  for (int i = 0; i < d; ++i)
    for (int q = 0; q < d - 1; ++q)
      if (b[q] > b[q + 1]) {
        const float t = b[q + 1];
        b[q + 1] = b[q];
        b[q] = t;
      }
  if (!er) {
    const float z = (d % 2) == 0 ? (b[d / 2 - 1] + b[d / 2]) / 2 : b[(d - 1) / 2];
    *upd = z;
    *score = fabsf(z);
  } else {
    const float eps = 0.0000001f;
    float mode = b[0], count = 1.0f, count_mode = 1.0f;
    for (int i = 1; i < d; ++i) {
      if (fabsf(__fsub_rn(b[i], b[i - 1])) <= eps) {
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

// every node's score (cuda_compute_scores_ssmp / _er)
__global__ void k_seq_scores(const GbState *st, int er, const float *__restrict__ res, const int *__restrict__ rows,
                             int n, int d, float *__restrict__ upd, float *__restrict__ score) {
  if (!st->active) return;
  for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x)
    seq_score(er, res, rows + (size_t)j * d, d, &upd[j], &score[j]);
}

// the scores of the nodes that share a row with the node just updated (cuda_update_scores_ssmp
// / _er, kernels.cu:147-193, 247-305): block b walks row rows[h d + b] of the row-major copy.
// A node on several of those rows is scored by several blocks, with the same result.
__global__ void k_seq_rescore(const GbState *st, int er, const float *__restrict__ res, const int *__restrict__ rows,
                              const int *__restrict__ ptr, const int *__restrict__ col, int d,
                              float *__restrict__ upd, float *__restrict__ score) {
  if (!st->active) return;
  const int h = st->h_node;
  const int r = rows[(size_t)h * d + blockIdx.x];
  for (int e = ptr[r] + threadIdx.x; e < ptr[r + 1]; e += blockDim.x) {
    const int j = col[e];
    seq_score(er, res, rows + (size_t)j * d, d, &upd[j], &score[j]);
  }
}

// cublasIsamax over the scores: the first index of the largest |score|, as a grid reduction in
// a fixed order (each block its best (value, index), the last block to arrive picks among them)
__device__ __forceinline__ void better(float &v, int &i, float v2, int i2) {
  if (v2 > v || (v2 == v && i2 < i)) {
    v = v2;
    i = i2;
  }
}
__global__ void __launch_bounds__(256) k_seq_argmax(GbState *st, const float *__restrict__ score, int n,
                                                    float *parts, unsigned int *tickets) {
  if (!st->active) return;
  float bv = -1.0f;
  int bi = 0x7fffffff;
  for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
    const float v = fabsf(score[j]);
    if (v > bv) {
      bv = v;
      bi = j;
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) better(bv, bi, __shfl_xor_sync(0xffffffffu, bv, o), __shfl_xor_sync(0xffffffffu, bi, o));
  __shared__ float sv[32];
  __shared__ int si[32];
  __shared__ int last;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  if (lane == 0) {
    sv[wid] = bv;
    si[wid] = bi;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int q = 1; q < nw; ++q) better(bv, bi, sv[q], si[q]);
    parts[R_SEQ_VAL * GB_MAXRB + blockIdx.x] = bv;
    parts[R_SEQ_IDX * GB_MAXRB + blockIdx.x] = __int_as_float(bi);
    __threadfence();
    const unsigned int t = atomicAdd(&tickets[R_SEQ_VAL], 1u);
    last = (t == gridDim.x - 1);
  }
  __syncthreads();
  if (last && threadIdx.x == 0) {
    __threadfence();
    float v = -1.0f;
    int i = 0x7fffffff;
    for (int q = 0; q < (int)gridDim.x; ++q)
      better(v, i, __ldcg(&parts[R_SEQ_VAL * GB_MAXRB + q]), __float_as_int(__ldcg(&parts[R_SEQ_IDX * GB_MAXRB + q])));
    st->h_node = (i >= 0 && i < n) ? i : 0;
    tickets[R_SEQ_VAL] = 0u;
  }
}

// cudaUpdateSignal + cudaUpdateResidual (GAGA/gaga/expander/kernels.cu:1014-1032) for node h:
// x_h += update_h and, unless ssmp takes its periodic H_k step this iteration (iter % k == 0,
// iter > 0, ssmp.cu:102-117), res -= update_h * A_h (one lane per row of the column)
__global__ void k_seq_node(GbState *st, float *__restrict__ x, float *__restrict__ res, const int *__restrict__ rows,
                           const float *__restrict__ vals, const float *__restrict__ upd, int d,
                           cudaGraphConditionalHandle h_if) {
  if (!st->active) {
    if (threadIdx.x == 0) set_cond(h_if, 0u);
    return;
  }
  const int h = st->h_node;
  const bool ssmp = st->alg == GB_ALG_SSMP || st->alg == GB_ALG_SSMP_NAIVE;
  const bool periodic = ssmp && st->k > 0 && (st->iter % st->k == 0) && (st->iter > 0);
  const float u = upd[h];
  if (!periodic && (int)threadIdx.x < d) {
    const size_t e = (size_t)h * d + threadIdx.x;
    const int r = rows[e];
    res[r] = fmaf(-u, vals[e], res[r]);
  }
  if (threadIdx.x == 0) {
    x[h] = x[h] + u;
    st->periodic = periodic ? 1 : 0;
    set_cond(h_if, periodic ? 1u : 0u);
  }
}

// ThresholdK (GAGA/gaga/expander/functions.cu:103-123): after Threshold, per-tile counts of
// the support and of the entries in the k-th bin (second half of tile_cnt)
__global__ void __launch_bounds__(256) k_hk_count(const GbState *st, const float *__restrict__ v,
                                                  const int *__restrict__ bins, int n, int *__restrict__ tile_cnt) {
  if (!st->active) return;
  __shared__ float sm[32];
  const int kb = st->k_bin, base = blockIdx.x * GB_TILE;
  float nz = 0.0f, kc = 0.0f;
  for (int q = threadIdx.x; q < GB_TILE; q += blockDim.x) {
    const int i = base + q;
    if (i < n) {
      nz += v[i] != 0.0f ? 1.0f : 0.0f;
      kc += bins[i] == kb ? 1.0f : 0.0f;
    }
  }
  nz = block_reduce<0>(nz, sm);
  if (threadIdx.x == 0) tile_cnt[blockIdx.x] = (int)nz;
  kc = block_reduce<0>(kc, sm);
  if (threadIdx.x == 0) tile_cnt[gridDim.x + blockIdx.x] = (int)kc;
}

// ... then the first (support - K) entries of the k-th bin, in index order, are zeroed
// (the reference takes them in atomic order)
__global__ void __launch_bounds__(256) k_hk_trim(const GbState *st, float *__restrict__ v, const int *__restrict__ bins,
                                                 int n, const int *__restrict__ tile_cnt, int K) {
  if (!st->active) return;
  __shared__ int s_off, s_before;
  __shared__ int warp_cnt[8];
  if (threadIdx.x == 0) {
    int tot = 0, before = 0;
    for (int t = 0; t < (int)gridDim.x; ++t) {
      tot += tile_cnt[t];
      if (t < (int)blockIdx.x) before += tile_cnt[gridDim.x + t];
    }
    s_off = tot - K;
    s_before = before;
  }
  __syncthreads();
  const int offset = s_off;
  if (offset <= 0 || s_before >= offset) return;  // uniform over the block
  const int kb = st->k_bin, base = blockIdx.x * GB_TILE;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  int running = s_before;
  for (int q0 = 0; q0 < GB_TILE; q0 += blockDim.x) {
    const int i = base + q0 + threadIdx.x;
    const bool in = i < n && bins[i] == kb;
    const unsigned bal = __ballot_sync(0xffffffffu, in);
    if (lane == 0) warp_cnt[wid] = __popc(bal);
    __syncthreads();
    int wb = 0, tot = 0;
    for (int w2 = 0; w2 < 8; ++w2) {
      if (w2 < wid) wb += warp_cnt[w2];
      tot += warp_cnt[w2];
    }
    if (in && running + wb + __popc(bal & ((1u << lane) - 1u)) < offset) v[i] = 0.0f;
    running += tot;
    __syncthreads();
  }
}

// cuda_update_residual (GAGA/gaga/expander/kernels.cu:3-14) as a row gather over the CSR
// copy: each row applies its accepted updates in ascending column order; ||res||^2
__global__ void k_l0_update(GbState *st, float *__restrict__ res, const int *__restrict__ ptr,
                            const int *__restrict__ col, const float *__restrict__ upd, int m, float *rp,
                            unsigned int *tk) {
  if (!st->active) return;
  float s2 = 0.0f;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < m; i += gridDim.x * blockDim.x) {
    float r = res[i];
    const int e1 = ptr[i + 1];
    for (int e = ptr[i]; e < e1; ++e) {
      const float u = upd[col[e]];
      if (fabsf(u) > 0.0f) r = __fadd_rn(r, -u);
    }
    res[i] = r;
    s2 = fmaf(r, r, s2);
  }
  grid_reduce_publish<0>(s2, R_RES, st, rp, tk);
}

// ------------------------------------------------------------------ state init
__global__ void k_init_state(GbState *st, GbState init) {
  if (threadIdx.x == 0 && blockIdx.x == 0) *st = init;
}

// ------------------------------------------------------------------ graph helpers
namespace {

// A conditional handle is created on the graph being captured on `parent`; the kernel
// that sets its first value is captured next, then the WHILE node itself.
gb_status make_handle(cudaStream_t parent, cudaGraphConditionalHandle *h) {
  cudaStreamCaptureStatus cs;
  cudaGraph_t g;
  GB_CUDA_TRY(cudaStreamGetCaptureInfo(parent, &cs, nullptr, &g, nullptr, nullptr, nullptr));
  GB_CUDA_TRY(cudaGraphConditionalHandleCreate(h, g, 0, 0));
  return GB_OK;
}

gb_status open_cond(cudaStream_t parent, cudaStream_t body, cudaGraphConditionalHandle h, cudaGraphConditionalNodeType type) {
  cudaStreamCaptureStatus cs;
  cudaGraph_t g;
  const cudaGraphNode_t *deps = nullptr;
  size_t nd = 0;
  GB_CUDA_TRY(cudaStreamGetCaptureInfo(parent, &cs, nullptr, &g, &deps, nullptr, &nd));
  cudaGraphNodeParams p = {};
  p.type = cudaGraphNodeTypeConditional;
  p.conditional.handle = h;
  p.conditional.type = type;
  p.conditional.size = 1;
  cudaGraphNode_t node;
  GB_CUDA_TRY(cudaGraphAddNode(&node, g, deps, nullptr, nd, &p));
  GB_CUDA_TRY(cudaStreamUpdateCaptureDependencies(parent, &node, nullptr, 1, cudaStreamSetCaptureDependencies));
  GB_CUDA_TRY(cudaStreamBeginCaptureToGraph(body, p.conditional.phGraph_out[0], nullptr, nullptr, 0,
                                            cudaStreamCaptureModeRelaxed));
  return GB_OK;
}

gb_status open_while(cudaStream_t parent, cudaStream_t body, cudaGraphConditionalHandle h) {
  return open_cond(parent, body, h, cudaGraphCondTypeWhile);
}

gb_status close_while(cudaStream_t body) {
  cudaGraph_t g;
  GB_CUDA_TRY(cudaStreamEndCapture(body, &g));
  return GB_OK;
}

}  // namespace

static void enq_mask(GbWork &w, cudaStream_t s, int pf, const float *src, float *dst, int slot_sq, int slot_max) {
  k_mask<<<w.red_blocks, 256, 0, s>>>(w.st, pf, src, dst, w.bins, argN(w), slot_sq, slot_max, w.red_part, w.tickets);
}
static void enq_axpy(GbWork &w, cudaStream_t s, int pf, int which, const float *x, float *y, int n, int slot_max,
                     bool clear_counters, int num_bins) {
  k_axpy<<<w.red_blocks, 256, 0, s>>>(w.st, pf, which, x, y, n, slot_max, -1, clear_counters ? w.counters : nullptr,
                                      num_bins, w.red_part, w.tickets);
}
static void enq_ctrl(GbWork &w, cudaStream_t s, int phase, cudaGraphConditionalHandle h = 0) {
  k_ctrl<<<1, 32, 0, s>>>(w.st, phase, h);
}

// FindSupportSet + Threshold: binning, k-th bin and ordered compaction predicated on
// F_DOBIN; the threshold of x always runs
static void enq_support(GbWork &w, cudaStream_t s, int k, bool save_prev) {
  const int n = argN(w);
  k_hist<<<w.red_blocks, 256, 0, s>>>(w.st, F_DOBIN, w.x, w.bins, save_prev ? w.bins_prev : nullptr, w.counters, n);
  k_kbin<<<1, 1024, 0, s>>>(w.st, F_DOBIN, w.counters, w.dyn ? D_K : k);
  const int tiles = (w.op.n + GB_TILE - 1) / GB_TILE;  // capacity; tiles past n count 0
  k_thresh_count<<<tiles, 256, 0, s>>>(w.st, F_ALWAYS, w.x, w.bins, save_prev ? w.bins_prev : nullptr, n, w.tile_cnt);
  k_compact<<<tiles, 256, 0, s>>>(w.st, F_DOBIN, w.bins, n, w.tile_cnt, w.S, w.smv_bm);
}

// supportFlag 2/3: a new T when F_SORT (radix select), the threshold, and for the dense
// operator the support list of the thresholded x
static void enq_sort_support(GbWork &w, cudaStream_t s) {
  const int n = argN(w);
  for (int pass = 0; pass < 3; ++pass) {
    k_sel_hist<<<w.red_blocks, 256, 0, s>>>(w.st, w.x, n, w.sel_hist + pass * GB_SEL_BINS, pass);
    k_sel_scan<<<1, 1024, 0, s>>>(w.st, w.sel_hist + pass * GB_SEL_BINS, pass);
  }
  const int tiles = (n + GB_TILE - 1) / GB_TILE;
  k_sort_thresh<<<tiles, 256, 0, s>>>(w.st, w.x, w.bins, n, w.tile_cnt);
  if (w.op.kind == GB_OP_DENSE) k_sort_compact<<<tiles, 256, 0, s>>>(w.st, w.x, n, w.tile_cnt, w.S);
}

void enq_stamp(GbWork &w, cudaStream_t s, int which, int which2) {
  if (w.tstamp) k_stamp<<<1, 1, 0, s>>>(w.st, w.tstamp, w.tcg, which, which2);
}

// CG start on the current support (HTP's projection, ThresholdCG, CSMPSP): r = y - A x,
// grad = grad_previous = (A^T r) restricted to the support; ||r||^2 and ||grad||^2
static void enq_cg_start(GbWork &w, cudaStream_t s) {
  const int n = argN(w);
  enq_A(w, s, w.x, w.resid, w.y, R_RES, F_ALWAYS);
  enq_AT(w, s, w.resid, w.grad, F_ALWAYS);
  k_threshold<<<w.red_blocks, 256, 0, s>>>(w.st, F_ALWAYS, w.grad, w.bins, n);
  k_copy_norm<<<w.red_blocks, 256, 0, s>>>(w.st, F_ALWAYS, w.grad, w.gp, n, R_DOT1, -1, w.red_part, w.tickets);
}

// CSMPSP loop, first part (GAGA/gaga/algorithms.cu:3513-3541): top-k of the gradient joins
// the support of x; then the CG start on the joined support
static void enq_csmpsp_join(SolvePlan &P, cudaStream_t s) {
  GbWork &w = *P.w;
  const int n = argN(w);
  enq_AT(w, s, w.resid, w.grad, F_ALWAYS);
  k_copy_norm<<<w.red_blocks, 256, 0, s>>>(w.st, F_ALWAYS, w.grad, nullptr, n, -1, R_XMAX, w.red_part, w.tickets);
  enq_ctrl(w, s, C_CSMPSP_GBIN);
  cudaMemsetAsync(w.counters, 0, sizeof(int) * P.num_bins, s);
  k_hist<<<w.red_blocks, 256, 0, s>>>(w.st, F_DOBIN, w.grad, w.bins_prev, nullptr, w.counters, n);
  k_kbin<<<1, 1024, 0, s>>>(w.st, F_DOBIN, w.counters, P.k);
  enq_ctrl(w, s, C_CSMPSP_JOIN);
  k_join<<<w.red_blocks, 256, 0, s>>>(w.st, w.bins, w.bins_prev, n);
  const int tiles = (w.op.n + GB_TILE - 1) / GB_TILE;
  k_thresh_count<<<tiles, 256, 0, s>>>(w.st, F_ALWAYS, w.x, w.bins, nullptr, n, w.tile_cnt);
  // the join changes the bins even when the gradient's binning was skipped
  k_compact<<<tiles, 256, 0, s>>>(w.st, F_ALWAYS, w.bins, n, w.tile_cnt, w.S, w.smv_bm);
  enq_cg_start(w, s);
}

// CSMPSP loop, last part (algorithms.cu:3580-3620): forced binning of x to its k largest,
// the residual and the stopping rules
static void enq_csmpsp_rebin(SolvePlan &P, cudaStream_t s, cudaGraphConditionalHandle h_outer) {
  GbWork &w = *P.w;
  const int n = argN(w);
  k_copy_norm<<<w.red_blocks, 256, 0, s>>>(w.st, F_ALWAYS, w.x, nullptr, n, -1, R_XMAX, w.red_part, w.tickets);
  enq_ctrl(w, s, C_CSMPSP_XBIN);
  cudaMemsetAsync(w.counters, 0, sizeof(int) * P.num_bins, s);
  enq_support(w, s, P.k, false);
  enq_A(w, s, w.x, w.resid, w.y, R_RES, F_ALWAYS);
  enq_ctrl(w, s, C_CSMPSP_STOP, h_outer);
}

static void lin(GbWork &w, cudaStream_t s, int pf, float *out, const float *a, int which, const float *b, int n,
                const float *dv = nullptr, int slot_dot = -1, int slot_sq = -1) {
  k_lin<<<w.red_blocks, 256, 0, s>>>(w.st, pf, out, a, which, b, n, dv, slot_dot, slot_sq, w.red_part, w.tickets);
}

// forced binning of x (minVal = 0, maxChange = 1) and Threshold, as FIHT / ALPS do after
// every change of x (GAGA/gaga/algorithms.cu:5475-5481)
static void enq_fh_bin(SolvePlan &P, cudaStream_t s) {
  GbWork &w = *P.w;
  const int n = argN(w);
  k_copy_norm<<<w.red_blocks, 256, 0, s>>>(w.st, F_ALWAYS, w.x, nullptr, n, -1, R_XMAX, w.red_part, w.tickets);
  enq_ctrl(w, s, C_FH_BIN);
  cudaMemsetAsync(w.counters, 0, sizeof(int) * P.num_bins, s);
  enq_support(w, s, P.k, false);
}

// grad = A^T r and v = grad on the support with ||v||^2 in red[slot]
static void enq_grad_masked(GbWork &w, cudaStream_t s, int pf, const float *r, float *v, int slot) {
  if (w.op.kind == GB_OP_DENSE) {
    enq_AT_mask(w, s, r, w.grad, v, slot, -1, pf);
  } else {
    enq_AT(w, s, r, w.grad, pf);
    enq_mask(w, s, pf, w.grad, v, slot, -1);
  }
}

// FIHT / ALPS loop (GAGA/gaga/algorithms.cu:5523-5560, 6356-6393; functions.cu:1668-1843)
static void enq_fiht_body(SolvePlan &P, cudaStream_t s, cudaGraphConditionalHandle h_outer) {
  GbWork &w = *P.w;
  const int n = argN(w), m = argM(w);
  float *xp = w.gp, *ex = w.gpt, *vt = w.xt, *Apv = w.am1, *Aex = w.am2;
  // extrapolated point v = x + tau (x_prev - x), A v, the residual at v and the gradient
  lin(w, s, F_ALWAYS, Apv, Apv, SC_NEG_ONE, w.ru, m, w.resid, R_DOT1, R_DOT2);
  enq_ctrl(w, s, C_FH_TAU);
  lin(w, s, F_ALWAYS, xp, xp, SC_NEG_ONE, w.x, n);
  lin(w, s, F_ALWAYS, ex, w.x, SC_CG_BETA, xp, n);
  lin(w, s, F_ALWAYS, Aex, w.ru, SC_CG_BETA, Apv, m);
  lin(w, s, F_ALWAYS, w.resid, w.y, SC_NEG_ONE, Aex, m);
  enq_AT(w, s, w.resid, w.grad, F_ALWAYS);
  lin(w, s, F_ALWAYS, xp, w.x, SC_ONE, nullptr, n);
  lin(w, s, F_ALWAYS, Apv, w.ru, SC_ONE, nullptr, m);
  if (P.alg == GB_ALG_FIHT) {
    k_flagmask<<<w.red_blocks, 256, 0, s>>>(w.st, F_ALWAYS, vt, w.grad, ex, 0, n);
  } else {
    // ALPS: the k largest of the gradient outside supp(v), then the gradient on supp(v)
    k_flagmask<<<w.red_blocks, 256, 0, s>>>(w.st, F_ALWAYS, vt, w.grad, ex, 1, n);
    k_copy_norm<<<w.red_blocks, 256, 0, s>>>(w.st, F_ALWAYS, vt, nullptr, n, -1, R_XMAX, w.red_part, w.tickets);
    enq_ctrl(w, s, C_ALPS_LBIN);
    cudaMemsetAsync(w.counters, 0, sizeof(int) * P.num_bins, s);
    k_hist<<<w.red_blocks, 256, 0, s>>>(w.st, F_DOBIN, vt, w.bins, nullptr, w.counters, n);
    k_kbin<<<1, 1024, 0, s>>>(w.st, F_DOBIN, w.counters, P.k);
    k_threshold<<<w.red_blocks, 256, 0, s>>>(w.st, F_ALWAYS, vt, w.bins, n);
    enq_ctrl(w, s, C_ALPS_LRESTORE);
    k_flagmask<<<w.red_blocks, 256, 0, s>>>(w.st, F_ALWAYS, vt, w.grad, ex, 2, n);
  }
  // vt is not on the compacted support: the support the products read becomes vt's
  if (w.op.kind == GB_OP_DENSE || w.smv_bm_ok) enq_support_of_nonzeros(w, s, vt, n);
  enq_A(w, s, vt, Aex, nullptr, R_AXT, F_ALWAYS);
  k_copy_norm<<<w.red_blocks, 256, 0, s>>>(w.st, F_ALWAYS, vt, nullptr, n, R_XT, -1, w.red_part, w.tickets);
  enq_ctrl(w, s, C_FH_MU);
  lin(w, s, F_ALWAYS, w.x, ex, SC_MU, w.grad, n);
  enq_fh_bin(P, s);
  enq_A(w, s, w.x, w.ru, nullptr, -1, F_ALWAYS);
  lin(w, s, F_ALWAYS, w.resid, w.y, SC_NEG_ONE, w.ru, m);
  // steepest descent restricted to the support
  enq_grad_masked(w, s, F_ALWAYS, w.resid, vt, R_XT);
  enq_A(w, s, vt, Aex, nullptr, R_AXT, F_ALWAYS);
  enq_ctrl(w, s, C_FH_MU);
  lin(w, s, F_ALWAYS, w.x, w.x, SC_MU, vt, n);
  lin(w, s, F_ALWAYS, w.ru, w.ru, SC_MU, Aex, m);
  lin(w, s, F_ALWAYS, w.resid, w.y, SC_NEG_ONE, w.ru, m, nullptr, -1, R_RES);
  enq_ctrl(w, s, C_FH_STOP, h_outer);
}

// CGIHTprojected loop (GAGA/gaga/algorithms.cu:4572-4660): steepest descent with a new
// support (F_UCG) or a CG step on the previous one (F_RCG), chosen by the projection fraction
static void enq_cgproj_body(SolvePlan &P, cudaStream_t s, cudaGraphConditionalHandle h_outer) {
  GbWork &w = *P.w;
  const int n = argN(w), m = argM(w);
  float *vt = w.xt, *p = w.gp, *gpt = w.gpt, *Ap = w.am2, *diff = w.upd;
  k_dot2<<<w.red_blocks, 256, 0, s>>>(w.st, F_UCG, vt, vt, R_DOT1, n, w.ru, w.ru, R_DOT2, m, w.red_part, w.tickets);
  k_dot2<<<w.red_blocks, 256, 0, s>>>(w.st, F_RCG, vt, vt, R_DOT1, n, Ap, Ap, R_DOT2, m, w.red_part, w.tickets);
  enq_ctrl(w, s, C_CP_MU);
  lin(w, s, F_UCG, w.x, w.x, SC_MU, w.grad, n);
  lin(w, s, F_RCG, w.x, w.x, SC_MU, p, n);
  k_copy_norm<<<w.red_blocks, 256, 0, s>>>(w.st, F_UCG, w.x, nullptr, n, -1, R_XMAX, w.red_part, w.tickets);
  enq_ctrl(w, s, C_CP_BIN);
  cudaMemsetAsync(w.counters, 0, sizeof(int) * P.num_bins, s);
  enq_support(w, s, P.k, false);
  enq_A(w, s, w.x, w.ru, nullptr, -1, F_ALWAYS);
  lin(w, s, F_ALWAYS, w.resid, w.y, SC_NEG_ONE, w.ru, m);
  lin(w, s, F_RCG, gpt, vt, SC_ONE, nullptr, n);
  enq_grad_masked(w, s, F_ALWAYS, w.resid, vt, -1);
  enq_A(w, s, vt, w.ru, nullptr, -1, F_ALWAYS);
  lin(w, s, F_UCG, p, vt, SC_ONE, nullptr, n);
  lin(w, s, F_UCG, Ap, w.ru, SC_ONE, nullptr, m);
  k_dot2<<<w.red_blocks, 256, 0, s>>>(w.st, F_RCG, vt, vt, R_DOT3, n, gpt, gpt, R_DOT4, n, w.red_part, w.tickets);
  enq_ctrl(w, s, C_CP_BETA);
  k_scale_add<<<w.red_blocks, 256, 0, s>>>(w.st, F_RCG, SC_CG_BETA, p, vt, n);
  k_scale_add<<<w.red_blocks, 256, 0, s>>>(w.st, F_RCG, SC_CG_BETA, Ap, w.ru, m);
  lin(w, s, F_ALWAYS, diff, w.grad, SC_NEG_ONE, p, n, nullptr, -1, R_DOT1);
  k_copy_norm<<<w.red_blocks, 256, 0, s>>>(w.st, F_ALWAYS, vt, nullptr, n, R_XT, -1, w.red_part, w.tickets);
  k_copy_norm<<<w.red_blocks, 256, 0, s>>>(w.st, F_ALWAYS, w.resid, nullptr, m, R_RES, -1, w.red_part, w.tickets);
  enq_ctrl(w, s, C_CP_PROJ, h_outer);
}

// H_K of the expander decoders on v: a fresh binning, Threshold, ThresholdK
static void enq_expander_hk(SolvePlan &P, cudaStream_t s, float *v, int K) {
  GbWork &w = *P.w;
  const int n = argN(w);
  k_copy_norm<<<w.red_blocks, 256, 0, s>>>(w.st, F_ALWAYS, v, nullptr, n, -1, R_XMAX, w.red_part, w.tickets);
  k_ctrl_l0<<<1, 32, 0, s>>>(w.st, C_SMP_HK, w.rec, 0);
  cudaMemsetAsync(w.counters, 0, sizeof(int) * P.num_bins, s);
  k_hist<<<w.red_blocks, 256, 0, s>>>(w.st, F_DOBIN, v, w.bins, nullptr, w.counters, n);
  k_kbin<<<1, 1024, 0, s>>>(w.st, F_DOBIN, w.counters, K);
  k_threshold<<<w.red_blocks, 256, 0, s>>>(w.st, F_ALWAYS, v, w.bins, n);
  const int tiles = (n + GB_TILE - 1) / GB_TILE;
  k_hk_count<<<tiles, 256, 0, s>>>(w.st, v, w.bins, n, w.tile_cnt);
  k_hk_trim<<<tiles, 256, 0, s>>>(w.st, v, w.bins, n, w.tile_cnt, K);
}

// ssmp / er: every node's score into w.grad (update) and w.xt (score)
static void enq_seq_scores(SolvePlan &P, cudaStream_t s) {
  GbWork &w = *P.w;
  const int n = argN(w);
  int blocks = (n + 255) / 256;
  if (blocks > w.num_sms * 16) blocks = w.num_sms * 16;
  const int er = (P.alg == GB_ALG_ER || P.alg == GB_ALG_ER_NAIVE) ? 1 : 0;
  k_seq_scores<<<blocks, 256, 0, s>>>(w.st, er, w.resid, w.op.smv_rows, n, w.op.d, w.grad, w.xt);
}

static void enq_seq_tail(SolvePlan &P, cudaStream_t s, cudaGraphConditionalHandle h_outer);

// One iteration of ssmp / er (GAGA/gaga/expander/ssmp.cu:82-145, er.cu:69-125; the naive
// forms, ssmp.cu:235-295 and er.cu:186-225, score every node each iteration instead of the
// neighbours of the node updated): the node of the largest score, its update, ssmp's
// periodic H_k with a fresh residual (an IF node, h_if, when s_if is a capture stream), the
// rescoring, ||res||, the stopping rules.  With h_if == 0 (eager), the periodic step is left
// to the caller.
static gb_status enq_seq_body(SolvePlan &P, cudaStream_t s, cudaStream_t s_if, cudaGraphConditionalHandle h_outer,
                              bool graph) {
  GbWork &w = *P.w;
  const int n = argN(w), m = argM(w), d = w.op.d;
  const bool er = P.alg == GB_ALG_ER || P.alg == GB_ALG_ER_NAIVE;
  const bool naive = P.alg == GB_ALG_SSMP_NAIVE || P.alg == GB_ALG_ER_NAIVE;
  const int ier = er ? 1 : 0;
  if (naive) enq_seq_scores(P, s);
  k_seq_argmax<<<w.red_blocks, 256, 0, s>>>(w.st, w.xt, n, w.red_part, w.tickets);
  cudaGraphConditionalHandle h_if = 0;
  if (graph && !er) GB_TRY(make_handle(s, &h_if));
  k_seq_node<<<1, 32, 0, s>>>(w.st, w.x, w.resid, w.op.smv_rows, w.op.smv_vals, w.grad, d, h_if);
  if (graph && !er) {
    // ssmp: every k-th iteration H_k(x) and res = y - A x (ssmp.cu:102-110)
    GB_TRY(open_cond(s, s_if, h_if, cudaGraphCondTypeIf));
    enq_expander_hk(P, s_if, w.x, P.k);
    enq_A(w, s_if, w.x, w.resid, w.y, -1, F_ALWAYS);
    if (!naive) enq_seq_scores(P, s_if);
    GB_TRY(close_while(s_if));
  }
  if (!naive)
    k_seq_rescore<<<d, 128, 0, s>>>(w.st, ier, w.resid, w.op.smv_rows, w.op.csr_ptr, w.op.csr_col, d, w.grad, w.xt);
  if (graph) enq_seq_tail(P, s, h_outer);
  (void)m;
  return GB_OK;
}

// ||res|| and the stopping rules of one ssmp / er iteration
static void enq_seq_tail(SolvePlan &P, cudaStream_t s, cudaGraphConditionalHandle h_outer) {
  GbWork &w = *P.w;
  k_copy_norm<<<w.red_blocks, 256, 0, s>>>(w.st, F_ALWAYS, w.resid, nullptr, argM(w), R_RES, -1, w.red_part,
                                           w.tickets);
  k_ctrl_l0<<<1, 32, 0, s>>>(w.st, C_SEQ_STOP, w.rec, h_outer);
}

// ssmp's final H_k after the loop (ssmp.cu:146-148)
static void enq_seq_final(SolvePlan &P, cudaStream_t s) {
  GbWork &w = *P.w;
  if (P.alg != GB_ALG_SSMP && P.alg != GB_ALG_SSMP_NAIVE) return;
  k_ctrl_l0<<<1, 32, 0, s>>>(w.st, C_SEQ_END1, w.rec, 0);
  enq_expander_hk(P, s, w.x, P.k);
  k_ctrl_l0<<<1, 32, 0, s>>>(w.st, C_SEQ_END2, w.rec, 0);
}

// smp loop (GAGA/gaga/expander/smp.cu:67-131)
static void enq_smp_body(SolvePlan &P, cudaStream_t s, cudaGraphConditionalHandle h_outer) {
  GbWork &w = *P.w;
  const int n = argN(w);
  int blocks = (n + 255) / 256;
  if (blocks > w.num_sms * 16) blocks = w.num_sms * 16;
  k_smp_scores<<<blocks, 256, 0, s>>>(w.st, w.resid, w.op.smv_rows, n, w.op.d, w.grad);
  enq_expander_hk(P, s, w.grad, 2 * P.k);
  lin(w, s, F_ALWAYS, w.x, w.x, SC_ONE, w.grad, n);
  enq_expander_hk(P, s, w.x, P.k);
  enq_A(w, s, w.x, w.resid, w.y, R_RES, F_ALWAYS);
  k_ctrl_l0<<<1, 32, 0, s>>>(w.st, C_SMP_STOP, w.rec, h_outer);
}

// The solve as pieces: prologue, loop body (with the HTP inner CG loop), run either as one
// graph with WHILE nodes or eagerly (GB_CS_EAGER=1: same kernels, host-checked loops;
// used for profiling, since kernels inside conditional graphs cannot be profiled).
void enq_prologue(SolvePlan &P, cudaStream_t s0, cudaGraphConditionalHandle h_outer) {
  GbWork &w = *P.w;
  const int n = argN(w), m = argM(w), k = P.k, num_bins = w.dyn ? D_NBINS : P.num_bins;
  if (P.alg == GB_ALG_SMP) {
    // res = y - A x^0 (smp.cu:45-48)
    enq_A(w, s0, w.x, w.resid, w.y, R_RES, F_ALWAYS);
    k_ctrl_l0<<<1, 32, 0, s0>>>(w.st, C_SMP_INIT, w.rec, h_outer);
    return;
  }
  if (gb_is_seq(P.alg)) {
    // res = y - A x^0, err, the first scores (ssmp.cu:56-75, er.cu:43-61)
    enq_A(w, s0, w.x, w.resid, w.y, R_RES, F_ALWAYS);
    k_ctrl_l0<<<1, 32, 0, s0>>>(w.st, C_SEQ_INIT, w.rec, h_outer);
    enq_seq_scores(P, s0);
    return;
  }
  if (gb_is_l0(P.alg)) {
    // res = y - A x with x = 0 (computeResidual, GAGA/gaga/expander/functions.cu:73-79)
    enq_A(w, s0, w.x, w.resid, w.y, R_RES, F_ALWAYS);
    k_ctrl_l0<<<1, 32, 0, s0>>>(w.st, C_L0_INIT, w.rec, h_outer);
    return;
  }
  // resid = y; err = ||y||  (algorithms.cu:1296-1300)
  k_copy_norm<<<w.red_blocks, 256, 0, s0>>>(w.st, F_ALWAYS, w.y, w.resid, m, R_RES, -1, w.red_part, w.tickets);
  enq_ctrl(w, s0, C_INIT0);
  if (P.alg == GB_ALG_IHT) {
    // IHT (algorithms.cu:347-405): x = 0; the bins take the scale of A^T y
    cudaMemsetAsync(w.x, 0, sizeof(float) * w.op.n, s0);
    enq_AT(w, s0, w.resid, w.grad, F_ALWAYS);
    k_copy_norm<<<w.red_blocks, 256, 0, s0>>>(w.st, F_ALWAYS, w.grad, nullptr, n, -1, R_XMAX, w.red_part,
                                              w.tickets);
    enq_ctrl(w, s0, C_IHT_INIT, h_outer);
    return;
  }
  // x = A^T y ; max |x| ; FindSupportSet ; Threshold  (algorithms.cu:1335-1354)
  enq_AT(w, s0, w.y, w.x, F_ALWAYS);
  k_copy_norm<<<w.red_blocks, 256, 0, s0>>>(w.st, F_ALWAYS, w.x, nullptr, n, -1, R_XMAX, w.red_part, w.tickets);
  if (P.alg == GB_ALG_CGIHT && w.ml_params) {
    // learned warm start: x = g . net(features of g); the support selection below keeps
    // the k largest |x| (GAGA/gaga/algorithms.cu:3776 starts from H_k(A^T y) instead)
    enq_learned_warm(w, s0, F_ALWAYS);
    k_copy_norm<<<w.red_blocks, 256, 0, s0>>>(w.st, F_ALWAYS, w.x, nullptr, n, -1, R_XMAX, w.red_part, w.tickets);
  }
  enq_ctrl(w, s0, C_INIT_BINPREP);
  k_axpy<<<w.red_blocks, 256, 0, s0>>>(w.st, F_ALWAYS, SC_ONE, w.x, w.x, 0, -1, -1, w.counters, num_bins,
                                       w.red_part, w.tickets);
  enq_support(w, s0, k, false);
  if (P.alg == GB_ALG_HT_CG) {
    // r = y - A x; grad = grad_previous = (A^T r) on the support (algorithms.cu:1870-1911)
    enq_cg_start(w, s0);
    enq_ctrl(w, s0, C_HTCG_INIT, h_outer);
  } else if (P.alg == GB_ALG_CSMPSP) {
    // the first CG projection on the support of x follows (algorithms.cu:3462-3476)
    enq_cg_start(w, s0);
  } else if (P.alg == GB_ALG_FIHT || P.alg == GB_ALG_ALPS) {
    // one more iteration: x_prev = x, x = H_k(x + A^T (y - A x)) (algorithms.cu:5484-5515)
    enq_A(w, s0, w.x, w.ru, nullptr, -1, F_ALWAYS);
    lin(w, s0, F_ALWAYS, w.resid, w.resid, SC_NEG_ONE, w.ru, m, nullptr, -1, R_RES);
    enq_ctrl(w, s0, C_FH_INIT1);
    enq_AT(w, s0, w.resid, w.grad, F_ALWAYS);
    lin(w, s0, F_ALWAYS, w.gp, w.x, SC_ONE, nullptr, n);
    lin(w, s0, F_ALWAYS, w.am1, w.ru, SC_ONE, nullptr, m);
    lin(w, s0, F_ALWAYS, w.x, w.x, SC_ONE, w.grad, n);
    enq_fh_bin(P, s0);
    enq_A(w, s0, w.x, w.ru, nullptr, -1, F_ALWAYS);
    lin(w, s0, F_ALWAYS, w.resid, w.y, SC_NEG_ONE, w.ru, m, nullptr, -1, R_RES);
    enq_ctrl(w, s0, C_FH_INIT2, h_outer);
  } else if (P.alg == GB_ALG_CGIHT_PROJ) {
    // r = y - A x; v = (A^T r) on the support; A v (algorithms.cu:4532-4556)
    enq_A(w, s0, w.x, w.ru, nullptr, -1, F_ALWAYS);
    lin(w, s0, F_ALWAYS, w.resid, w.resid, SC_NEG_ONE, w.ru, m, nullptr, -1, R_RES);
    enq_ctrl(w, s0, C_FH_INIT1);
    enq_grad_masked(w, s0, F_ALWAYS, w.resid, w.xt, -1);
    enq_A(w, s0, w.xt, w.ru, nullptr, -1, F_ALWAYS);
    enq_ctrl(w, s0, C_CP_INIT2, h_outer);
  } else if (P.alg == GB_ALG_CGIHT) {
    // r0, grad_previous = A^T r0, grad_prev_thres (algorithms.cu:3776-3808)
    enq_A(w, s0, w.x, w.resid, w.y, R_RES, F_ALWAYS);
    enq_AT(w, s0, w.resid, w.gp, F_ALWAYS);
    enq_mask(w, s0, F_ALWAYS, w.gp, w.gpt, -1, -1);
    enq_ctrl(w, s0, C_CGIHT_INIT, h_outer);
  } else {
    enq_ctrl(w, s0, C_INIT_DONE, h_outer);
  }
}

// first part of an outer iteration (everything for NIHT / CGIHT; up to the CG loop for HTP)
void enq_body(SolvePlan &P, cudaStream_t s1, cudaGraphConditionalHandle h_outer) {
  GbWork &w = *P.w;
  const int n = argN(w), m = argM(w), k = P.k, num_bins = w.dyn ? D_NBINS : P.num_bins;
  if (P.alg == GB_ALG_IHT) {
    // IHT_S_gen loop (GAGA/gaga/algorithms.cu:416-466), fixed step mu
    enq_AT(w, s1, w.resid, w.grad, F_ALWAYS);
    k_copy_norm<<<w.red_blocks, 256, 0, s1>>>(w.st, F_ALWAYS, w.grad, nullptr, n, -1, R_GMAX, w.red_part,
                                              w.tickets);
    enq_ctrl(w, s1, C_IHT_PREP);
    enq_axpy(w, s1, F_ALWAYS, SC_MU, w.grad, w.x, n, -1, true, num_bins);
    enq_support(w, s1, k, false);
    enq_A(w, s1, w.x, w.resid, w.y, R_RES, F_ALWAYS);
    enq_ctrl(w, s1, C_IHT_STOP, h_outer);
    return;
  }
  if (P.alg == GB_ALG_HT_SD) {
    // HT_SD_S_gen loop (algorithms.cu:861-890): RestrictedSD on the fixed support
    enq_A(w, s1, w.x, w.resid, w.y, R_RES, F_ALWAYS);
    enq_ctrl(w, s1, C_PUSH_RES);
    if (w.op.kind == GB_OP_DENSE) {
      enq_AT_mask(w, s1, w.resid, w.grad, w.xt, R_XT, R_GMAX, F_ALWAYS);
    } else {
      enq_AT(w, s1, w.resid, w.grad, F_ALWAYS);
      enq_mask(w, s1, F_ALWAYS, w.grad, w.xt, R_XT, R_GMAX);
    }
    enq_A(w, s1, w.xt, w.ru, nullptr, R_AXT, F_ALWAYS);
    enq_ctrl(w, s1, C_HTSD_MU);
    enq_axpy(w, s1, F_ALWAYS, SC_MU, w.grad, w.x, n, -1, false, 0);
    k_threshold<<<w.red_blocks, 256, 0, s1>>>(w.st, F_ALWAYS, w.x, w.bins, n);
    enq_ctrl(w, s1, C_HTSD_STOP, h_outer);
    return;
  }
  if (P.alg == GB_ALG_HT_CG) {
    // HT_CG_S_gen loop (algorithms.cu:1937-1960): RestrictedCG steps on the fixed support
    enq_cg_body(P, s1, h_outer, C_HTCG_STOP);
    return;
  }
  if (P.alg == GB_ALG_FIHT || P.alg == GB_ALG_ALPS) {
    enq_fiht_body(P, s1, h_outer);
    return;
  }
  if (P.alg == GB_ALG_SMP) {
    enq_smp_body(P, s1, h_outer);
    return;
  }
  if (P.alg == GB_ALG_CGIHT_PROJ) {
    enq_cgproj_body(P, s1, h_outer);
    return;
  }
  if (P.alg == GB_ALG_NIHT || P.alg == GB_ALG_HTP) {
    // RestrictedSD (GAGA/gaga/functions.cu:659-745)
    enq_stamp(w, s1, 0);
    enq_A(w, s1, w.x, w.resid, w.y, R_RES, F_ALWAYS);
    enq_ctrl(w, s1, C_PUSH_RES);
    if (w.op.kind == GB_OP_DENSE) {
      enq_AT_mask(w, s1, w.resid, w.grad, w.xt, R_XT, R_GMAX, F_ALWAYS);
    } else {
      enq_AT(w, s1, w.resid, w.grad, F_ALWAYS);
      enq_mask(w, s1, F_ALWAYS, w.grad, w.xt, R_XT, R_GMAX);
    }
    enq_A(w, s1, w.xt, w.ru, nullptr, R_AXT, F_ALWAYS);
    enq_ctrl(w, s1, C_SD_MU);
    enq_axpy(w, s1, F_ALWAYS, SC_MU, w.grad, w.x, n, R_XMAX, true, num_bins);
    enq_stamp(w, s1, 1);
    enq_ctrl(w, s1, C_BINPREP);
    if (P.supp_flag >= 2) enq_sort_support(w, s1);
    else enq_support(w, s1, k, false);
    enq_stamp(w, s1, 2);
    if (P.alg == GB_ALG_NIHT) {
      enq_stamp(w, s1, 5);
      enq_ctrl(w, s1, C_NIHT_STOP, h_outer);
    } else {
      // CG projection on the support (GAGA/gaga/algorithms.cu:2588-2669)
      enq_A(w, s1, w.x, w.resid, w.y, R_RES, F_ALWAYS);
      enq_AT(w, s1, w.resid, w.grad, F_ALWAYS);
      k_threshold<<<w.red_blocks, 256, 0, s1>>>(w.st, F_ALWAYS, w.grad, w.bins, n);
      k_copy_norm<<<w.red_blocks, 256, 0, s1>>>(w.st, F_ALWAYS, w.grad, w.gp, n, R_DOT1, -1, w.red_part, w.tickets);
      enq_stamp(w, s1, 3);
    }
  } else if (P.alg == GB_ALG_CGIHT) {
    // RestrictedCGwithSupportEvolution (functions.cu:1004-1102) under F_RCG;
    // UnrestrictedCG (functions.cu:1107-1220) under F_UCG
    enq_A(w, s1, w.x, w.resid, w.y, R_RES, F_RESX);
    // (batched, rec_every > 0) after a restricted step on an unchanged support: r -= alpha A p
    k_lin<<<w.red_blocks, 256, 0, s1>>>(w.st, F_RESR, w.resid, w.resid, SC_NEG_CG_ALPHA, w.ru, m, nullptr, -1,
                                        R_RES, w.red_part, w.tickets);
    // UCG: r = y - A x and A grad_prev_thres share one pass over the support columns
    const bool two = w.op.kind == GB_OP_DENSE && w.part_two;
    if (two) enq_A2(w, s1, w.x, w.ru, w.y, R_RES, w.gpt, w.resid, F_UCG);
    else enq_A(w, s1, w.x, w.ru, w.y, R_RES, F_UCG);
    enq_ctrl(w, s1, C_PUSH_RES);
    // RCG branch
    if (w.op.kind == GB_OP_DENSE) {
      enq_AT_mask(w, s1, w.resid, w.grad, w.xt, R_XT, -1, F_RCG);
    } else {
      enq_AT(w, s1, w.resid, w.grad, F_RCG);
      enq_mask(w, s1, F_RCG, w.grad, w.xt, R_XT, -1);
    }
    enq_ctrl(w, s1, C_RCG_BETA);
    k_scale_add<<<w.red_blocks, 256, 0, s1>>>(w.st, F_RCG, SC_CG_BETA, w.gp, w.grad, n);
    enq_mask(w, s1, F_RCG, w.gp, w.gpt, -1, R_GMAX);
    enq_A(w, s1, w.gpt, w.ru, nullptr, R_AXT, F_RCG);
    enq_ctrl(w, s1, C_RCG_ALPHA);
    // UCG branch
    if (w.op.kind == GB_OP_DENSE) {
      enq_AT_mask(w, s1, w.ru, w.grad, w.xt, R_XT, -1, F_UCG);
    } else {
      enq_AT(w, s1, w.ru, w.grad, F_UCG);
      enq_mask(w, s1, F_UCG, w.grad, w.xt, R_XT, -1);
    }
    if (!two) enq_A(w, s1, w.gpt, w.resid, nullptr, -1, F_UCG);
    enq_A(w, s1, w.xt, w.ru, nullptr, -1, F_UCG);
    k_dot2<<<w.red_blocks, 256, 0, s1>>>(w.st, F_UCG, w.resid, w.ru, R_DOT1, m, w.resid, w.resid, R_DOT2, m,
                                         w.red_part, w.tickets);
    enq_ctrl(w, s1, C_UCG_BETA);
    k_scale_add<<<w.red_blocks, 256, 0, s1>>>(w.st, F_UCG, SC_CG_BETA, w.gp, w.grad, n);
    enq_mask(w, s1, F_UCG, w.gp, w.gpt, -1, R_GMAX);
    k_scale_add<<<w.red_blocks, 256, 0, s1>>>(w.st, F_UCG, SC_CG_BETA, w.resid, w.ru, m);
    k_dot2<<<w.red_blocks, 256, 0, s1>>>(w.st, F_UCG, w.gpt, w.xt, R_DOT3, n, w.resid, w.resid, R_DOT4, m,
                                         w.red_part, w.tickets);
    enq_ctrl(w, s1, C_UCG_ALPHA);
    // x += alpha * grad_previous; bins; support change (algorithms.cu:3849-3899)
    enq_axpy(w, s1, F_ALWAYS, SC_CG_ALPHA, w.gp, w.x, n, R_XMAX, true, num_bins);
    enq_ctrl(w, s1, C_CGIHT_BINDEC);
    enq_ctrl(w, s1, C_BINPREP);
    enq_support(w, s1, k, true);
    enq_ctrl(w, s1, C_CGIHT_POST);
    enq_mask(w, s1, F_REMASK, w.gp, w.gpt, -1, -1);
    enq_ctrl(w, s1, C_CGIHT_STOP, h_outer);
  } else {
    // parallel_l0 loop (GAGA/gaga/expander/parallel_l0.cu:56-137)
    k_ctrl_l0<<<1, 32, 0, s1>>>(w.st, C_L0_PRE, w.rec, 0);
    int blocks = (w.op.n + 255) / 256;
    if (blocks > w.num_sms * 16) blocks = w.num_sms * 16;
    k_l0_scores<<<blocks, 256, 0, s1>>>(w.st, w.resid, w.x, w.upd, w.op.smv_rows, n, w.op.d);
    k_l0_update<<<w.red_blocks, 256, 0, s1>>>(w.st, w.resid, w.op.csr_ptr, w.op.csr_col, w.upd, m, w.red_part,
                                               w.tickets);
    k_ctrl_l0<<<1, 32, 0, s1>>>(w.st, C_L0_STOP, w.rec, h_outer);
  }
}

// HTP inner CG step (RestrictedCG_S_gen, GAGA/gaga/functions.cu:922-1000)
void enq_cg_body(SolvePlan &P, cudaStream_t s2, cudaGraphConditionalHandle h_inner, int stop_phase) {
  GbWork &w = *P.w;
  const int n = argN(w);
  enq_A(w, s2, w.grad, w.resid, nullptr, R_CG, F_CG);
  enq_ctrl(w, s2, C_HTP_CG1);
  enq_axpy(w, s2, F_CG, SC_CG_ALPHA, w.grad, w.x, n, -1, false, 0);
  enq_AT(w, s2, w.resid, w.xt, F_CG);
  k_threshold<<<w.red_blocks, 256, 0, s2>>>(w.st, F_CG, w.xt, w.bins, n);
  k_axpy<<<w.red_blocks, 256, 0, s2>>>(w.st, F_CG, SC_NEG_CG_ALPHA, w.xt, w.gp, n, -1, R_DOT3, nullptr, 0, w.red_part,
                                       w.tickets);
  enq_ctrl(w, s2, C_HTP_CG2);
  k_scale_add<<<w.red_blocks, 256, 0, s2>>>(w.st, F_CG, SC_CG_BETA, w.grad, w.gp, n);
  enq_A(w, s2, w.x, w.resid, w.y, R_RES, F_CG);
  enq_ctrl(w, s2, stop_phase < 0 ? C_HTP_CG3 : stop_phase, h_inner);
}

void enq_ctrl_phase(GbWork &w, cudaStream_t s, int phase, cudaGraphConditionalHandle h) {
  enq_ctrl(w, s, phase == GB_PHASE_HTP_CGINIT ? C_HTP_CGINIT : phase == GB_PHASE_HTP_STOP ? C_HTP_STOP : phase, h);
}
gb_status gb_make_handle(cudaStream_t parent, cudaGraphConditionalHandle *h) { return make_handle(parent, h); }
gb_status gb_open_while(cudaStream_t parent, cudaStream_t body, cudaGraphConditionalHandle h) {
  return open_while(parent, body, h);
}
gb_status gb_close_while(cudaStream_t body) { return close_while(body); }

static gb_status build_graph(SolvePlan &P, cudaStream_t s0, cudaStream_t s1, cudaStream_t s2, cudaGraph_t *graph) {
  GbWork &w = *P.w;
  GB_CUDA_TRY(cudaStreamBeginCapture(s0, cudaStreamCaptureModeThreadLocal));
  cudaGraphConditionalHandle h_outer = 0, h_inner = 0;
  GB_TRY(make_handle(s0, &h_outer));
  enq_prologue(P, s0, h_outer);
  if (gb_is_seq(P.alg)) {
    // WHILE(outer) { argmax; node update; IF(periodic) { H_k; res }; rescore; stop }; final H_k
    GB_TRY(open_while(s0, s1, h_outer));
    GB_TRY(enq_seq_body(P, s1, s2, h_outer, true));
    GB_TRY(close_while(s1));
    enq_seq_final(P, s0);
    GB_CUDA_TRY(cudaStreamEndCapture(s0, graph));
    return GB_OK;
  }
  if (P.alg == GB_ALG_CSMPSP) {
    // first projection, then WHILE(outer) { join; WHILE(CG) { step }; rebin; stop }
    cudaGraphConditionalHandle h_first = 0;
    GB_TRY(make_handle(s0, &h_first));
    enq_ctrl(w, s0, C_HTP_CGINIT, h_first);
    GB_TRY(open_while(s0, s2, h_first));
    enq_cg_body(P, s2, h_first, C_HTP_CG3);
    GB_TRY(close_while(s2));
    enq_ctrl(w, s0, C_CSMPSP_INIT_DONE, h_outer);
    GB_TRY(open_while(s0, s1, h_outer));
    enq_csmpsp_join(P, s1);
    GB_TRY(make_handle(s1, &h_inner));
    enq_ctrl(w, s1, C_HTP_CGINIT, h_inner);
    GB_TRY(open_while(s1, s2, h_inner));
    enq_cg_body(P, s2, h_inner, C_CSMPSP_CG3);
    GB_TRY(close_while(s2));
    enq_csmpsp_rebin(P, s1, h_outer);
    GB_TRY(close_while(s1));
    GB_CUDA_TRY(cudaStreamEndCapture(s0, graph));
    return GB_OK;
  }
  GB_TRY(open_while(s0, s1, h_outer));
  enq_body(P, s1, h_outer);
  if (P.alg == GB_ALG_HTP) {
    GB_TRY(make_handle(s1, &h_inner));
    enq_ctrl(w, s1, C_HTP_CGINIT, h_inner);
    GB_TRY(open_while(s1, s2, h_inner));
    enq_cg_body(P, s2, h_inner);
    GB_TRY(close_while(s2));
    enq_stamp(w, s1, 4, 5);
    enq_ctrl(w, s1, C_HTP_STOP, h_outer);
  }
  GB_TRY(close_while(s1));
  GB_CUDA_TRY(cudaStreamEndCapture(s0, graph));
  return GB_OK;
}

static gb_status read_int(const int *d, int *h, cudaStream_t s) {
  GB_CUDA_TRY(cudaMemcpyAsync(h, d, sizeof(int), cudaMemcpyDeviceToHost, s));
  GB_CUDA_TRY(cudaStreamSynchronize(s));
  return GB_OK;
}

// Eager execution: the same kernels, the loop conditions read back by the host.
static gb_status run_cg_eager(SolvePlan &P, cudaStream_t s, int stop_phase) {
  GbWork &w = *P.w;
  enq_ctrl(w, s, C_HTP_CGINIT, 0);
  int cg = 0, g2 = 0;
  GB_TRY(read_int(&w.st->flags[F_CG], &cg, s));
  while (cg && g2++ < 16) {
    enq_cg_body(P, s, 0, stop_phase);
    GB_TRY(read_int(&w.st->flags[F_CG], &cg, s));
  }
  return GB_OK;
}

static gb_status run_eager(SolvePlan &P, cudaStream_t s) {
  GbWork &w = *P.w;
  enq_prologue(P, s, 0);
  if (gb_is_seq(P.alg)) {
    const bool naive = P.alg == GB_ALG_SSMP_NAIVE || P.alg == GB_ALG_ER_NAIVE;
    int active = 0, guard = 0, periodic = 0;
    GB_TRY(read_int(&w.st->active, &active, s));
    while (active && guard++ <= w.op.n + 4 + 100000) {
      GB_TRY(enq_seq_body(P, s, s, 0, false));
      GB_TRY(read_int(&w.st->periodic, &periodic, s));
      if (periodic) {
        enq_expander_hk(P, s, w.x, P.k);
        enq_A(w, s, w.x, w.resid, w.y, -1, F_ALWAYS);
        if (!naive) enq_seq_scores(P, s);
      }
      enq_seq_tail(P, s, 0);
      GB_TRY(read_int(&w.st->active, &active, s));
    }
    enq_seq_final(P, s);
    GB_CUDA_TRY(cudaGetLastError());
    return GB_OK;
  }
  if (P.alg == GB_ALG_CSMPSP) {
    GB_TRY(run_cg_eager(P, s, C_HTP_CG3));
    enq_ctrl(w, s, C_CSMPSP_INIT_DONE, 0);
    GbState probe;
    GB_CUDA_TRY(cudaMemcpy(&probe, w.st, sizeof(probe), cudaMemcpyDeviceToHost));
    int active = probe.active, guard = 0;
    while (active && guard++ <= probe.pass_limit) {
      enq_csmpsp_join(P, s);
      GB_TRY(run_cg_eager(P, s, C_CSMPSP_CG3));
      enq_csmpsp_rebin(P, s, 0);
      GB_TRY(read_int(&w.st->active, &active, s));
    }
    GB_CUDA_TRY(cudaGetLastError());
    return GB_OK;
  }
  int active = 0, guard = 0;
  GB_TRY(read_int(&w.st->active, &active, s));
  const int limit = P.w->op.n + 1;  // replaced below by the state's pass limit
  (void)limit;
  GbState probe;
  GB_CUDA_TRY(cudaMemcpy(&probe, w.st, sizeof(probe), cudaMemcpyDeviceToHost));
  while (active && guard++ <= probe.pass_limit) {
    enq_body(P, s, 0);
    if (P.alg == GB_ALG_HTP) {
      enq_ctrl(w, s, C_HTP_CGINIT, 0);
      int cg = 0, g2 = 0;
      GB_TRY(read_int(&w.st->flags[F_CG], &cg, s));
      while (cg && g2++ < 16) {
        enq_cg_body(P, s, 0);
        GB_TRY(read_int(&w.st->flags[F_CG], &cg, s));
      }
      enq_stamp(w, s, 4, 5);
      enq_ctrl(w, s, C_HTP_STOP, 0);
    }
    GB_TRY(read_int(&w.st->active, &active, s));
  }
  GB_CUDA_TRY(cudaGetLastError());
  return GB_OK;
}

// Initial device state for a solve.
static GbState initial_state(const GbWork &w, int alg, const gb_options &o, int k, float tol_abs) {
  GbState st;
  memset(&st, 0, sizeof(st));
  st.m = w.op.m;
  st.n = w.op.n;
  st.k = k;
  st.lda = w.op.lda;
  st.num_bins = o.num_bins;
  st.maxiter = o.maxiter;
  st.alg = alg;
  st.restart = o.restart_flag;
  st.l0_thresh = o.l0_thresh;
  st.d = w.op.d;
  st.tol = tol_abs;
  st.active = 1;
  st.cycle = 1;
  st.pass_limit = o.watchdog_passes > 0 ? o.watchdog_passes : o.maxiter + 4;
  st.resid_diff = 1.0f;
  for (int j = 0; j < 16; ++j) { st.prev[j] = 0.0f; st.evol[j] = 1.0f; }
  // ThresholdSD / ThresholdCG start with alpha = 0 (MaxBin = num_bins, algorithms.cu:800-802)
  st.alpha_bin = (alg == GB_ALG_HT_SD || alg == GB_ALG_HT_CG) ? 0.0f : 0.25f;
  st.max_bin = (int)((float)o.num_bins * (1.0f - st.alpha_bin));
  if (alg == GB_ALG_IHT) st.mu = 0.65f;  // gaga_gen.cu:640 (case 2)
  st.proj_frac_tol = o.proj_frac_tol;
  st.l0_mode = alg == GB_ALG_PARALLEL_LDDSR ? 1 : alg == GB_ALG_PARALLEL_L0_SWIPE ? 2 : 0;
  st.beta_to_zero = 1;
  st.supp_change = 1;
  st.tol_cg = tol_abs * tol_abs;
  st.tol2 = 10.0f * st.tol_cg;
  st.l0_len = 2 * w.op.d;
  st.flags[F_ALWAYS] = 1;
  st.op_kind = w.op.kind;
  st.learned = (w.ml_params && alg == GB_ALG_CGIHT) ? 1 : 0;
  st.tlog = w.tlog;
  // timing variants (NIHT, HTP only; gaga_gen.cu:331-334): alpha from the options
  // (algorithms_timings.cu:477), supportFlag
  if (o.timing && (alg == GB_ALG_NIHT || alg == GB_ALG_HTP)) {
    st.timing = 1;
    st.supp_flag = o.support_flag;
    st.alpha_bin = o.alpha;
    st.max_bin = (int)((float)o.num_bins * (1.0f - st.alpha_bin));
  }
  return st;
}

// Runs one solve on the prepared workspace (x zero, y uploaded); results stay in GbState.
gb_status gb_run_solver(GbWork &w, int alg, const gb_options &o, int k, cudaStream_t s, float tol_abs) {
  if (gb_is_l0(alg) && (w.op.d <= 0 || 2 * w.op.d > 64)) return GB_UNSUPPORTED;
  if ((alg == GB_ALG_SMP || gb_is_seq(alg)) && (w.op.d <= 0 || w.op.d > 32)) return GB_UNSUPPORTED;
  if (gb_is_seq(alg) && k < 1) return GB_BAD_ARG;
  GbState init = initial_state(w, alg, o, k, tol_abs);
  k_init_state<<<1, 1, 0, s>>>(w.st, init);
  GB_CUDA_TRY(cudaGetLastError());
  SolvePlan P{&w, alg, k, o.num_bins};
  if (o.timing && (alg == GB_ALG_NIHT || alg == GB_ALG_HTP)) P.supp_flag = o.support_flag;
  // the expander A v may skip the columns outside the support bitmap: every product of these
  // algorithms is of a vector on the compacted support (as the dense A x_S assumes); the
  // decoders and the sort-based support (which leaves S alone for the expander) do not use it
  w.smv_bm_ok = w.smv_bm && !gb_is_ccs(alg) && P.supp_flag < 2;
  static const bool eager = getenv("GB_CS_EAGER") && atoi(getenv("GB_CS_EAGER")) != 0;
  if (eager) return run_eager(P, s);
  // dense NIHT, HTP or CGIHT (plain or learned start): one thread-block cluster runs the
  // whole solve (gb_resident.cu), without a kernel launch per step
  static const bool no_resident = getenv("GB_CS_SINGLE_RESIDENT") && atoi(getenv("GB_CS_SINGLE_RESIDENT")) == 0;
  // (timing on selects NIHT's and HTP's timing variants; CGIHT ignores it, gaga_gen.cu:331-334)
  if (!no_resident && (alg == GB_ALG_NIHT || alg == GB_ALG_CGIHT || alg == GB_ALG_HTP) &&
      !(o.timing && (alg == GB_ALG_NIHT || alg == GB_ALG_HTP)) && !w.tstamp) {
    int used = 0;
    GB_TRY(gb_resident_solve_single(w, alg, o.num_bins, s, &used));
    if (used) return GB_OK;
  }
  cudaStream_t s0, s1, s2;
  GB_CUDA_TRY(cudaStreamCreateWithFlags(&s0, cudaStreamNonBlocking));
  GB_CUDA_TRY(cudaStreamCreateWithFlags(&s1, cudaStreamNonBlocking));
  GB_CUDA_TRY(cudaStreamCreateWithFlags(&s2, cudaStreamNonBlocking));
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  gb_status rc = build_graph(P, s0, s1, s2, &graph);
  if (rc == GB_OK) {
    cudaError_t e = cudaGraphInstantiate(&exec, graph, 0);
    if (e != cudaSuccess) {
      gb_set_error_message(cudaGetErrorString(e), __FILE__, __LINE__);
      rc = GB_CUDA_ERROR;
    }
  }
  if (rc == GB_OK) {
    cudaError_t e = cudaGraphLaunch(exec, s);
    if (e != cudaSuccess) {
      gb_set_error_message(cudaGetErrorString(e), __FILE__, __LINE__);
      rc = GB_CUDA_ERROR;
    }
  }
  if (exec) cudaGraphExecDestroy(exec);
  if (graph) cudaGraphDestroy(graph);
  cudaStreamDestroy(s0);
  cudaStreamDestroy(s1);
  cudaStreamDestroy(s2);
  return rc;
}

// ------------------------------------------------------------------ FindSupportSet_sort component
// FindSupportSet_sort (GAGA/gaga/functions.cu:446-465) on a device vector: the solver's
// radix select and threshold kernels with a one-off state.  Returns the new T.
extern "C" gb_status gb_cs_find_support_set_sort(float *d_v, int *d_bins, int n, int k, float T, float max_change,
                                                 float *T_out, void *stream) {
  if (!d_v || !d_bins || !T_out || n < 1 || k < 1 || k > n) {
    gb_set_error_message("bad FindSupportSet_sort arguments", __FILE__, __LINE__);
    return GB_BAD_ARG;
  }
  cudaStream_t s = (cudaStream_t)stream;
  GbState h;
  memset(&h, 0, sizeof(h));
  h.active = 1;
  h.n = n;
  h.k = k;
  h.flags[F_ALWAYS] = 1;
  if (T > max_change) {
    h.sort_T = T - max_change;
    h.flags[F_SORT] = 0;
  } else {
    h.flags[F_SORT] = 1;
  }
  const int tiles = (n + GB_TILE - 1) / GB_TILE;
  GbState *st = nullptr;
  unsigned int *hist = nullptr;
  int *tile_cnt = nullptr;
  gb_status rc = GB_OK;
  cudaError_t e = cudaMalloc(&st, sizeof(GbState));
  if (e == cudaSuccess) e = cudaMalloc(&hist, sizeof(unsigned int) * 3 * GB_SEL_BINS);
  if (e == cudaSuccess) e = cudaMalloc(&tile_cnt, sizeof(int) * tiles);
  if (e == cudaSuccess) e = cudaMemsetAsync(hist, 0, sizeof(unsigned int) * 3 * GB_SEL_BINS, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(st, &h, sizeof(h), cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) {
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int blocks = std::max(1, std::min(GB_MAXRB, 2 * sms));
    for (int pass = 0; pass < 3; ++pass) {
      k_sel_hist<<<blocks, 256, 0, s>>>(st, d_v, n, hist + pass * GB_SEL_BINS, pass);
      k_sel_scan<<<1, 1024, 0, s>>>(st, hist + pass * GB_SEL_BINS, pass);
    }
    k_sort_thresh<<<tiles, 256, 0, s>>>(st, d_v, d_bins, n, tile_cnt);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpyAsync(&h, st, sizeof(h), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) {
    gb_set_error_message(cudaGetErrorString(e), __FILE__, __LINE__);
    rc = e == cudaErrorMemoryAllocation ? GB_OOM : GB_CUDA_ERROR;
  } else {
    *T_out = h.sort_T;
  }
  cudaFree(tile_cnt);
  cudaFree(hist);
  cudaFree(st);
  return rc;
}

// ------------------------------------------------------------------ component helpers
// S := ascending { j : v_j != 0 }, with the ordered compaction of the solver
__global__ void __launch_bounds__(256) k_nonzero_count(const float *__restrict__ v, int n, int *__restrict__ tile_cnt) {
  const int base = blockIdx.x * GB_TILE;
  int cnt = 0;
  for (int q = threadIdx.x; q < GB_TILE; q += blockDim.x) {
    const int i = base + q;
    if (i < n && v[i] != 0.0f) cnt++;
  }
  __shared__ float sm[32];
  const float tot = block_reduce<0>((float)cnt, sm);
  if (threadIdx.x == 0) tile_cnt[blockIdx.x] = (int)tot;
}

__global__ void __launch_bounds__(256) k_nonzero_compact(GbState *st, const float *__restrict__ v, int n,
                                                         const int *__restrict__ tile_cnt, int *__restrict__ S,
                                                         unsigned *__restrict__ bm) {
  __shared__ float sm[32];
  __shared__ int warp_base[8];
  __shared__ int s_off;
  float off = 0.0f;
  for (int t = threadIdx.x; t < (int)blockIdx.x; t += blockDim.x) off += (float)tile_cnt[t];
  const int offset = (int)block_reduce<0>(off, sm);
  if (threadIdx.x == 0) s_off = offset;
  __syncthreads();
  int running = s_off;
  const int base = blockIdx.x * GB_TILE;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  for (int q0 = 0; q0 < GB_TILE; q0 += blockDim.x) {
    const int i = base + q0 + threadIdx.x;
    const bool in = i < n && v[i] != 0.0f;
    const unsigned bal = __ballot_sync(0xffffffffu, in);
    if (lane == 0) warp_base[wid] = __popc(bal);
    if (bm && lane == 0) bm[i >> 5] = bal;
    __syncthreads();
    int wb = 0, tot = 0;
    for (int w2 = 0; w2 < 8; ++w2) {
      if (w2 < wid) wb += warp_base[w2];
      tot += warp_base[w2];
    }
    if (in) S[running + wb + __popc(bal & ((1u << lane) - 1u))] = i;
    running += tot;
    __syncthreads();
  }
  if (blockIdx.x == gridDim.x - 1 && threadIdx.x == 0) st->s_cnt = running;
}

// (and the expander's support bitmap when the products read it)
void enq_support_of_nonzeros(GbWork &w, cudaStream_t s, const float *v, int n) {
  const int tiles = (n + GB_TILE - 1) / GB_TILE;
  k_nonzero_count<<<tiles, 256, 0, s>>>(v, n, w.tile_cnt);
  k_nonzero_compact<<<tiles, 256, 0, s>>>(w.st, v, n, w.tile_cnt, w.S, w.smv_bm_ok ? w.smv_bm : nullptr);
}
