// gb_ctrl.cuh -- the reference's per-iteration scalar logic, run on the device.
//
// Each phase is a straight restatement of the host code between two device operations in
// GAGA/gaga/algorithms.cu (NIHT_S_gen, HTP_S_gen, CGIHT_S_gen) and GAGA/gaga/functions.cu
// (RestrictedSD/CG steps).  Included by the single-trial solver (one thread runs a phase)
// and by the shared-matrix batched form (one thread per trial).
#pragma once
#include "gb_internal.cuh"

// LinearBinning (GAGA/gaga/kernels.cu:135-146), bit-exact.  The double-precision test
// (double)t > (double)intercept * 1e-6 equals t > F in float with F the double product
// rounded toward -inf.  float -> int stores use round-toward-zero with saturation and
// NaN -> 0, as the reference's compiled kernel does; `slope*intercept + 1.0f` is one
// fused multiply-add there and here.
static __device__ __forceinline__ int lin_bin(float v, float slope, float intercept, float small_f, bool &counted) {
  const float t = fabsf(v);
  if (t > small_f) {
    counted = true;
    return __float2int_rz(fmaxf(0.0f, __fmul_rn(slope, __fsub_rn(intercept, t))));
  }
  counted = false;
  return __float2int_rz(__fmaf_rn(slope, intercept, 1.0f));
}


// ------------------------------------------------------------------ control phases
enum {
  C_INIT0,        // after ||y||^2 : err, err_start
  C_INIT_BINPREP, // after A^T y and max|x| : decide binning
  C_BINPREP,      // new max|x| and slope when binning
  C_INIT_DONE,    // after threshold : (CGIHT needs more) evaluate the loop condition
  C_CGIHT_INIT,   // CGIHT prologue after r0 = y - A x
  C_PUSH_RES,     // push sqrt(red[R_RES]) into prev[]
  C_SD_MU,        // RestrictedSD step size and maxChange; binning decision
  C_NIHT_STOP,
  C_HTP_CGINIT,
  C_HTP_CG1,
  C_HTP_CG2,
  C_HTP_CG3,
  C_HTP_STOP,
  C_RCG_BETA,
  C_RCG_ALPHA,
  C_UCG_BETA,
  C_UCG_ALPHA,
  C_CGIHT_BINDEC,
  C_CGIHT_POST,
  C_CGIHT_STOP,
  C_L0_INIT,
  C_L0_PRE,
  C_L0_STOP,
  C_IHT_INIT,     // IHT: bins keep the scale of A^T y; first loop test
  C_IHT_PREP,     // IHT: maxChange = 2 mu max|grad|; binning decision
  C_IHT_STOP,     // IHT: residual history and stopping rules (no cycle test)
  C_HTSD_MU,      // ThresholdSD: RestrictedSD step size, support kept
  C_HTSD_STOP,    // ThresholdSD: stopping rules
  C_HTCG_INIT,    // ThresholdCG: CG start on the thresholded support
  C_HTCG_STOP,    // ThresholdCG: squared-residual history and stopping rules
  C_CSMPSP_INIT_DONE,  // CSMPSP: after the first CG projection (counts as an iteration)
  C_CSMPSP_GBIN,  // CSMPSP: bins of the gradient (forced binning, k-th bin to k_bin_prev)
  C_CSMPSP_JOIN,  // CSMPSP: back to the support of x before joining
  C_CSMPSP_CG3,   // CSMPSP: CG projection step bookkeeping (stall test disabled)
  C_CSMPSP_XBIN,  // CSMPSP: forced binning of x after the projection
  C_CSMPSP_STOP,  // CSMPSP: residual history and stopping rules (fail after 125)
  C_FH_INIT1,     // FIHT/ALPS/CGIHTprojected: residNorm_prev[15] = ||y - A x||
  C_FH_BIN,       // FIHT/ALPS: forced binning of x (minVal = 0, maxChange = 1)
  C_FH_INIT2,     // FIHT/ALPS: after the extra first iteration; first loop test
  C_FH_TAU,       // FIHT/ALPS: extrapolation weight tau
  C_FH_MU,        // FIHT/ALPS: step mu = <v,v>/<Av,Av> (1 when guarded out)
  C_ALPS_LBIN,    // ALPS: local binning of the gradient outside supp(v), outer state kept
  C_ALPS_LRESTORE,// ALPS: outer bin state back
  C_FH_STOP,      // FIHT/ALPS/CGIHTprojected: residual history, stopping rules
  C_CP_INIT2,     // CGIHTprojected: first loop test
  C_CP_MU,        // CGIHTprojected: step mu for the active branch
  C_CP_BIN,       // CGIHTprojected: forced binning in the steepest-descent branch
  C_CP_BETA,      // CGIHTprojected: CG direction weight
  C_CP_PROJ,      // CGIHTprojected: projection fraction -> next branch
  C_SMP_INIT,     // smp: err of the zero start, first loop test
  C_SMP_HK,       // smp: H_k's fresh binning of the vector whose max is in red[R_XMAX]
  C_SMP_STOP,     // smp: residual history and stopping rules
  C_SEQ_INIT,     // ssmp / er: err of the start, records, first loop test
  C_SEQ_STOP,     // ssmp / er: residual history (ssmp) or cycle test (er), stopping rules
  C_SEQ_END1,     // ssmp: reopen the predicates for the final H_k
  C_SEQ_END2      // ssmp: close them again
};

static __device__ float max_list(const float *a, int n) {
  float m = a[0];
  for (int j = 1; j < n; ++j)
    if (a[j] > m) m = a[j];
  return m;
}

static __device__ float sqrt_red(const GbState *st, int slot) { return (float)sqrt(st->red[slot]); }

// stopping test of the reference loops, e.g. GAGA/gaga/algorithms.cu:1365
static __device__ int keep_going(GbState *st) {
  int go = (st->err > st->tol) & (st->iter < st->maxiter) & (st->err < (100.0f * st->err_start)) &
           ((double)st->resid_diff > 0.01 * (double)st->tol) & (st->fail == 0) & (st->cycle != 0);
  if (!go && st->stop_reason == 0) {
    if (!(st->err > st->tol)) st->stop_reason = 1;
    else if (!(st->iter < st->maxiter)) st->stop_reason = 2;
    else if (!(st->err < 100.0f * st->err_start)) st->stop_reason = 3;
    else if (!((double)st->resid_diff > 0.01 * (double)st->tol)) st->stop_reason = 4;
    else if (st->cycle == 0) st->stop_reason = 5;
    else st->stop_reason = 6;
  }
  return go;
}

// residual bookkeeping after each outer iteration (algorithms.cu:1398-1421)
static __device__ void stop_update(GbState *st, int fail_after) {
  for (int j = 0; j < 15; ++j) st->evol[j] = st->evol[j + 1];
  st->evol[15] = st->prev[14] - st->prev[15];
  st->resid_diff = max_list(st->evol, 16);
  // the timing variants have no cycle test and take the 1/16-th root
  // (GAGA/gaga/algorithms_timings.cu:610-624, 1509-1523)
  if (!st->timing)
    for (int j = 0; j < 15; ++j)
      if ((st->prev[15] == st->prev[j]) && (st->iter > 4)) st->cycle = 0;
  if (st->iter > fail_after) {
    float root = st->timing ? 1.0f / 16.0f : 1.0f / 15.0f;
    float rate = st->prev[15] / st->prev[0];
    rate = powf(rate, root);
    if (rate > 0.999f) st->fail = 1;
  }
}

static __device__ void push16(float *a, float v) {
  for (int j = 0; j < 15; ++j) a[j] = a[j + 1];
  a[15] = v;
}

static __device__ void finish_iteration(GbState *st, int fail_after) {
  stop_update(st, fail_after);
  st->iter++;
  st->passes++;
  st->active = keep_going(st);
  if (st->passes > st->pass_limit && st->active) {
    st->active = 0;
    st->status = GB_WATCHDOG;
  }
}

// FIHT / ALPS step-size guard factor: 1000 in the reference's _dct forms, 400 in _gen, _smv
static __device__ __forceinline__ float fiht_guard(const GbState *st) {
  return st->op_kind == GB_OP_DCT ? 1000.0f : 400.0f;
}

// the binning decision shared by every algorithm: FindSupportSet's skip path
// (GAGA/gaga/functions.cu:401-403) or a new binning with a new max (algorithms.cu:1380-1383)
static __device__ void bin_decision(GbState *st) {
  if (st->min_val <= st->max_change) {
    st->flags[F_DOBIN] = 1;
  } else {
    st->flags[F_DOBIN] = 0;
    st->min_val = st->min_val - st->max_change;
  }
}

// The support decision after RestrictedSD (NIHT, HTP).  supportFlag 0 (and every
// non-timing solve) is FindSupportSet's skip-or-bin rule.  The timing variants
// (GAGA/gaga/algorithms_timings.cu:566-599): supportFlag 1 takes a new max when minVal <=
// maxChange and bins every iteration (C_BINPREP decides with the new max); supportFlag 2
// lowers the sort threshold T by maxChange while T > maxChange and sorts otherwise;
// supportFlag 3 sorts every iteration (FindSupportSet_sort, functions.cu:446-465); both set
// k_bin = 1.
static __device__ void support_decision(GbState *st) {
  if (st->supp_flag == 1) {
    st->newmax = (st->min_val <= st->max_change);
    st->flags[F_DOBIN] = 1;
  } else if (st->supp_flag >= 2) {
    st->flags[F_DOBIN] = 0;
    st->k_bin = 1;
    const float mc = st->supp_flag == 2 ? st->max_change : st->sort_T;
    if (st->sort_T > mc) {
      st->sort_T = st->sort_T - mc;
      st->flags[F_SORT] = 0;
    } else {
      st->flags[F_SORT] = 1;
    }
  } else {
    bin_decision(st);
  }
}

// IHT loop test (GAGA/gaga/algorithms.cu:416): NIHT's rules without the cycle test
static __device__ int iht_going(GbState *st) {
  const int go = (st->err > st->tol) & (st->iter < st->maxiter) & (st->err < (100.0f * st->err_start)) &
                 ((double)st->resid_diff > 0.01 * (double)st->tol) & (st->fail == 0);
  if (!go && st->stop_reason == 0) {
    if (!(st->err > st->tol)) st->stop_reason = 1;
    else if (!(st->iter < st->maxiter)) st->stop_reason = 2;
    else if (!(st->err < 100.0f * st->err_start)) st->stop_reason = 3;
    else if (!((double)st->resid_diff > 0.01 * (double)st->tol)) st->stop_reason = 4;
    else st->stop_reason = 6;
  }
  return go;
}

// ThresholdSD / ThresholdCG loop tests (algorithms.cu:861, 1937): tolerance, maxiter and a
// stall threshold (0.1 tol on norms for SD, 10 tol^2 on squared norms for CG)
static __device__ int ht_going(GbState *st, float err_tol, float stall_tol) {
  const int go = (st->err > err_tol) & (st->iter < st->maxiter) & (st->resid_diff > stall_tol);
  if (!go && st->stop_reason == 0) {
    if (!(st->err > err_tol)) st->stop_reason = 1;
    else if (!(st->iter < st->maxiter)) st->stop_reason = 2;
    else st->stop_reason = 4;
  }
  return go;
}

static __device__ void evolve16(GbState *st) {
  for (int j = 0; j < 15; ++j) st->evol[j] = st->evol[j + 1];
  st->evol[15] = st->prev[14] - st->prev[15];
  st->resid_diff = max_list(st->evol, 16);
}

static __device__ void pass_watchdog(GbState *st) {
  st->passes++;
  if (st->passes > st->pass_limit && st->active) {
    st->active = 0;
    st->status = GB_WATCHDOG;
  }
}

// In eager mode (no graph) the handle is 0 and the host reads GbState instead.
__device__ __forceinline__ void set_cond(cudaGraphConditionalHandle h, unsigned v) {
  if (h) cudaGraphSetConditional(h, v);
}

__device__ __forceinline__ void ctrl_phase(GbState *st, int phase, cudaGraphConditionalHandle h) {
  const int live = st->active;
  switch (phase) {
    case C_INIT0:
      st->err = sqrt_red(st, R_RES);
      st->err_start = st->err;
      break;
    case C_INIT_BINPREP:
      // max_value = MaxMagnitude(A^T y); slope = (num_bins-1)/max_value; HTP passes
      // max_value as maxChange to force the first binning (algorithms.cu:1335-1354,2575)
      st->max_value = (float)st->red[R_XMAX];
      st->slope = ((float)(st->num_bins - 1) / st->max_value);
      st->max_change =
          (st->alg == GB_ALG_HTP || st->alg == GB_ALG_CSMPSP || st->alg == GB_ALG_CGIHT_PROJ) ? st->max_value : 1.0f;
      bin_decision(st);
      break;
    case C_BINPREP:
      // if (minVal <= maxChange) { max_value = MaxMagnitude(d_vec,n); slope = ...; }
      if (live && st->supp_flag == 1) {
        // FindSupportSet(..., maxChange = max_value): bins unless minVal > max_value
        if (st->newmax) {
          st->max_value = (float)st->red[R_XMAX];
          st->slope = ((float)(st->num_bins - 1) / st->max_value);
        }
        if (st->min_val <= st->max_value) {
          st->flags[F_DOBIN] = 1;
        } else {
          st->flags[F_DOBIN] = 0;
          st->min_val = st->min_val - st->max_value;
        }
      } else if (live && st->flags[F_DOBIN]) {
        st->max_value = (float)st->red[R_XMAX];
        st->slope = ((float)(st->num_bins - 1) / st->max_value);
      }
      break;
    case C_INIT_DONE:
      if (st->alg == GB_ALG_HT_SD) {
        st->active = ht_going(st, st->tol, (float)(0.1 * (double)st->tol));
        set_cond(h, st->active ? 1u : 0u);
      } else if (st->alg != GB_ALG_CGIHT) {
        st->active = keep_going(st);
        set_cond(h, st->active ? 1u : 0u);
      }
      break;
    case C_IHT_INIT:
      // max_value = MaxMagnitude(A^T y); slope; x = 0 (algorithms.cu:399-405)
      st->max_value = (float)st->red[R_XMAX];
      st->slope = ((float)(st->num_bins - 1) / st->max_value);
      st->max_change = 1.0f;
      st->active = iht_going(st);
      set_cond(h, st->active ? 1u : 0u);
      break;
    case C_IHT_PREP:
      if (!live) break;
      st->max_change = 2.0f * st->mu * (float)st->red[R_GMAX];
      bin_decision(st);
      break;
    case C_IHT_STOP:
      if (live) {
        st->err = sqrt_red(st, R_RES);
        push16(st->prev, st->err);
        evolve16(st);
        if (st->iter > 749) {
          float rate = st->prev[15] / st->prev[0];
          rate = powf(rate, 1.0f / 15.0f);
          if (rate > 0.999f) st->fail = 1;
        }
        st->iter++;
        st->active = iht_going(st);
        pass_watchdog(st);
      }
      set_cond(h, st->active ? 1u : 0u);
      break;
    case C_HTSD_MU: {
      if (!live) break;
      // RestrictedSD_S_gen step size (functions.cu:715-744); the support stays fixed
      float err2 = sqrt_red(st, R_AXT);
      float mu = sqrt_red(st, R_XT);
      if (mu < 400.0f * err2) {
        mu = mu / err2;
        mu = mu * mu;
      } else {
        mu = 0.0f;
      }
      st->mu = mu;
      st->flags[F_DOBIN] = 0;
      break;
    }
    case C_HTSD_STOP:
      if (live) {
        st->err = st->prev[15];
        evolve16(st);
        st->iter++;
        st->active = ht_going(st, st->tol, (float)(0.1 * (double)st->tol));
        pass_watchdog(st);
      }
      set_cond(h, st->active ? 1u : 0u);
      break;
    case C_CSMPSP_INIT_DONE:
      // err = sqrt(errCG); residNorm_prev[15] = err; iter++ (algorithms.cu:3491-3495)
      st->err = sqrtf(st->err_cg);
      st->prev[15] = st->err;
      st->iter = 1;
      st->active = keep_going(st);
      set_cond(h, st->active ? 1u : 0u);
      break;
    case C_CSMPSP_GBIN:
      if (!live) break;
      // max_value = MaxMagnitude(grad); minVal = 0; FindSupportSet(grad, ..., max_value)
      // into d_bin_grad / k_bin_grad (algorithms.cu:3519-3526).  CSMPSP_S_dct does not
      // reset minVal (algorithms.cu:2907), so its FindSupportSet may skip the binning and
      // keep the previous gradient bins and k_bin_grad.
      st->max_value = (float)st->red[R_XMAX];
      if (st->op_kind != GB_OP_DCT) st->min_val = 0.0f;
      st->slope = ((float)(st->num_bins - 1) / st->max_value);
      st->max_change = st->max_value;
      bin_decision(st);
      st->flags[F_KBIN_ALT] = 1;
      break;
    case C_CSMPSP_JOIN:
      st->flags[F_KBIN_ALT] = 0;
      break;
    case C_CSMPSP_CG3:
      if (st->flags[F_CG] && live) {
        push16(st->prev_cg, (float)st->red[R_RES]);
        st->err_cg = st->prev_cg[15];
        st->it_cg++;
        for (int j = 0; j < 15; ++j) st->evol_cg[j] = st->evol_cg[j + 1];
        st->evol_cg[15] = st->prev_cg[14] - st->prev_cg[15];
        // CSMPSP_S_gen disables the stall test here (algorithms.cu:3600); the _dct and _smv
        // forms keep it (algorithms.cu:2963,3285)
        st->diff_cg = st->op_kind == GB_OP_DENSE ? 10.0f : max_list(st->evol_cg, 16);
        st->flags[F_CG] = (st->err_cg > st->tol_cg) & (st->it_cg < 15) & (st->diff_cg > st->tol2);
      } else {
        st->flags[F_CG] = 0;
      }
      set_cond(h, (st->flags[F_CG] && live) ? 1u : 0u);
      break;
    case C_CSMPSP_XBIN:
      if (!live) break;
      // forced binning of x (algorithms.cu:3606-3612); without the minVal reset in the _dct
      // form (algorithms.cu:2973)
      st->max_value = (float)st->red[R_XMAX];
      if (st->op_kind != GB_OP_DCT) st->min_val = 0.0f;
      st->slope = ((float)(st->num_bins - 1) / st->max_value);
      st->max_change = st->max_value;
      bin_decision(st);
      break;
    case C_CSMPSP_STOP:
      if (live) {
        st->err = sqrt_red(st, R_RES);
        push16(st->prev, st->err);
        finish_iteration(st, 125);
      }
      set_cond(h, st->active ? 1u : 0u);
      break;
    case C_FH_INIT1:
      st->err = sqrt_red(st, R_RES);
      st->prev[15] = st->err;
      break;
    case C_FH_BIN:
      if (!live) break;
      st->min_val = 0.0f;
      st->max_change = 1.0f;
      st->max_value = (float)st->red[R_XMAX];
      st->slope = ((float)(st->num_bins - 1) / st->max_value);
      st->flags[F_DOBIN] = 1;
      break;
    case C_FH_INIT2:
      st->err = sqrt_red(st, R_RES);
      push16(st->prev, st->err);
      evolve16(st);
      st->active = keep_going(st);
      set_cond(h, st->active ? 1u : 0u);
      break;
    case C_FH_TAU: {
      if (!live) break;
      // RestrictedFIHT/ALPS (GAGA/gaga/functions.cu:1680-1686); the guard is 1000 x the
      // denominator in the _dct forms (functions.cu:1867,1948), 400 x otherwise
      float tau = (float)st->red[R_DOT1], tmp = (float)st->red[R_DOT2];
      if (fabsf(tau) < fiht_guard(st) * fabsf(tmp)) tau = tau / tmp;
      else tau = 0.0f;
      st->cg_beta = tau;
      break;
    }
    case C_FH_MU: {
      if (!live) break;
      // functions.cu:1733 and algorithms.cu:5633 (1000 x in the _dct forms: functions.cu:1918,
      // algorithms.cu:5912)
      float mu = (float)st->red[R_XT], tmp = (float)st->red[R_AXT];
      if (mu < fiht_guard(st) * tmp) mu = mu / tmp;
      else mu = 1.0f;
      st->mu = mu;
      break;
    }
    case C_ALPS_LBIN:
      if (!live) break;
      // FindSupportSet on v with the bin state passed by value (functions.cu:1803-1807)
      st->sv_alpha = st->alpha_bin;
      st->sv_max_bin = st->max_bin;
      st->sv_min_val = st->min_val;
      st->sv_k_bin = st->k_bin;
      st->min_val = 0.0f;
      st->max_value = (float)st->red[R_XMAX];
      st->slope = ((float)(st->num_bins - 1) / st->max_value);
      st->flags[F_DOBIN] = 1;
      break;
    case C_ALPS_LRESTORE:
      if (!live) break;
      st->alpha_bin = st->sv_alpha;
      st->max_bin = st->sv_max_bin;
      st->min_val = st->sv_min_val;
      st->k_bin = st->sv_k_bin;
      break;
    case C_FH_STOP:
      if (live) {
        st->err = sqrt_red(st, R_RES);
        push16(st->prev, st->err);
        finish_iteration(st, 749);
      }
      set_cond(h, st->active ? 1u : 0u);
      break;
    case C_CP_INIT2:
      for (int j = 0; j < 15; ++j) st->evol[j] = st->evol[j + 1];
      st->evol[15] = st->prev[14] - st->prev[15];
      st->flags[F_UCG] = 1;  // steepest-descent branch first
      st->flags[F_RCG] = 0;
      st->active = keep_going(st);
      set_cond(h, st->active ? 1u : 0u);
      break;
    case C_CP_MU: {
      if (!live) break;
      // mu = <v,v> / <Ap,Ap> (SD: Ap = A v), 1 when guarded out (algorithms.cu:4578-4582)
      float mu = (float)st->red[R_DOT1], tmp = (float)st->red[R_DOT2];
      if (mu < 400.0f * tmp) mu = mu / tmp;
      else mu = 1.0f;
      st->mu = mu;
      break;
    }
    case C_CP_BIN:
      if (!live) break;
      st->flags[F_DOBIN] = st->flags[F_UCG];
      if (st->flags[F_UCG]) {
        st->min_val = 0.0f;
        st->max_change = 1.0f;
        st->max_value = (float)st->red[R_XMAX];
        st->slope = ((float)(st->num_bins - 1) / st->max_value);
      }
      break;
    case C_CP_BETA: {
      if (!live || !st->flags[F_RCG]) break;
      float beta = (float)st->red[R_DOT3], tmp = (float)st->red[R_DOT4];
      if (beta < 400.0f * tmp) beta = beta / tmp;
      else beta = 0.0f;
      st->cg_beta = beta;
      break;
    }
    case C_CP_PROJ:
      if (live) {
        // proj_frac = ||grad - p|| / ||v|| decides the next branch (algorithms.cu:4637-4648)
        float pf = (float)sqrt(st->red[R_DOT1]), tmp = (float)sqrt(st->red[R_XT]);
        int supp;
        if (pf < 1000.0f * tmp) {
          pf = pf / tmp;
          supp = pf > st->proj_frac_tol ? 1 : 0;
        } else {
          supp = 1;
        }
        st->flags[F_UCG] = supp;
        st->flags[F_RCG] = !supp;
        st->err = sqrt_red(st, R_RES);
        push16(st->prev, st->err);
        finish_iteration(st, 749);
      }
      set_cond(h, st->active ? 1u : 0u);
      break;
    case C_HTCG_INIT:
      // mu = <grad_prev, grad_prev>; err = ||y - A x||^2 into residNorm_prev[15]
      // (algorithms.cu:1900-1911)
      st->mu = (float)st->red[R_DOT1];
      st->err = (float)st->red[R_RES];
      st->prev[15] = st->err;
      st->active = ht_going(st, st->tol_cg, st->tol2);
      st->flags[F_CG] = st->active;
      set_cond(h, st->active ? 1u : 0u);
      break;
    case C_HTCG_STOP:
      if (live) {
        push16(st->prev, (float)st->red[R_RES]);
        st->err = st->prev[15];
        evolve16(st);
        st->iter++;
        st->active = ht_going(st, st->tol_cg, st->tol2);
        pass_watchdog(st);
        st->flags[F_CG] = st->active;
      }
      set_cond(h, st->active ? 1u : 0u);
      break;
    case C_CGIHT_INIT:
      st->err = sqrt_red(st, R_RES);
      st->err_warm0 = st->err;
      st->prev[15] = st->err;
      for (int j = 0; j < 15; ++j) st->evol[j] = st->evol[j + 1];
      st->evol[15] = st->prev[14] - st->prev[15];
      st->beta_to_zero = 1;
      st->supp_change = 1;
      st->k_bin_prev = 0;
      st->flags[F_UCG] = st->restart ? 0 : 1;
      st->flags[F_RCG] = st->restart ? 1 : 0;
      st->flags[F_RESX] = st->flags[F_RCG];
      st->flags[F_RESR] = 0;
      st->supp_same = 0;
      st->active = keep_going(st);
      set_cond(h, st->active ? 1u : 0u);
      break;
    case C_PUSH_RES:
      if (!live) break;
      push16(st->prev, sqrt_red(st, R_RES));
      break;
    case C_SD_MU: {
      if (!live) break;
      // RestrictedSD_S_gen (GAGA/gaga/functions.cu:715-744)
      float err2 = sqrt_red(st, R_AXT);
      float mu = sqrt_red(st, R_XT);
      if (mu < 400.0f * err2) {
        mu = mu / err2;
        mu = mu * mu;
      } else {
        mu = 0.0f;
      }
      st->mu = mu;
      st->max_change = 2.0f * mu * (float)st->red[R_GMAX];
      support_decision(st);
      break;
    }
    case C_NIHT_STOP:
      if (live) {
        if (st->op_kind == GB_OP_DENSE) st->bytes += dense_bytes(st, 1, 2);
        st->err = st->prev[15];
        finish_iteration(st, 749);
      }
      set_cond(h, st->active ? 1u : 0u);
      break;
    case C_HTP_CGINIT:
      if (!live) {
        st->flags[F_CG] = 0;
        set_cond(h, 0u);
        break;
      }
      for (int j = 0; j < 16; ++j) { st->prev_cg[j] = 0.0f; st->evol_cg[j] = 1.0f; }
      st->diff_cg = 1.0f;
      st->prev_cg[15] = st->prev[15];
      st->mu = (float)st->red[R_DOT1];
      st->err_cg = (float)st->red[R_RES];
      st->prev_cg[15] = st->err_cg;
      st->it_cg = 0;
      st->flags[F_CG] = (st->err_cg > st->tol_cg) & (st->it_cg < 15) & (st->diff_cg > st->tol2);
      set_cond(h, st->flags[F_CG] ? 1u : 0u);
      break;
    case C_HTP_CG1: {
      // RestrictedCG_S_gen (GAGA/gaga/functions.cu:944-950)
      float alpha = (float)st->red[R_CG];
      if (st->mu < 1000.0f * alpha) alpha = st->mu / alpha;
      else alpha = 0.0f;
      st->cg_alpha = alpha;
      break;
    }
    case C_HTP_CG2: {
      float beta = st->mu;
      st->mu = (float)st->red[R_DOT3];
      if (st->mu < 1000.0f * beta) beta = st->mu / beta;
      else beta = 0.0f;
      st->cg_beta = beta;
      break;
    }
    case C_HTP_CG3:
      if (st->flags[F_CG] && live) {
        push16(st->prev_cg, (float)st->red[R_RES]);
        st->err_cg = st->prev_cg[15];
        st->it_cg++;
        for (int j = 0; j < 15; ++j) st->evol_cg[j] = st->evol_cg[j + 1];
        st->evol_cg[15] = st->prev_cg[14] - st->prev_cg[15];
        st->diff_cg = max_list(st->evol_cg, 16);
        st->flags[F_CG] = (st->err_cg > st->tol_cg) & (st->it_cg < 15) & (st->diff_cg > st->tol2);
      } else {
        st->flags[F_CG] = 0;
      }
      set_cond(h, (st->flags[F_CG] && live) ? 1u : 0u);
      break;
    case C_HTP_STOP:
      if (live) {
        if (st->op_kind == GB_OP_DENSE) st->bytes += dense_bytes(st, 2 + st->it_cg, 3 + 2 * st->it_cg);
        st->err = sqrtf(st->err_cg);
        push16(st->prev, st->err);
        finish_iteration(st, 125);
      }
      set_cond(h, st->active ? 1u : 0u);
      break;
    case C_RCG_BETA: {
      if (!live || !st->flags[F_RCG]) break;
      // RestrictedCGwithSupportEvolution (GAGA/gaga/functions.cu:1054-1064)
      float beta;
      if (st->beta_to_zero == 1) {
        beta = 0.0f;
        st->mu = (float)st->red[R_XT];
      } else {
        beta = st->mu;
        st->mu = (float)st->red[R_XT];
        if (st->mu < 1000.0f * beta) beta = st->mu / beta;
        else beta = 0.0f;
      }
      st->cg_beta = beta;
      break;
    }
    case C_RCG_ALPHA: {
      if (!live || !st->flags[F_RCG]) break;
      float alpha = (float)st->red[R_AXT];
      if (st->mu < 1000.0f * alpha) alpha = st->mu / alpha;
      else alpha = 0.0f;
      st->cg_alpha = alpha;
      st->max_change = 2.0f * alpha * (float)st->red[R_GMAX];
      break;
    }
    case C_UCG_BETA:
      if (!live || !st->flags[F_UCG]) break;
      // UnrestrictedCG (GAGA/gaga/functions.cu:1169-1178)
      if (st->beta_to_zero == 1) st->cg_beta = 0.0f;
      else st->cg_beta = -((float)st->red[R_DOT1]) / (float)st->red[R_DOT2];
      break;
    case C_UCG_ALPHA:
      if (!live || !st->flags[F_UCG]) break;
      st->cg_alpha = ((float)st->red[R_DOT3]) / (float)st->red[R_DOT4];
      st->mu = (float)st->red[R_XT];
      st->max_change = 2.0f * st->cg_alpha * (float)st->red[R_GMAX];
      break;
    case C_CGIHT_BINDEC:
      if (!live) break;
      // CGIHT_S_gen (GAGA/gaga/algorithms.cu:3849-3899)
      st->beta_to_zero = 0;
      if (st->min_val <= st->max_change) {
        st->flags[F_DOBIN] = 1;
        st->k_bin_prev = st->k_bin;
        st->changed = 0;
        st->s_cnt_prev = st->s_cnt;
      } else {
        st->flags[F_DOBIN] = 0;
        st->supp_change = 0;
        st->min_val = st->min_val - st->max_change;
        st->supp_same = 1;  // no binning: the same bins threshold x
      }
      st->flags[F_REMASK] = 0;
      break;
    case C_CGIHT_POST:
      if (!live || !st->flags[F_DOBIN]) break;
      st->supp_change = st->changed ? 1 : 0;
      // no entry left and as many entries as before: the same support set
      st->supp_same = !st->changed && st->s_cnt == st->s_cnt_prev;
      if (st->supp_change) {
        if (st->restart) st->beta_to_zero = 1;
        else st->flags[F_REMASK] = 1;
      }
      break;
    case C_CGIHT_STOP:
      if (live) {
        // passes over A_S: 2 for the unrestricted step (y - A x and A p share one), 2 for the
        // restricted one, 1 when its residual came from the recurrence
        if (st->op_kind == GB_OP_DENSE)
          st->bytes += dense_bytes(st, 1, st->flags[F_RESR] ? 1 : 2);
        const bool was_rcg = st->flags[F_RCG] != 0;
        st->err = st->prev[15];
        finish_iteration(st, 749);
        // learned warm start: give up when the residual has not dropped below the warm
        // start's within 10 iterations (the caller then solves from zero)
        if (st->learned && st->iter == 10 && st->active && !(st->err < st->err_warm0)) {
          st->active = 0;
          st->fell_back = 1;
          st->stop_reason = 8;
        }
        if (st->restart) { st->flags[F_UCG] = 0; st->flags[F_RCG] = 1; }
        else { st->flags[F_UCG] = st->supp_change ? 1 : 0; st->flags[F_RCG] = st->supp_change ? 0 : 1; }
        // x moved by alpha p on an unchanged support: r - alpha A p is y - A x in exact
        // arithmetic; every rec_every-th iteration recomputes it from x
        const bool rec = st->rec_every > 0 && was_rcg && st->supp_same && !st->supp_change &&
                         (st->iter % st->rec_every) != 0;
        st->flags[F_RESR] = st->flags[F_RCG] && rec;
        st->flags[F_RESX] = st->flags[F_RCG] && !rec;
      }
      set_cond(h, st->active ? 1u : 0u);
      break;
    default:
      break;
  }
}


// ------------------------------------------------------------------ batched trials
// The fields of GbState a batched trial starts from (dense operator, its own m, n, k).
static __device__ void batch_trial_fields(GbState *st, int trial, int m, int n, int k, int maxiter, int alg) {
  st->trial = trial;
  st->m = m;
  st->n = n;
  st->k = k;
  st->num_bins = max(n / 20, 1000);
  st->maxiter = maxiter;
  st->alg = alg;
  st->restart = 0;
  st->op_kind = GB_OP_DENSE;
  st->active = 1;
  for (int f = 0; f < GB_NFLAG; ++f) st->flags[f] = 0;
  st->flags[F_ALWAYS] = 1;
  st->bytes = 0.0;
}

// The solver's initial state of a batched trial (initial_state of the single-trial solver)
// with tol = tol_rel ||y||, red[R_RES] holding ||y||^2.
static __device__ void batch_solver_init(GbState *st, float tol_rel, int learned) {
  const float tol = tol_rel * (float)sqrt(st->red[R_RES]);
  st->tol = tol;
  st->iter = 0; st->fail = 0; st->cycle = 1; st->passes = 0; st->pass_limit = st->maxiter + 4;
  st->status = 0; st->stop_reason = 0;
  st->err = 0.0f; st->err_start = 0.0f; st->resid_diff = 1.0f;
  for (int j = 0; j < 16; ++j) { st->prev[j] = 0.0f; st->evol[j] = 1.0f; }
  st->alpha_bin = 0.25f;
  st->max_bin = (int)((float)st->num_bins * (1.0f - st->alpha_bin));
  st->k_bin = 0; st->sum = 0; st->k_bin_prev = 0;
  st->min_val = 0.0f; st->slope = 0.0f; st->max_value = 0.0f; st->max_change = 0.0f;
  st->mu = 0.0f; st->cg_alpha = 0.0f; st->cg_beta = 0.0f;
  st->beta_to_zero = 1; st->supp_change = 1;
  st->it_cg = 0; st->tol_cg = tol * tol; st->tol2 = 10.0f * st->tol_cg;
  for (int f = 0; f < GB_NFLAG; ++f) st->flags[f] = 0;
  st->flags[F_ALWAYS] = 1;
  st->changed = 0;
  st->bytes = 0.0;
  st->learned = learned;
  st->fell_back = 0;
  st->err_warm0 = 0.0f;
}
