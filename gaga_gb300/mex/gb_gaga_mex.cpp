/*
 * gb_gaga_mex.cpp -- MATLAB MEX gateways over libgb_cs.so: drop-in replacements for GAGA's
 * gaga_gen, gaga_dct and gaga_smv (GAGA/gaga/gaga_gen.cu:41-848, gaga_dct.cu:40-831,
 * gaga_smv.cu:39-1198), so that gaga_cs.m and gagaOptions.m work unchanged.
 *
 * Build one MEX file per gateway with GB_MEX_GATEWAY set to 1 (gen), 2 (dct) or 3 (smv):
 *     mex -DGB_MEX_GATEWAY=1 -I<repo>/include gb_gaga_mex.cpp -L<repo>/gaga_gb300/lib -lgb_cs \
 *         -output gaga_gen
 * Usages (argument order, classes and outputs as the reference's):
 *   [norms times iters support convRate x] = gaga_gen(alg, k, m, n[, opts])
 *   [x iters convRate] = gaga_gen(alg, y, A, k[, opts])
 *   [norms times iters support convRate x] = gaga_dct(alg, k, m, n[, opts])
 *   [x iters convRate] = gaga_dct(alg, y, rows, k, m, n[, opts])            rows 1-based
 *   [norms times iters support convRate x resRecord timeRecord] = gaga_smv(alg, k, m, n, p[, opts])
 *   [x iters convRate resRecord timeRecord] = gaga_smv(alg, y, rows, cols, vals, k[, opts])
 * opts is gagaOptions' l x 2 cell of names and typed values (single, int32, uint32, char).
 * Errors: the reference prints and returns without outputs; this shim reports the library's
 * status text through mexErrMsgIdAndTxt("gaga:gb_cs", ...).
 */
#include <stdlib.h>
#include <string.h>

#include <vector>

#include "gb_cs.h"
#include "mex.h"

#ifndef GB_MEX_GATEWAY
#define GB_MEX_GATEWAY 1
#endif

namespace {

bool str_eq(const mxArray *a, const char *s) {
  char buf[64];
  return mxGetString(a, buf, sizeof buf) == 0 && strcmp(buf, s) == 0;
}

// gagaOptions' name/value cell (GAGA/gaga/gagaOptions.m, parsed as in gaga_gen.cu:204-321)
// into the library's options; names the reference does not know are reported.
void parse_options(const mxArray *cell, gb_options *o, int *noise_on) {
  if (!mxIsCell(cell) || mxGetN(cell) != 2) return;
  const int num = (int)mxGetM(cell);
  for (int i = 0; i < num; ++i) {
    int subs[2] = {i, 0};
    const mxArray *name = mxGetCell(cell, mxCalcSingleSubscript(cell, 2, subs));
    subs[1] = 1;
    const mxArray *val = mxGetCell(cell, mxCalcSingleSubscript(cell, 2, subs));
    char buf[64];
    if (!name || !val || mxGetString(name, buf, sizeof buf) != 0) continue;
    const void *d = mxGetData(val);
    if (!strcmp(buf, "tol")) o->tol = *(const float *)d;
    else if (!strcmp(buf, "maxiter")) o->maxiter = *(const int *)d;
    else if (!strcmp(buf, "numBins")) o->num_bins = *(const int *)d;
    else if (!strcmp(buf, "noise")) { o->noise = *(const float *)d; *noise_on = 1; }
    else if (!strcmp(buf, "projFracTol")) o->proj_frac_tol = *(const float *)d;
    else if (!strcmp(buf, "gpuNumber")) o->gpu_number = *(const int *)d;
    else if (!strcmp(buf, "convRateNum")) o->conv_rate_num = *(const int *)d;
    else if (!strcmp(buf, "seed")) o->seed = *(const unsigned int *)d;
    else if (!strcmp(buf, "alpha")) o->alpha = *(const float *)d;
    else if (!strcmp(buf, "supportFlag")) o->support_flag = *(const int *)d;
    else if (!strcmp(buf, "l0_thresh")) o->l0_thresh = *(const int *)d;
    else if (!strcmp(buf, "vecDistribution"))
      o->vec_distribution = str_eq(val, "binary") ? 1 : str_eq(val, "uniform") ? 0 : str_eq(val, "gaussian") ? 2
                                                                                                 : o->vec_distribution;
    else if (!strcmp(buf, "kFixed")) o->k_fixed = str_eq(val, "on") ? 1 : 0;
    else if (!strcmp(buf, "restartFlag")) o->restart_flag = str_eq(val, "on") ? 1 : 0;
    else if (!strcmp(buf, "timing")) o->timing = str_eq(val, "on") ? 1 : 0;
    else if (!strcmp(buf, "matrixEnsemble")) {
      if (GB_MEX_GATEWAY == 1) o->matrix_ensemble = str_eq(val, "binary") ? 2 : 1;
      else o->matrix_ensemble = str_eq(val, "ones") ? 1 : str_eq(val, "binary") ? 2 : 3;
    } else if (strncmp(buf, "threadsPerBlock", 15) != 0 && strcmp(buf, "debug_mode") != 0 &&
               strcmp(buf, "band_percentage") != 0)
      mexPrintf("The following option is not recognised: %s\n", buf);
  }
}

template <class T>
mxArray *column(int rows, mxClassID cls, const T *src) {
  mxArray *a = mxCreateNumericMatrix(rows, 1, cls, mxREAL);
  if (src) memcpy(mxGetData(a), src, sizeof(T) * rows);
  return a;
}

bool fail(gb_status s) {
  if (s == GB_OK) return false;
  mexErrMsgIdAndTxt("gaga:gb_cs", "%s", gb_cs_last_error());
  return true;
}

// generate-and-solve outputs: norms, times, iters (int32), support (int32), convRate, x
void put_generate_outputs(mxArray *plhs[], const gb_result &r, const std::vector<float> &x) {
  plhs[0] = column(3, mxSINGLE_CLASS, r.norms);
  plhs[1] = column(3, mxSINGLE_CLASS, r.times);
  plhs[2] = column(1, mxINT32_CLASS, &r.iter);
  plhs[3] = column(4, mxINT32_CLASS, r.support);
  plhs[4] = column(1, mxSINGLE_CLASS, &r.conv_rate);
  plhs[5] = column((int)x.size(), mxSINGLE_CLASS, x.data());
}

}  // namespace

void mexFunction(int nlhs, mxArray *plhs[], int nrhs, const mxArray *prhs[]) {
  const int gen_out = GB_MEX_GATEWAY == 3 ? 8 : 6, given_out = GB_MEX_GATEWAY == 3 ? 5 : 3;
  if ((nlhs != gen_out && nlhs != given_out) || nrhs < 4) {
    mexErrMsgIdAndTxt("gaga:gb_cs", "usage: see the reference's gaga_%s",
                      GB_MEX_GATEWAY == 1 ? "gen" : GB_MEX_GATEWAY == 2 ? "dct" : "smv");
    return;
  }
  char alg[64];
  if (mxGetString(prhs[0], alg, sizeof alg) != 0 || gb_cs_alg_id(alg) < 0) {
    mexErrMsgIdAndTxt("gaga:gb_cs", "unknown algorithm");
    return;
  }
  const mxArray *opts = mxIsCell(prhs[nrhs - 1]) ? prhs[nrhs - 1] : nullptr;
  const int kind = GB_MEX_GATEWAY == 1 ? GB_OP_DENSE : GB_MEX_GATEWAY == 2 ? GB_OP_DCT : GB_OP_SMV;
  gb_result r;
  memset(&r, 0, sizeof r);
  int noise_on = 0;
  if (nlhs == gen_out) {
    // generate and solve: (alg, k, m, n[, p][, opts])
    const int k = (int)mxGetScalar(prhs[1]), m = (int)mxGetScalar(prhs[2]), n = (int)mxGetScalar(prhs[3]);
    const int d = GB_MEX_GATEWAY == 3 ? (int)mxGetScalar(prhs[4]) : 0;
    gb_options o;
    gb_cs_default_options(&o, alg, n);
    o.results_dir = "";  // the reference appends its result line in MATLAB's current directory
    if (opts) parse_options(opts, &o, &noise_on);
    std::vector<float> x(n), xt(n), rec, trec;
    if (GB_MEX_GATEWAY == 3) {
      rec.assign((size_t)o.maxiter + 1, 0.0f);
      trec.assign((size_t)o.maxiter + 1, 0.0f);
      r.res_record = rec.data();
      r.time_record = trec.data();
    }
    if (fail(gb_cs_generate_and_solve(alg, kind, k, m, n, d, &o, x.data(), xt.data(), &r))) return;
    put_generate_outputs(plhs, r, x);
    if (GB_MEX_GATEWAY == 3) {
      plhs[6] = column((int)rec.size(), mxSINGLE_CLASS, rec.data());
      plhs[7] = column((int)trec.size(), mxSINGLE_CLASS, trec.data());
    }
    return;
  }
  gb_problem p;
  memset(&p, 0, sizeof p);
  p.kind = kind;
  p.location = GB_HOST;
  p.index_base = 1;  // MATLAB indices (the reference shifts them down on the device)
  p.y = (const float *)mxGetData(prhs[1]);
  if (GB_MEX_GATEWAY == 1) {  // (alg, y, A, k[, opts]): A is column-major m x n
    p.A = (const float *)mxGetData(prhs[2]);
    p.m = (int)mxGetM(prhs[2]);
    p.n = (int)mxGetN(prhs[2]);
    p.lda = p.m;
    p.k = (int)mxGetScalar(prhs[3]);
  } else if (GB_MEX_GATEWAY == 2) {  // (alg, y, rows, k, m, n[, opts])
    p.rows = (const int *)mxGetData(prhs[2]);
    p.k = (int)mxGetScalar(prhs[3]);
    p.m = (int)mxGetScalar(prhs[4]);
    p.n = (int)mxGetScalar(prhs[5]);
  } else {  // (alg, y, rows, cols, vals, k[, opts]); p, m, n inferred (gaga_smv.cu:166-182)
    p.rows = (const int *)mxGetData(prhs[2]);
    p.cols = (const int *)mxGetData(prhs[3]);
    p.vals = (const float *)mxGetData(prhs[4]);
    p.k = (int)mxGetScalar(prhs[5]);
    const int nz = (int)mxGetM(prhs[4]);
    int d = 1;
    while (d < nz && p.cols[d - 1] == p.cols[d]) ++d;
    int m = p.rows[0], n = p.cols[0];
    for (int e = 1; e < nz; ++e) {
      if (p.rows[e] > m) m = p.rows[e];
      if (p.cols[e] > n) n = p.cols[e];
    }
    p.d = d;
    p.m = m;
    p.n = n;
  }
  gb_options o;
  gb_cs_default_options(&o, alg, p.n);
  if (opts) parse_options(opts, &o, &noise_on);
  std::vector<float> x(p.n), rec, trec;
  if (GB_MEX_GATEWAY == 3) {
    rec.assign((size_t)o.maxiter + 1, 0.0f);
    trec.assign((size_t)o.maxiter + 1, 0.0f);
    r.res_record = rec.data();
    r.time_record = trec.data();
  }
  if (fail(gb_cs_solve(alg, &p, &o, x.data(), &r))) return;
  plhs[0] = column(p.n, mxSINGLE_CLASS, x.data());
  plhs[1] = column(1, mxINT32_CLASS, &r.iter);  // int32, as gaga_gen.cu:125-126 creates it
  plhs[2] = column(1, mxSINGLE_CLASS, &r.conv_rate);
  if (GB_MEX_GATEWAY == 3) {
    plhs[3] = column((int)rec.size(), mxSINGLE_CLASS, rec.data());
    plhs[4] = column((int)trec.size(), mxSINGLE_CLASS, trec.data());
  }
}
