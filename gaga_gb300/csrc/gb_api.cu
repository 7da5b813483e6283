// gb_api.cu -- the C ABI (include/gb_cs.h): validation, device layout, entry points.
//
// The reference gateways (GAGA/gaga/gaga_gen.cu, gaga_dct.cu, gaga_smv.cu) parse MATLAB
// arguments, allocate device buffers, upload or generate the problem, run one algorithm
// and pack results.  The same steps are done here for plain C buffers; every
// allocation is released before returning, as in the reference (re-entrant: no globals
// on the solve path).
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include <algorithm>
#include <string>
#include <thread>
#include <vector>

#include "gb_internal.cuh"
#include "gb_resident.h"
#include "gb_philox.cuh"

gb_status gb_ops_init_attributes();

static thread_local std::string g_last_error;

void gb_set_error_message(const char *msg, const char *file, int line) {
  char buf[512];
  snprintf(buf, sizeof(buf), "%s (%s:%d)", msg, file, line);
  g_last_error = buf;
}

static gb_status bad(const char *msg, gb_status code = GB_BAD_ARG) {
  g_last_error = msg;
  return code;
}

extern "C" const char *gb_cs_version(void) { return "gb_cs 1.0 (sm_103a)"; }
extern "C" const char *gb_cs_last_error(void) { return g_last_error.c_str(); }

extern "C" int gb_cs_alg_id(const char *alg) {
  if (!alg) return -1;
  if (!strcmp(alg, "NIHT")) return GB_ALG_NIHT;
  if (!strcmp(alg, "HTP")) return GB_ALG_HTP;
  if (!strcmp(alg, "IHT")) return GB_ALG_IHT;
  if (!strcmp(alg, "ThresholdSD")) return GB_ALG_HT_SD;
  if (!strcmp(alg, "ThresholdCG")) return GB_ALG_HT_CG;
  if (!strcmp(alg, "CSMPSP")) return GB_ALG_CSMPSP;
  if (!strcmp(alg, "FIHT")) return GB_ALG_FIHT;
  if (!strcmp(alg, "ALPS")) return GB_ALG_ALPS;
  if (!strcmp(alg, "CGIHTprojected")) return GB_ALG_CGIHT_PROJ;
  if (!strcmp(alg, "CGIHT")) return GB_ALG_CGIHT;
  if (!strcmp(alg, "parallel_l0")) return GB_ALG_PARALLEL_L0;
  if (!strcmp(alg, "parallel_lddsr")) return GB_ALG_PARALLEL_LDDSR;
  if (!strcmp(alg, "smp")) return GB_ALG_SMP;
  if (!strcmp(alg, "parallel_l0_swipe")) return GB_ALG_PARALLEL_L0_SWIPE;
  if (!strcmp(alg, "ssmp")) return GB_ALG_SSMP;
  if (!strcmp(alg, "er")) return GB_ALG_ER;
  if (!strcmp(alg, "ssmp_naive")) return GB_ALG_SSMP_NAIVE;
  if (!strcmp(alg, "er_naive")) return GB_ALG_ER_NAIVE;
  return -1;
}

extern "C" void gb_cs_default_options(gb_options *o, const char *alg, int n) {
  memset(o, 0, sizeof(*o));
  o->tol = (float)(10 ^ (-4));  // the reference's default, C XOR (GAGA/gaga/gaga_gen.cu:183)
  o->tol_is_relative = 0;
  o->maxiter = (alg && !strcmp(alg, "HTP")) ? 300 : 5000;
  o->num_bins = std::max(n / 20, 1000);
  o->restart_flag = 0;
  o->l0_thresh = 1;
  o->vec_distribution = 1;
  o->matrix_ensemble = 0;  // 0: the operator's own default (gen 1, smv 3)
  o->k_fixed = 0;
  o->seed = 0;
  o->noise = 0.0f;
  o->gpu_number = 0;
  o->conv_rate_num = 16;
  o->alpha = 0.25f;
  o->support_flag = 0;
  o->timing = 0;
  o->proj_frac_tol = 3.0f;
  o->watchdog_passes = 0;
}

// ------------------------------------------------------------------ workspace
namespace {

struct DeviceBuffers {
  std::vector<void *> ptrs;
  ~DeviceBuffers() {
    for (void *p : ptrs) cudaFree(p);
  }
  template <class T>
  gb_status alloc(T **p, size_t count, bool zero = true) {
    void *q = nullptr;
    size_t bytes = std::max<size_t>(count, 1) * sizeof(T);
    cudaError_t e = cudaMalloc(&q, bytes);
    if (e != cudaSuccess) {
      gb_set_error_message(cudaGetErrorString(e), __FILE__, __LINE__);
      return GB_OOM;
    }
    ptrs.push_back(q);
    if (zero) {
      e = cudaMemset(q, 0, bytes);
      if (e != cudaSuccess) {
        gb_set_error_message(cudaGetErrorString(e), __FILE__, __LINE__);
        return GB_CUDA_ERROR;
      }
    }
    *p = (T *)q;
    return GB_OK;
  }
};

int ilog2(int v) {
  int l = 0;
  while ((1 << l) < v) ++l;
  return l;
}

gb_status select_device(int gpu) {
  int count = 0;
  if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) return bad("no CUDA device", GB_NO_DEVICE);
  if (gpu < 0 || gpu >= count) gpu = 0;  // gaga_gen.cu:233-241 resets to 0
  GB_CUDA_TRY(cudaSetDevice(gpu));
  static std::atomic<unsigned long long> attr_done{0};
  return gb_once_per_device(attr_done, gb_ops_init_attributes);
}

gb_status alloc_work(DeviceBuffers &db, GbWork &w, int m, int n, int lda, int num_bins, int maxiter) {
  int dev = 0;
  GB_CUDA_TRY(cudaGetDevice(&dev));
  GB_CUDA_TRY(cudaDeviceGetAttribute(&w.num_sms, cudaDevAttrMultiProcessorCount, dev));
  w.red_blocks = std::min(GB_MAXRB, w.num_sms * 2);
  w.wide_blocks = w.num_sms * 8;
  GB_TRY(db.alloc(&w.st, 1));
  GB_TRY(db.alloc(&w.red_part, (size_t)GB_NSLOT * GB_MAXRB));
  GB_TRY(db.alloc(&w.tickets, GB_NSLOT));
  GB_TRY(db.alloc(&w.x, n));
  GB_TRY(db.alloc(&w.xt, n));
  GB_TRY(db.alloc(&w.grad, n));
  GB_TRY(db.alloc(&w.gp, n));
  GB_TRY(db.alloc(&w.gpt, n));
  GB_TRY(db.alloc(&w.upd, n));
  GB_TRY(db.alloc(&w.y, lda));
  GB_TRY(db.alloc(&w.resid, lda));
  GB_TRY(db.alloc(&w.ru, lda));
  GB_TRY(db.alloc(&w.am1, lda));
  GB_TRY(db.alloc(&w.am2, lda));
  GB_TRY(db.alloc(&w.bins, n));
  GB_TRY(db.alloc(&w.bins_prev, n));
  GB_TRY(db.alloc(&w.counters, std::max(num_bins, 1)));
  GB_TRY(db.alloc(&w.S, n));
  GB_TRY(db.alloc(&w.tile_cnt, 2 * ((n + GB_TILE - 1) / GB_TILE)));  // second half: smp's k-th bin counts
  GB_TRY(db.alloc(&w.rec, (size_t)maxiter + 2));
  GB_TRY(db.alloc(&w.sel_hist, (size_t)3 * GB_SEL_BINS));  // zeroed; the select keeps it zero
  gb_dense_av_shape(m, w.num_sms, false, &w.av_ntile, &w.av_nsplit, &w.av_rows);
  w.part_cap = gb_dense_part_floats_av(w.av_ntile, w.av_nsplit, w.av_rows);
  GB_TRY(db.alloc(&w.av_tickets, w.av_ntile));
  return GB_OK;
}

// Normalise a problem onto the device.  Host data is copied; dense A gets a leading
// dimension rounded up to 32 floats (128-byte aligned columns).
// Sets *flag when a rows x cols column-major block (leading dimension ld) holds NaN or Inf:
// one pass over the caller's data, read back with the solve's final state.
__global__ void k_nonfinite(const float *__restrict__ a, int rows, int cols, int ld, int *flag) {
  int bad = 0;
  for (int j = blockIdx.x; j < cols; j += gridDim.x)
    for (int i = threadIdx.x; i < rows; i += blockDim.x) bad |= !isfinite(__ldg(a + (size_t)j * ld + i));
  if (__syncthreads_or(bad) && threadIdx.x == 0) atomicOr(flag, 1);
}

gb_status setup_problem(DeviceBuffers &db, GbWork &w, const gb_problem &p, cudaStream_t s, int num_bins,
                        int maxiter, bool need_y = true) {
  GbOp &op = w.op;
  memset(&op, 0, sizeof(op));
  op.kind = p.kind;
  op.m = p.m;
  op.n = p.n;
  const bool host = p.location == GB_HOST;
  const int base = p.index_base;
  if (p.kind == GB_OP_DENSE) {
    if (p.m <= 0 || p.n <= 0 || !p.A) return bad("dense problem needs m, n > 0 and A");
    const int lda_src = p.lda > 0 ? p.lda : p.m;
    if (lda_src < p.m) return bad("lda < m");
    if (host) {
      op.lda = (p.m + 31) / 32 * 32;
      float *A = nullptr;
      GB_TRY(db.alloc(&A, (size_t)op.lda * p.n, op.lda != p.m));
      GB_CUDA_TRY(cudaMemcpy2DAsync(A, (size_t)op.lda * 4, p.A, (size_t)lda_src * 4, (size_t)p.m * 4, p.n,
                                    cudaMemcpyHostToDevice, s));
      op.A = A;
    } else {
      op.lda = lda_src;
      op.A = p.A;
    }
    op.vec4 = (op.lda % 4 == 0) && (((uintptr_t)op.A & 15) == 0);
  } else if (p.kind == GB_OP_DCT) {
    if (p.n < 16 || (p.n & (p.n - 1))) return bad("DCT length must be a power of two >= 16", GB_UNSUPPORTED);
    if (p.m <= 0 || p.m > p.n || !p.rows) return bad("DCT problem needs 0 < m <= n and rows");
    if (p.n > (1 << 24)) return bad("DCT length above 2^24", GB_UNSUPPORTED);
    op.lda = p.m;
    op.logn = ilog2(p.n);
    op.log1 = op.logn / 2;
    op.log2 = op.logn - op.log1;
    std::vector<int> rows(p.m);
    if (host) memcpy(rows.data(), p.rows, sizeof(int) * p.m);
    else GB_CUDA_TRY(cudaMemcpy(rows.data(), p.rows, sizeof(int) * p.m, cudaMemcpyDeviceToHost));
    std::vector<char> seen(p.n, 0);
    for (int i = 0; i < p.m; ++i) {
      rows[i] -= base;  // indexShiftDown (GAGA/gaga/kernels.cu:155-159)
      if (rows[i] < 0 || rows[i] >= p.n) return bad("DCT row index out of range");
      if (seen[rows[i]]) return bad("DCT rows must be distinct");
      seen[rows[i]] = 1;
    }
    int *drows = nullptr;
    GB_TRY(db.alloc(&drows, p.m, false));
    GB_CUDA_TRY(cudaMemcpyAsync(drows, rows.data(), sizeof(int) * p.m, cudaMemcpyHostToDevice, s));
    GB_CUDA_TRY(cudaStreamSynchronize(s));
    op.rows = drows;
    GB_TRY(db.alloc(&op.cbuf0, p.n, false));
    GB_TRY(db.alloc(&op.cbuf1, p.n, false));
    GB_TRY(db.alloc(&op.freq, p.n, true));
  } else if (p.kind == GB_OP_SMV) {
    if (!p.rows || !p.vals) return bad("smv problem needs rows and vals");
    const int n = p.n, m = p.m, d = p.d;
    std::vector<int> cols;
    if (d <= 0) return bad("smv problem needs d, the number of nonzeros per column");
    if (n <= 0 || m <= 0) return bad("smv problem needs m, n > 0");
    const size_t nz = (size_t)n * d;
    std::vector<int> rows(nz);
    std::vector<float> vals(nz);
    if (host) {
      memcpy(rows.data(), p.rows, sizeof(int) * nz);
      memcpy(vals.data(), p.vals, sizeof(float) * nz);
      if (p.cols) cols.assign(p.cols, p.cols + nz);
    } else {
      GB_CUDA_TRY(cudaMemcpy(rows.data(), p.rows, sizeof(int) * nz, cudaMemcpyDeviceToHost));
      GB_CUDA_TRY(cudaMemcpy(vals.data(), p.vals, sizeof(float) * nz, cudaMemcpyDeviceToHost));
      if (p.cols) {
        cols.resize(nz);
        GB_CUDA_TRY(cudaMemcpy(cols.data(), p.cols, sizeof(int) * nz, cudaMemcpyDeviceToHost));
      }
    }
    for (size_t e = 0; e < nz; ++e)
      if (!std::isfinite(vals[e])) return bad("smv values hold non-finite values");
    for (size_t e = 0; e < nz; ++e) {
      rows[e] -= base;
      if (rows[e] < 0 || rows[e] >= m) return bad("smv row index out of range");
      if (!cols.empty() && cols[e] - base != (int)(e / d))
        return bad("smv entries must be grouped by column, d per column (GAGA/Matrices/smv_gpu.cu:52-59)");
    }
    // CSR copy, columns ascending inside each row (stable counting sort)
    std::vector<int> ptr(m + 1, 0), ccol(nz);
    std::vector<float> cval(nz);
    for (size_t e = 0; e < nz; ++e) ptr[rows[e] + 1]++;
    for (int i = 0; i < m; ++i) ptr[i + 1] += ptr[i];
    std::vector<int> fill(ptr.begin(), ptr.end() - 1);
    for (size_t e = 0; e < nz; ++e) {
      int q = fill[rows[e]]++;
      ccol[q] = (int)(e / d);
      cval[q] = vals[e];
    }
    int *drows, *dptr, *dcol;
    float *dvals, *dcval;
    GB_TRY(db.alloc(&drows, nz, false));
    GB_TRY(db.alloc(&dvals, nz, false));
    GB_TRY(db.alloc(&dptr, m + 1, false));
    GB_TRY(db.alloc(&dcol, nz, false));
    GB_TRY(db.alloc(&dcval, nz, false));
    GB_CUDA_TRY(cudaMemcpyAsync(drows, rows.data(), sizeof(int) * nz, cudaMemcpyHostToDevice, s));
    GB_CUDA_TRY(cudaMemcpyAsync(dvals, vals.data(), sizeof(float) * nz, cudaMemcpyHostToDevice, s));
    GB_CUDA_TRY(cudaMemcpyAsync(dptr, ptr.data(), sizeof(int) * (m + 1), cudaMemcpyHostToDevice, s));
    GB_CUDA_TRY(cudaMemcpyAsync(dcol, ccol.data(), sizeof(int) * nz, cudaMemcpyHostToDevice, s));
    GB_CUDA_TRY(cudaMemcpyAsync(dcval, cval.data(), sizeof(float) * nz, cudaMemcpyHostToDevice, s));
    GB_CUDA_TRY(cudaStreamSynchronize(s));
    op.lda = m;
    op.d = d;
    op.smv_rows = drows;
    op.smv_vals = dvals;
    op.csr_ptr = dptr;
    op.csr_col = dcol;
    op.csr_val = dcval;
    // one value for every entry (bitwise): the operator kernels multiply by it and stream no
    // values (the products, and so the sums, are the same floats)
    uint32_t v0;
    memcpy(&v0, vals.data(), sizeof(v0));
    op.smv_cv = 1;
    for (size_t e = 0; e < nz && op.smv_cv; ++e) {
      uint32_t ve;
      memcpy(&ve, &vals[e], sizeof(ve));
      op.smv_cv = ve == v0;
    }
    op.smv_cval = vals[0];
    op.smv_r16 = nullptr;
    if (m <= 65536) {
      std::vector<unsigned short> r16(nz);
      for (size_t e = 0; e < nz; ++e) r16[e] = (unsigned short)rows[e];
      unsigned short *dr16;
      GB_TRY(db.alloc(&dr16, nz, false));
      GB_CUDA_TRY(cudaMemcpyAsync(dr16, r16.data(), sizeof(unsigned short) * nz, cudaMemcpyHostToDevice, s));
      GB_CUDA_TRY(cudaStreamSynchronize(s));
      op.smv_r16 = dr16;
    }
  } else {
    return bad("unknown operator kind");
  }
  GB_TRY(alloc_work(db, w, op.m, op.n, op.lda, num_bins, maxiter));
  if (op.kind == GB_OP_DENSE) {
    GB_TRY(db.alloc(&w.part, 2 * w.part_cap, false));
    w.part_two = 1;
  }
  if (op.kind == GB_OP_SMV && op.n <= GB_SMV_BM_MAX_N)  // zero: the empty support of x = 0
    GB_TRY(db.alloc(&w.smv_bm, (size_t)(op.n + GB_TILE - 1) / GB_TILE * (GB_TILE / 32), true));
  if (need_y) {
    if (!p.y) return bad("y is required");
    GB_CUDA_TRY(cudaMemcpyAsync(w.y, p.y, sizeof(float) * op.m,
                                host ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice, s));
  }
  return GB_OK;
}

// the caller's dense A and y, once, into w.nonfinite (read back after the solve)
gb_status check_finite_inputs(DeviceBuffers &db, GbWork &w, cudaStream_t s) {
  GB_TRY(db.alloc(&w.nonfinite, 1));
  if (w.op.kind == GB_OP_DENSE)
    k_nonfinite<<<std::max(1, std::min(w.num_sms * 8, w.op.n)), 256, 0, s>>>(w.op.A, w.op.m, w.op.n, w.op.lda,
                                                                               w.nonfinite);
  k_nonfinite<<<1, 256, 0, s>>>(w.y, w.op.m, 1, w.op.m, w.nonfinite);
  GB_CUDA_TRY(cudaGetLastError());
  return GB_OK;
}

float conv_rate_from(const float *prev, int iter, int conv_num) {
  // given-data convRate (GAGA/gaga/gaga_gen.cu:733-741): temp = min(iter, convRateNum)
  int temp = std::min(iter, conv_num);
  if (temp <= 0) return 0.0f;
  float root = 1.0f / (float)temp;
  temp = conv_num - temp;
  return powf(prev[conv_num - 1] / prev[temp], root);
}

gb_status check_options(const gb_options &o) {
  if (o.maxiter < 0) return bad("maxiter must be >= 0");
  if (o.timing && (o.support_flag < 0 || o.support_flag > 3)) return bad("supportFlag must be 0, 1, 2 or 3");
  if (o.timing && !(o.alpha >= 0.0f && o.alpha < 1.0f)) return bad("alpha must be in [0, 1)");
  if (o.num_bins < 1) return bad("numBins must be >= 1");
  if (o.conv_rate_num != 16) return bad("convRateNum other than 16 is not supported", GB_UNSUPPORTED);
  return GB_OK;
}

bool timing_applies(const gb_options &o, int alg_id) {
  return o.timing && (alg_id == GB_ALG_NIHT || alg_id == GB_ALG_HTP);
}

// stamp buffers of the timing variants and of the expander decoders' time record
gb_status alloc_timing(DeviceBuffers &db, GbWork &w, const gb_options &o, int alg_id) {
  if (gb_is_ccs(alg_id)) GB_TRY(db.alloc(&w.tlog, (size_t)std::max(o.maxiter, 0) + 1));
  if (!timing_applies(o, alg_id) || o.maxiter <= 0) return GB_OK;
  GB_TRY(db.alloc(&w.tstamp, (size_t)o.maxiter * GB_NSTAMP));
  GB_TRY(db.alloc(&w.tcg, (size_t)o.maxiter));
  return GB_OK;
}

// Per-iteration times (ms) of a timing-variant solve from its stamps: iteration, support
// identification, CG steps and CG time (HTP).  Returns their sum over iterations (time_sum,
// algorithms_timings.cu:641).
struct TimingRecord {
  std::vector<float> iter_ms, supp_ms, cg_steps, cg_ms;
  float sum = 0.0f;
};
gb_status collect_timing(const GbWork &w, int iters, TimingRecord *t) {
  const int n = std::max(iters, 0);
  std::vector<unsigned long long> ts((size_t)n * GB_NSTAMP);
  std::vector<int> cg((size_t)n);
  if (n > 0) {
    GB_CUDA_TRY(cudaMemcpy(ts.data(), w.tstamp, sizeof(unsigned long long) * ts.size(), cudaMemcpyDeviceToHost));
    GB_CUDA_TRY(cudaMemcpy(cg.data(), w.tcg, sizeof(int) * cg.size(), cudaMemcpyDeviceToHost));
  }
  t->iter_ms.assign(n, 0.0f);
  t->supp_ms.assign(n, 0.0f);
  t->cg_steps.assign(n, 0.0f);
  t->cg_ms.assign(n, 0.0f);
  t->sum = 0.0f;
  auto ms = [](unsigned long long a, unsigned long long b) { return b >= a ? (float)((double)(b - a) * 1e-6) : 0.0f; };
  for (int j = 0; j < n; ++j) {
    const unsigned long long *q = &ts[(size_t)j * GB_NSTAMP];
    t->iter_ms[j] = ms(q[0], q[5]);
    t->supp_ms[j] = ms(q[1], q[2]);
    t->cg_ms[j] = ms(q[3], q[4]);
    t->cg_steps[j] = (float)cg[j];
    t->sum += t->iter_ms[j];
  }
  return GB_OK;
}

void put_timing(const TimingRecord &t, gb_result *r, int iters) {
  const size_t bytes = sizeof(float) * (size_t)std::max(iters, 0);
  if (r->time_per_iteration) memcpy(r->time_per_iteration, t.iter_ms.data(), bytes);
  if (r->time_supp_set) memcpy(r->time_supp_set, t.supp_ms.data(), bytes);
  if (r->cg_per_iteration) memcpy(r->cg_per_iteration, t.cg_steps.data(), bytes);
  if (r->time_for_cg) memcpy(r->time_for_cg, t.cg_ms.data(), bytes);
  // h_times[1] = time_sum / iter (GAGA/gaga/results.cu:1430)
  r->times[1] = iters > 0 ? t.sum / (float)iters : 0.0f;
}

// timeRecord of the expander decoders: ms from the loop start to the end of each iteration
gb_status put_time_record(const GbWork &w, int iters, int maxiter, float *out) {
  if (!out || !w.tlog) return GB_OK;
  const int n = std::min(std::max(iters, 0), maxiter);
  std::vector<unsigned long long> t((size_t)n + 1);
  GB_CUDA_TRY(cudaMemcpy(t.data(), w.tlog, sizeof(unsigned long long) * t.size(), cudaMemcpyDeviceToHost));
  memset(out, 0, sizeof(float) * ((size_t)maxiter + 1));
  for (int j = 1; j <= n; ++j) out[j] = t[j] >= t[0] ? (float)((double)(t[j] - t[0]) * 1e-6) : 0.0f;
  return GB_OK;
}

// a result's caller-owned pointers survive its reset
void reset_result(gb_result *r) {
  float *rec = r->res_record, *a = r->time_per_iteration, *b = r->time_supp_set, *c = r->cg_per_iteration,
        *d = r->time_for_cg, *tr = r->time_record;
  memset(r, 0, sizeof(*r));
  r->time_record = tr;
  r->res_record = rec;
  r->time_per_iteration = a;
  r->time_supp_set = b;
  r->cg_per_iteration = c;
  r->time_for_cg = d;
}

}  // namespace

// ------------------------------------------------------------------ gb_cs_solve
// Non-finite data: the reference's loops have no check (a NaN residual ends them through
// the comparisons of the stopping rules, GAGA/gaga/algorithms.cu:1365); here such a run
// returns GB_BAD_ARG instead of GB_OK.  ||y|| (err_start, or norm0 for the expander
// decoders) not finite: y holds NaN or Inf; the last residual norm not finite: A or y does.
static gb_status check_finite_run(const GbState &st, int alg_id) {
  const float start = gb_is_ccs(alg_id) ? st.norm0 : st.err_start;
  const float last = gb_is_ccs(alg_id) ? st.norm : st.err;
  if (!std::isfinite(start)) return bad("y holds non-finite values");
  if (!std::isfinite(last)) return bad("the residual norm is not finite: A or y holds non-finite values");
  return GB_OK;
}

extern "C" gb_status gb_cs_solve(const char *alg, const gb_problem *p, const gb_options *opts, float *x_out,
                                 gb_result *r) {
  if (!p || !x_out) return bad("null argument");
  const int alg_id = gb_cs_alg_id(alg);
  if (alg_id < 0) return bad("algorithm must be one of NIHT, HTP, IHT, ThresholdSD, ThresholdCG, CSMPSP, CGIHT, FIHT, ALPS, "
                         "CGIHTprojected, smp, ssmp, er, ssmp_naive, er_naive, parallel_l0, parallel_lddsr, parallel_l0_swipe");
  if (gb_is_ccs(alg_id) && p->kind != GB_OP_SMV) return bad("the expander decoders require the smv operator");
  gb_options o;
  if (opts) o = *opts;
  else gb_cs_default_options(&o, alg, p->n);
  GB_TRY(check_options(o));
  if (p->k < 0) return bad("k must be >= 0");
  if (p->location == GB_HOST && p->y)
    for (int i = 0; i < p->m; ++i)
      if (!std::isfinite(p->y[i])) return bad("y holds non-finite values");
  GB_TRY(select_device(o.gpu_number));
  cudaStream_t s = (cudaStream_t)p->stream;
  DeviceBuffers db;
  GbWork w;
  memset(&w, 0, sizeof(w));
  GB_TRY(setup_problem(db, w, *p, s, o.num_bins, o.maxiter));
  GB_TRY(check_finite_inputs(db, w, s));
  if (gb_is_ccs(alg_id)) {
    if (o.l0_thresh < 1 || o.l0_thresh > w.op.d) o.l0_thresh = 1;  // gaga_smv.cu:313
  }
  if (o.learned_params && alg_id == GB_ALG_CGIHT) {
    w.ml_params = o.learned_params;
    GB_TRY(db.alloc(&w.ml_counts, gb_ml_rank_bins()));
    GB_TRY(db.alloc(&w.ml_cum, gb_ml_rank_bins()));
  }
  GB_TRY(alloc_timing(db, w, o, alg_id));
  float tol_abs = o.tol;
  if (o.tol_is_relative) {
    std::vector<float> yh(p->m);
    GB_CUDA_TRY(cudaMemcpyAsync(yh.data(), w.y, sizeof(float) * p->m, cudaMemcpyDeviceToHost, s));
    GB_CUDA_TRY(cudaStreamSynchronize(s));
    double ss = 0.0;
    for (float v : yh) ss += (double)v * v;
    tol_abs = o.tol * (float)sqrt(ss);
  }
  cudaEvent_t e0, e1;
  GB_CUDA_TRY(cudaEventCreate(&e0));
  GB_CUDA_TRY(cudaEventCreate(&e1));
  GB_CUDA_TRY(cudaEventRecord(e0, s));
  GB_TRY(gb_run_solver(w, alg_id, o, p->k, s, tol_abs));
  GbState st;
  int warm = 0, warm_iters = 0;
  if (w.ml_params) {
    GB_CUDA_TRY(cudaMemcpyAsync(&st, w.st, sizeof(st), cudaMemcpyDeviceToHost, s));
    GB_CUDA_TRY(cudaStreamSynchronize(s));
    GB_TRY(gb_resident_check());
    warm = 1;
    if (st.fell_back) {
      // the warm start did not reduce the residual: plain zero-initialised CGIHT decides
      warm = 2;
      warm_iters = st.iter;
      w.ml_params = nullptr;
      GB_CUDA_TRY(cudaMemsetAsync(w.x, 0, sizeof(float) * p->n, s));
      GB_TRY(gb_run_solver(w, alg_id, o, p->k, s, tol_abs));
    }
  }
  GB_CUDA_TRY(cudaEventRecord(e1, s));
  GB_CUDA_TRY(cudaMemcpyAsync(&st, w.st, sizeof(st), cudaMemcpyDeviceToHost, s));
  int nonfinite = 0;
  GB_CUDA_TRY(cudaMemcpyAsync(&nonfinite, w.nonfinite, sizeof(int), cudaMemcpyDeviceToHost, s));
  GB_CUDA_TRY(cudaMemcpyAsync(x_out, w.x, sizeof(float) * p->n,
                              p->location == GB_HOST ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice, s));
  std::vector<float> rec;
  if (gb_is_ccs(alg_id)) {
    rec.resize((size_t)o.maxiter + 1);
    GB_CUDA_TRY(cudaMemcpyAsync(rec.data(), w.rec, sizeof(float) * (o.maxiter + 1), cudaMemcpyDeviceToHost, s));
  }
  GB_CUDA_TRY(cudaStreamSynchronize(s));
  GB_TRY(gb_resident_check());
  float ms = 0.0f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (r) {
    float *user_rec = r->res_record;
    reset_result(r);
    r->iter = st.iter + warm_iters;
    r->stop_reason = st.stop_reason;
    r->warm_start = warm;
    r->times[0] = ms;
    r->times[1] = st.iter > 0 ? ms / st.iter : 0.0f;
    r->times[2] = ms;
    if (w.tstamp) {
      TimingRecord t;
      GB_TRY(collect_timing(w, st.iter, &t));
      put_timing(t, r, st.iter);
    }
    if (gb_is_ccs(alg_id)) {
      // the last <= 16 residual records become residNorm_prev (gaga_smv.cu:1013-1020)
      for (int j = 0; j < std::min(st.iter, 16); ++j) r->resid_prev[15 - j] = rec[st.iter - j];
      if (user_rec) memcpy(user_rec, rec.data(), sizeof(float) * (o.maxiter + 1));
      GB_TRY(put_time_record(w, st.iter, o.maxiter, r->time_record));
    } else {
      memcpy(r->resid_prev, st.prev, sizeof(st.prev));
    }
    r->conv_rate = conv_rate_from(r->resid_prev, st.iter, 16);
  }
  if (nonfinite) return bad("A or y holds non-finite values");
  if (st.status == GB_WATCHDOG) return bad("device iteration bound reached", GB_WATCHDOG);
  GB_TRY(check_finite_run(st, alg_id));
  return GB_OK;
}

// ------------------------------------------------------------------ problem generation
// problem generation: Philox-4x32-10 streams (gb_philox.cuh)
namespace {
using gbgen::KEY_HI;
using gbgen::philox;
using gbgen::u01;
enum { ST_MATRIX = gbgen::ST_MATRIX, ST_VALUES = gbgen::ST_VALUES, ST_SUPPORT = gbgen::ST_SUPPORT,
       ST_ROWS = gbgen::ST_ROWS, ST_SMV = gbgen::ST_SMV, ST_SIGNS = gbgen::ST_SIGNS, ST_NOISE = gbgen::ST_NOISE };

// dense A, column-major with lda: one warp per column (gbgen::gen_dense_column)
__global__ void k_gen_dense(float *A, int m, int n, int lda, int ens, uint32_t seed, uint32_t trial) {
  const int lane = threadIdx.x & 31;
  const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, nw = (gridDim.x * blockDim.x) >> 5;
  for (int j = gw; j < n; j += nw) gbgen::gen_dense_column(A + (size_t)j * lda, j, m, seed, trial, ens, lane, 32);
}

float h_uniform(uint32_t seed, uint32_t trial, uint32_t stream, uint64_t e) {
  uint32_t o[4];
  philox((uint32_t)(e >> 2), (uint32_t)(e >> 34), stream, trial, seed, KEY_HI, o);
  return u01(o[e & 3]);
}
float h_gauss(uint32_t seed, uint32_t trial, uint32_t stream, uint64_t e) {
  uint32_t o[4];
  philox((uint32_t)(e >> 2), (uint32_t)(e >> 34), stream, trial, seed, KEY_HI, o);
  int lane = (int)(e & 3);
  uint32_t a = lane < 2 ? o[0] : o[2], b = lane < 2 ? o[1] : o[3];
  double r = sqrt(-2.0 * log((double)u01(a)));
  double t = 6.283185307179586 * u01(b);
  return (float)((lane & 1) ? r * sin(t) : r * cos(t));
}

#define GB_HOST_THREADS 16
// f(begin, end, part) over [0, count) split into at most GB_HOST_THREADS parts run on the
// host's cores (one part for small counts); part p only writes its own range and slot p
template <class F>
void host_parallel_for(int64_t count, F f) {
  const unsigned hw = std::max(1u, std::min((unsigned)GB_HOST_THREADS, std::thread::hardware_concurrency()));
  if (count < (1 << 15) || hw == 1) {
    f((int64_t)0, count, 0);
    return;
  }
  const int64_t chunk = (count + hw - 1) / hw;
  std::vector<std::thread> th;
  for (unsigned t = 0; t < hw; ++t) {
    const int64_t a = t * chunk, b = std::min<int64_t>(count, a + chunk);
    if (a < b) th.emplace_back(f, a, b, (int)t);
  }
  for (auto &x : th) x.join();
}

// createVector (GAGA/gaga/createVector.cu:207-300): the support is the set of entries whose
// uniform key falls in the top bins of an n-bin linear histogram, so |support| >= k.  One
// Philox block gives four consecutive entries (the values h_uniform / h_gauss return).
int gen_vector(int n, int k, int dist, uint32_t seed, uint32_t trial, float *x) {
  std::vector<float> keys(n), vals(n);
  const int64_t nblk = ((int64_t)n + 3) / 4;
  std::vector<float> part_max(GB_HOST_THREADS, 0.0f);
  host_parallel_for(nblk, [&](int64_t g0, int64_t g1, int part) {
    float mloc = 0.0f;
    for (int64_t g = g0; g < g1; ++g) {
      uint32_t ov[4], os[4];
      philox((uint32_t)g, (uint32_t)(g >> 32), ST_VALUES, trial, seed, KEY_HI, ov);
      philox((uint32_t)g, (uint32_t)(g >> 32), ST_SUPPORT, trial, seed, KEY_HI, os);
      for (int lane = 0; lane < 4; ++lane) {
        const int64_t i = g * 4 + lane;
        if (i >= n) break;
        const float u = u01(ov[lane]);
        float v;
        if (dist == 1) {
          v = signbit(u - 0.5f) ? -1.0f : 1.0f;
        } else if (dist == 2) {
          const uint32_t a = lane < 2 ? ov[0] : ov[2], b = lane < 2 ? ov[1] : ov[3];
          const double r = sqrt(-2.0 * log((double)u01(a)));
          const double t = 6.283185307179586 * u01(b);
          v = (float)((lane & 1) ? r * sin(t) : r * cos(t));
        } else {
          v = u;
        }
        vals[i] = v;
        keys[i] = u01(os[lane]);
        mloc = std::max(mloc, keys[i]);
      }
    }
    part_max[part] = mloc;
  });
  float mx = 0.0f;
  for (float v : part_max) mx = std::max(mx, v);
  const float slope = ((float)(n - 1) / mx);
  const double small = (double)mx * 0.000001;
  std::vector<int> bins(n), cnt(n, 0);
  for (int i = 0; i < n; ++i) {
    float t = keys[i];
    if ((double)t > small) {
      float b = fmaxf(0.0f, slope * (mx - t));
      bins[i] = (int)b;
      if (bins[i] < n) cnt[bins[i]]++;
    } else {
      bins[i] = n;
    }
  }
  int k_bin = 0, sum = 0;
  while ((sum < k) & (k_bin < n)) sum += cnt[k_bin++];
  k_bin -= 1;
  for (int i = 0; i < n; ++i) x[i] = bins[i] <= k_bin ? vals[i] : 0.0f;
  return sum;
}

}  // namespace

extern "C" gb_status gb_cs_generate_and_solve(const char *alg, int kind, int k, int m, int n, int d,
                                              const gb_options *opts, float *x_out, float *x_true_out,
                                              gb_result *r) {
  if (!x_out) return bad("null argument");
  const int alg_id = gb_cs_alg_id(alg);
  if (alg_id < 0) return bad("algorithm must be one of NIHT, HTP, IHT, ThresholdSD, ThresholdCG, CSMPSP, CGIHT, FIHT, ALPS, "
                         "CGIHTprojected, smp, ssmp, er, ssmp_naive, er_naive, parallel_l0, parallel_lddsr, parallel_l0_swipe");
  if (gb_is_ccs(alg_id) && kind != GB_OP_SMV) return bad("the expander decoders require the smv operator");
  if (k < 1 || m < 1 || n < 1 || (kind == GB_OP_SMV && d < 1)) return bad("k, m, n (and d) must be positive");
  gb_options o;
  if (opts) o = *opts;
  else gb_cs_default_options(&o, alg, n);
  GB_TRY(check_options(o));
  GB_TRY(select_device(o.gpu_number));
  cudaEvent_t t0, t1, t2;
  cudaEventCreate(&t0);
  cudaEventCreate(&t1);
  cudaEventCreate(&t2);
  cudaEventRecord(t0, 0);
  // x with the reference's support scheme; kFixed redraws with seed+1 until |supp| == k
  std::vector<float> xt(n);
  uint32_t seed = o.seed;
  int ks = gen_vector(n, k, o.vec_distribution, seed, 0, xt.data());
  if (o.k_fixed)
    for (int tries = 0; ks != k && tries < 1000; ++tries) ks = gen_vector(n, k, o.vec_distribution, ++seed, 0, xt.data());
  DeviceBuffers db;
  gb_problem p;
  memset(&p, 0, sizeof(p));
  p.kind = kind;
  p.m = m;
  p.n = n;
  p.k = ks;
  p.location = GB_HOST;
  std::vector<int> rows;
  std::vector<float> vals;
  std::vector<float> dummyA;
  float *dA = nullptr;
  int lda = (m + 31) / 32 * 32;
  if (kind == GB_OP_DENSE) {
    // A drawn on the device straight into the padded layout
    GB_TRY(db.alloc(&dA, (size_t)lda * n, true));
    int ens = o.matrix_ensemble == 2 ? 2 : 1;
    k_gen_dense<<<2048, 256>>>(dA, m, n, lda, ens, seed, 0);
    GB_CUDA_TRY(cudaGetLastError());
    p.location = GB_DEVICE;
    p.A = dA;
    p.lda = lda;
  } else if (kind == GB_OP_DCT) {
    // m of n rows by the reference's partial shuffle (createProblem_kernels.cu:65-75)
    std::vector<int> idx(n);
    for (int i = 0; i < n; ++i) idx[i] = i;
    // the swaps are sequential, their uniforms are not: one Philox block per four j
    std::vector<float> uj(n, 0.0f);
    const int64_t jlo = n - m + 1;  // j runs n-1 .. n-m+1
    host_parallel_for(((int64_t)n + 3) / 4 - jlo / 4, [&](int64_t a, int64_t b, int) {
      for (int64_t gi = a; gi < b; ++gi) {
        const int64_t g = jlo / 4 + gi;
        uint32_t o[4];
        philox((uint32_t)g, (uint32_t)(g >> 32), ST_ROWS, 0, seed, KEY_HI, o);
        for (int lane = 0; lane < 4; ++lane) {
          const int64_t j = g * 4 + lane;
          if (j >= jlo && j < n) uj[j] = u01(o[lane]);
        }
      }
    });
    for (int j = n - 1; j > n - m; --j) {
      int kk = (int)((float)j * uj[j]);
      std::swap(idx[j], idx[kk]);
    }
    rows.resize(m);
    for (int j = 0; j < m; ++j) rows[j] = idx[n - 1 - j];
    p.rows = rows.data();
  } else {
    int ens = o.matrix_ensemble ? o.matrix_ensemble : 3;
    if (gb_is_ccs(alg_id)) ens = 3;  // ccs algorithms force ones (gaga_smv.cu:403-405)
    rows.resize((size_t)n * d);
    vals.resize((size_t)n * d);
    float scale = (ens == 1 || ens == 2) ? 1.0f / sqrtf((float)d) : 1.0f;
    host_parallel_for(n, [&](int64_t j0, int64_t j1, int) {
    for (int j = (int)j0; j < (int)j1; ++j) {
      int have = 0;
      uint32_t draw = 0;
      while (have < d) {
        uint32_t q[4];
        philox((uint32_t)j, draw++, ST_SMV, 0, seed, KEY_HI, q);
        for (int t = 0; t < 4 && have < d; ++t) {
          int rr = (int)((float)m * u01(q[t]));
          if (rr == m) rr = m - 1;
          bool dup = false;
          for (int u = 0; u < have; ++u) dup |= rows[(size_t)j * d + u] == rr;
          if (!dup) rows[(size_t)j * d + have++] = rr;
        }
      }
      for (int t = 0; t < d; ++t) {
        float v = 1.0f;
        if (ens == 2) v = signbit(h_uniform(seed, 0, ST_SIGNS, (uint64_t)j * d + t) - 0.5f) ? -1.0f : 1.0f;
        vals[(size_t)j * d + t] = v * scale;
      }
    }
    });
    p.rows = rows.data();
    p.vals = vals.data();
    p.d = d;
  }
  GbWork w;
  memset(&w, 0, sizeof(w));
  GB_TRY(setup_problem(db, w, p, 0, o.num_bins, o.maxiter, false));
  GB_TRY(alloc_timing(db, w, o, alg_id));
  // y = A x (createMeasurements_*), then optional noise (createProblem_gen.cu:244-254)
  float *dxt = nullptr;
  GB_TRY(db.alloc(&dxt, n, false));
  GB_CUDA_TRY(cudaMemcpy(dxt, xt.data(), sizeof(float) * n, cudaMemcpyHostToDevice));
  {
    GbState st0;
    memset(&st0, 0, sizeof(st0));
    st0.active = 1;
    st0.flags[F_ALWAYS] = 1;
    GB_CUDA_TRY(cudaMemcpy(w.st, &st0, sizeof(st0), cudaMemcpyHostToDevice));
    enq_support_of_nonzeros(w, 0, dxt, n);
    enq_A(w, 0, dxt, w.y, nullptr, -1, F_ALWAYS);
    GB_CUDA_TRY(cudaGetLastError());
  }
  if (o.noise > 0.0f) {
    std::vector<float> yh(m);
    GB_CUDA_TRY(cudaMemcpy(yh.data(), w.y, sizeof(float) * m, cudaMemcpyDeviceToHost));
    double yn = 0, en = 0;
    std::vector<float> e(m);
    for (int i = 0; i < m; ++i) {
      e[i] = h_gauss(seed, 0, ST_NOISE, i);
      en += (double)e[i] * e[i];
      yn += (double)yh[i] * yh[i];
    }
    float scale = o.noise * (float)(sqrt(yn) / sqrt(en));
    for (int i = 0; i < m; ++i) yh[i] = fmaf(scale, e[i], yh[i]);
    GB_CUDA_TRY(cudaMemcpy(w.y, yh.data(), sizeof(float) * m, cudaMemcpyHostToDevice));
  }
  GB_CUDA_TRY(cudaMemset(w.x, 0, sizeof(float) * n));
  if (gb_is_ccs(alg_id) && (o.l0_thresh < 1 || o.l0_thresh > d)) o.l0_thresh = 1;
  float tol_abs = o.tol;
  if (o.tol_is_relative) {
    std::vector<float> yh(m);
    GB_CUDA_TRY(cudaMemcpy(yh.data(), w.y, sizeof(float) * m, cudaMemcpyDeviceToHost));
    double ss = 0;
    for (float v : yh) ss += (double)v * v;
    tol_abs = o.tol * (float)sqrt(ss);
  }
  cudaEventRecord(t1, 0);
  GB_TRY(gb_run_solver(w, alg_id, o, ks, 0, tol_abs));
  cudaEventRecord(t2, 0);
  GbState st;
  GB_CUDA_TRY(cudaMemcpy(&st, w.st, sizeof(st), cudaMemcpyDeviceToHost));
  GB_TRY(gb_resident_check());
  GB_CUDA_TRY(cudaMemcpy(x_out, w.x, sizeof(float) * n, cudaMemcpyDeviceToHost));
  std::vector<float> rec;
  if (gb_is_ccs(alg_id)) {
    rec.resize((size_t)o.maxiter + 1);
    GB_CUDA_TRY(cudaMemcpy(rec.data(), w.rec, sizeof(float) * (o.maxiter + 1), cudaMemcpyDeviceToHost));
  }
  float ms_alg = 0, ms_tot = 0;
  cudaEventElapsedTime(&ms_alg, t1, t2);
  cudaEventElapsedTime(&ms_tot, t0, t2);
  cudaEventDestroy(t0);
  cudaEventDestroy(t1);
  cudaEventDestroy(t2);
  if (x_true_out) memcpy(x_true_out, xt.data(), sizeof(float) * n);
  gb_result local_r;
  memset(&local_r, 0, sizeof(local_r));
  if (!r && o.results_dir) r = &local_r;
  TimingRecord trec;
  if (w.tstamp) GB_TRY(collect_timing(w, st.iter, &trec));
  if (r) {
    float *user_rec = r->res_record;
    reset_result(r);
    r->iter = st.iter;
    r->k_used = ks;
    r->stop_reason = st.stop_reason;
    if (gb_is_ccs(alg_id)) {
      for (int j = 0; j < std::min(st.iter, 16); ++j) r->resid_prev[15 - j] = rec[st.iter - j];
      if (user_rec) memcpy(user_rec, rec.data(), sizeof(float) * (o.maxiter + 1));
      GB_TRY(put_time_record(w, st.iter, o.maxiter, r->time_record));
    } else {
      memcpy(r->resid_prev, st.prev, sizeof(st.prev));
    }
    // generate-mode convRate (GAGA/gaga/results.cu:365-378)
    int temp = std::min(st.iter, 16);
    if (temp <= 1) r->conv_rate = 0.0f;
    else {
      temp = temp - 1;
      float root = 1.0f / (float)temp;
      temp = 15 - temp;
      r->conv_rate = powf(r->resid_prev[15] / r->resid_prev[temp], root);
    }
    // relative errors and support counts (GAGA/gaga/results.cu:408-487)
    double l1 = 0, l2 = 0, li = 0, e1 = 0, e2 = 0, ei = 0;
    int tp = 0, tn = 0;
    for (int i = 0; i < n; ++i) {
      if (xt[i] != 0.0f) { if (x_out[i] != 0.0f) tp++; }
      else if (x_out[i] == 0.0f) tn++;
      double a = fabs((double)xt[i]), e = fabs((double)xt[i] - (double)x_out[i]);
      l1 += a; l2 += a * a; li = std::max(li, a);
      e1 += e; e2 += e * e; ei = std::max(ei, e);
    }
    r->norms[0] = (float)(e1 / l1);
    r->norms[1] = (float)(sqrt(e2) / sqrt(l2));
    r->norms[2] = (float)(ei / li);
    r->support[0] = tp;
    r->support[1] = ks - tp;
    r->support[2] = tn;
    r->support[3] = n - ks - tn;
    r->times[0] = ms_alg;
    r->times[1] = st.iter > 0 ? ms_alg / st.iter : 0.0f;
    r->times[2] = ms_tot;
    if (w.tstamp) put_timing(trec, r, st.iter);
  }
  if (st.status == GB_WATCHDOG) return bad("device iteration bound reached", GB_WATCHDOG);
  if (o.results_dir) {
    gb_options ow = o;
    ow.seed = seed;  // the seed of the drawn problem (kFixed may have advanced it)
    gb_result rw = *r;
    if (w.tstamp) {
      // the timing file lists every iteration's times (File_output_timings*)
      rw.time_per_iteration = trec.iter_ms.data();
      rw.time_supp_set = trec.supp_ms.data();
      rw.cg_per_iteration = trec.cg_steps.data();
      rw.time_for_cg = trec.cg_ms.data();
    }
    GB_TRY(gb_cs_write_result(o.results_dir, alg, kind, k, m, n, d, &ow, &rw, nullptr, 0));
  }
  return GB_OK;
}

// ------------------------------------------------------------------ results file
extern "C" gb_status gb_cs_write_result(const char *dir, const char *alg, int kind, int k, int m, int n, int d,
                                        const gb_options *o, const gb_result *r, char *path_out, int path_len) {
  if (!alg || !o || !r || kind < GB_OP_DENSE || kind > GB_OP_SMV) return bad("bad arguments to gb_cs_write_result");
  time_t raw;
  time(&raw);
  struct tm tmv;
  localtime_r(&raw, &tmv);
  const char *tag = kind == GB_OP_DENSE ? "gen" : kind == GB_OP_DCT ? "dct" : "smv";
  char fname[160];
  const int alg_id = gb_cs_alg_id(alg);
  if (o->timing && (alg_id == GB_ALG_NIHT || alg_id == GB_ALG_HTP)) {
    // results_timings* (GAGA/gaga/results.cu:1195-1210, 1365-1380, 1535-1550 and the HTP
    // forms 1705-1720, 1880-1895, 2050-2065): gpu_timings[_HTP]_data_<kind><date>.txt with the
    // File_output_timings* lines (functions.cu:82-208), one line per iteration after the summary
    const bool htp = alg_id == GB_ALG_HTP;
    if (r->iter > 0 && (!r->time_per_iteration || !r->time_supp_set || (htp && (!r->cg_per_iteration || !r->time_for_cg))))
      return bad("the timing results need the per-iteration time arrays");
    snprintf(fname, sizeof(fname), "gpu_timings_%sdata_%s%d%02d%02d.txt", htp ? "HTP_" : "", tag, tmv.tm_year + 1900,
             tmv.tm_mon + 1, tmv.tm_mday);
    std::string path = (dir && *dir) ? std::string(dir) + "/" + fname : std::string(fname);
    FILE *f = fopen(path.c_str(), "a+");
    if (!f) return bad("results file did not open");
    const float *e = r->norms, *t = r->times;
    const int *sc = r->support;
    fprintf(f, "%s_S_%s output: ", alg, tag);
    fprintf(f, "k %d, m %d, n %d, vecDistribution %d ", k, m, n, o->vec_distribution);
    fprintf(f, "errorl1 %0.7e errorl2 %0.7e errorlinf %0.7e ", e[0], e[1], e[2]);
    fprintf(f, "timeALG %0.7e timeIter %0.7e timeTotal %0.7e ", t[0], t[1], t[2]);
    fprintf(f, "iterations %d ", r->iter);
    fprintf(f, "converge_rate %0.7e ", r->conv_rate);
    fprintf(f, "TruePos %d FalsePos %d TrueNeg %d FalseNeg %d ", sc[0], sc[1], sc[2], sc[3]);
    fprintf(f, "seed %u ", o->seed);
    fprintf(f, "alpha %0.7e ", o->alpha);
    if (kind == GB_OP_DCT) {
      fprintf(f, "supp_flag %d \n", o->support_flag);
    } else if (kind == GB_OP_DENSE) {
      fprintf(f, "supp_flag %d ", o->support_flag);
      fprintf(f, "matrixEnsemble %d \n", o->matrix_ensemble == 2 ? 2 : 1);
    } else {
      fprintf(f, "supp_flag %d ", o->support_flag);
      fprintf(f, "NonzerosPerCol %d ", d);
      fprintf(f, "matrixEnsemble %d \n", o->matrix_ensemble ? o->matrix_ensemble : 3);
    }
    for (int j = 0; j < r->iter; ++j) {
      if (htp)
        fprintf(f, "iteration %d time_iteration %0.7e time_supp_set %0.7e cg_per_iteration %0.0f time_for_cg %0.7e\n", j,
                r->time_per_iteration[j], r->time_supp_set[j], r->cg_per_iteration[j], r->time_for_cg[j]);
      else
        fprintf(f, "iteration %d time_iteration %0.7e time_supp_set %0.7e\n", j, r->time_per_iteration[j],
                r->time_supp_set[j]);
    }
    fclose(f);
    if (path_out && path_len > 0) {
      strncpy(path_out, path.c_str(), (size_t)path_len - 1);
      path_out[path_len - 1] = 0;
    }
    return GB_OK;
  }
  if (o->noise > 0.0f)
    snprintf(fname, sizeof(fname), "gpu_data_%s%d%02d%02d_noise%0.3f.txt", tag, tmv.tm_year + 1900, tmv.tm_mon + 1,
             tmv.tm_mday, o->noise);
  else
    snprintf(fname, sizeof(fname), "gpu_data_%s%d%02d%02d.txt", tag, tmv.tm_year + 1900, tmv.tm_mon + 1,
             tmv.tm_mday);
  std::string path = (dir && *dir) ? std::string(dir) + "/" + fname : std::string(fname);
  FILE *f = fopen(path.c_str(), "a+");
  if (!f) return bad("results file did not open");
  const float *e = r->norms, *t = r->times;
  const int *s = r->support;
  if (kind == GB_OP_DENSE) {
    // File_output_gen (GAGA/gaga/functions.cu:64-74)
    const int ens = o->matrix_ensemble == 2 ? 2 : 1;
    fprintf(f, "%s_S_gen output: ", alg);
    fprintf(f, "k %d, m %d, n %d, vecDistribution %d matrixEnsemble %d ", k, m, n, o->vec_distribution, ens);
  } else if (kind == GB_OP_DCT) {
    // File_output (functions.cu:34-44)
    fprintf(f, "%s_S_dct output: ", alg);
    fprintf(f, "k %d, m %d, n %d, vecDistribution %d ", k, m, n, o->vec_distribution);
  } else {
    // File_output_smv (functions.cu:47-61)
    const int ens = o->matrix_ensemble ? o->matrix_ensemble : 3;
    fprintf(f, "%s_S_smv output: ", alg);
    fprintf(f, "k %d, m %d, n %d, vecDistribution %d nonzeros_per_column %d matrixEnsemble %d ", k, m, n,
            o->vec_distribution, d, ens);
  }
  fprintf(f, "errorl1 %0.7e errorl2 %0.7e errorlinf %0.7e ", e[0], e[1], e[2]);
  fprintf(f, "timeALG %0.7e timeIter %0.7e timeTotal %0.7e ", t[0], t[1], t[2]);
  fprintf(f, "iterations %d ", r->iter);
  fprintf(f, "converge_rate %0.7e ", r->conv_rate);
  fprintf(f, "TruePos %d FalsePos %d TrueNeg %d FalseNeg %d ", s[0], s[1], s[2], s[3]);
  if (kind == GB_OP_SMV) {
    fprintf(f, "seed %u ", o->seed);
    fprintf(f, "band_percentage %1.2f ", 0.0f);
    fprintf(f, "noise_level %2.4f ", o->noise);
    fprintf(f, "\n");
  } else {
    fprintf(f, "seed %u \n", o->seed);
  }
  fclose(f);
  if (path_out && path_len > 0) {
    strncpy(path_out, path.c_str(), (size_t)path_len - 1);
    path_out[path_len - 1] = 0;
  }
  return GB_OK;
}

// ------------------------------------------------------------------ component entry points
__global__ void k_hist_component(const float *__restrict__ v, int *__restrict__ bins, int *__restrict__ counters,
                                 int n, int max_bin, float slope, float intercept) {
  const float small_f = __double2float_rd((double)intercept * 0.000001);
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const float t = fabsf(v[i]);
    int b;
    if (t > small_f) {
      b = __float2int_rz(fmaxf(0.0f, __fmul_rn(slope, __fsub_rn(intercept, t))));
      if (b < max_bin) atomicAdd(&counters[b], 1);
    } else {
      b = __float2int_rz(__fmaf_rn(slope, intercept, 1.0f));
    }
    bins[i] = b;
  }
}

extern "C" gb_status gb_cs_linear_binning(const float *d_v, int n, int num_bins, int max_bin, float slope,
                                          float intercept, int *d_bins, int *d_counters, void *stream) {
  if (!d_v || !d_bins || !d_counters || n < 0 || num_bins < 1 || max_bin > num_bins) return bad("bad binning arguments");
  if (n == 0) return GB_OK;
  k_hist_component<<<std::min((n + 255) / 256, 2048), 256, 0, (cudaStream_t)stream>>>(d_v, d_bins, d_counters, n,
                                                                                      max_bin, slope, intercept);
  GB_CUDA_TRY(cudaGetLastError());
  return GB_OK;
}

__global__ void k_kbin_component(const int *__restrict__ counters, int max_bin, int k, int *out) {
  // serial scan exactly as the host loop of FindSupportSet (functions.cu:414-420)
  if (threadIdx.x || blockIdx.x) return;
  int k_bin = 0, sum = 0;
  while ((sum < k) & (k_bin < max_bin)) sum += counters[k_bin++];
  out[0] = k_bin - 1;
  out[1] = sum;
}

__global__ void k_threshold_component(float *v, const int *bins, int k_bin, int n) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    if (bins[i] > k_bin) v[i] = 0.0f;
}

extern "C" gb_status gb_cs_find_support_set(float *d_v, int n, int k, float slope, float intercept, float max_change,
                                            gb_bin_state *st, int *d_bins, int *d_counters, int threshold_v,
                                            void *stream) {
  if (!d_v || !d_bins || !st || n < 1 || st->num_bins < 1) return bad("bad FindSupportSet arguments");
  cudaStream_t s = (cudaStream_t)stream;
  if (st->min_val > max_change) {
    st->min_val = st->min_val - max_change;
  } else {
    DeviceBuffers db;
    int *cnt = d_counters, *out = nullptr;
    if (!cnt) GB_TRY(db.alloc(&cnt, st->num_bins, false));
    GB_TRY(db.alloc(&out, 2, false));
    GB_CUDA_TRY(cudaMemsetAsync(cnt, 0, sizeof(int) * st->num_bins, s));
    k_hist_component<<<std::min((n + 255) / 256, 2048), 256, 0, s>>>(d_v, d_bins, cnt, n, st->max_bin, slope,
                                                                     intercept);
    k_kbin_component<<<1, 32, 0, s>>>(cnt, st->max_bin, k, out);
    int h[2];
    GB_CUDA_TRY(cudaMemcpyAsync(h, out, sizeof(h), cudaMemcpyDeviceToHost, s));
    GB_CUDA_TRY(cudaStreamSynchronize(s));
    st->k_bin = h[0];
    st->sum = h[1];
    if (st->sum < k) {
      st->alpha = st->alpha * 0.5f;
      st->max_bin = (int)((float)st->num_bins * (1.0f - st->alpha));
    }
    st->min_val = intercept - (float)(st->k_bin + 1) / slope;
  }
  if (threshold_v) {
    k_threshold_component<<<std::min((n + 255) / 256, 2048), 256, 0, s>>>(d_v, d_bins, st->k_bin, n);
    GB_CUDA_TRY(cudaGetLastError());
  }
  return GB_OK;
}

// Device time of one operator application, set up once: each of `reps` applications is
// bracketed by CUDA events on the problem's stream (after `warmup` untimed ones); with a
// flush buffer, it is overwritten before each application so that every timed application
// reads its operands from HBM, not L2.  *ms_out: mean ms per application.  For the dense
// A x the support list of d_in is built once, outside the timed region.
extern "C" gb_status gb_cs_operator_time(const gb_problem *p, int transpose, const float *d_in, float *d_out,
                                         int warmup, int reps, void *d_flush, size_t flush_bytes, float *ms_out) {
  if (!p || !d_in || !d_out || !ms_out || reps < 1 || warmup < 0) return bad("bad gb_cs_operator_time arguments");
  if (p->location != GB_DEVICE) return bad("gb_cs_operator_time takes device buffers");
  GB_TRY(select_device(0));
  cudaStream_t s = (cudaStream_t)p->stream;
  DeviceBuffers db;
  GbWork w;
  memset(&w, 0, sizeof(w));
  if (transpose < 0 || transpose > 3 || (transpose >= 2 && p->kind != GB_OP_DENSE))
    return bad("gb_cs_operator_time: transpose 0, 1, or 2 / 3 (dense A^T r with the batched form's 24-bit / BF16 operand)");
  GB_TRY(setup_problem(db, w, *p, s, 1, 0, false));
  GbState st0;
  memset(&st0, 0, sizeof(st0));
  st0.active = 1;
  st0.flags[F_ALWAYS] = 1;
  st0.m = p->m;
  st0.n = p->n;
  st0.lda = w.op.lda;
  st0.gfmt = transpose == 2 ? GB_GRAD_A24 : transpose == 3 ? GB_GRAD_BF16 : GB_GRAD_FP32;
  GB_CUDA_TRY(cudaMemcpyAsync(w.st, &st0, sizeof(st0), cudaMemcpyHostToDevice, s));
  if (transpose >= 2) {
    // the batched form's compact A^T r operand, split from A once (outside the timing)
    if (w.op.lda % 8) return bad("gb_cs_operator_time: the compact operand needs lda % 8 == 0");
    unsigned short *hi = nullptr;
    GB_TRY(db.alloc(&hi, (size_t)w.op.lda * p->n, false));
    w.op.A_hi = hi;
    if (transpose == 2) {
      unsigned char *lo = nullptr;
      GB_TRY(db.alloc(&lo, (size_t)w.op.lda * p->n, false));
      w.op.A_lo = lo;
    }
    w.op.gfmt = transpose == 2 ? GB_GRAD_A24 : GB_GRAD_BF16;
    enq_split_a(w, s);
  }
  if (transpose) GB_CUDA_TRY(cudaMemcpyAsync(w.resid, d_in, sizeof(float) * p->m, cudaMemcpyDeviceToDevice, s));
  else if (w.op.kind == GB_OP_DENSE) enq_support_of_nonzeros(w, s, d_in, p->n);
  cudaEvent_t e0, e1;
  GB_CUDA_TRY(cudaEventCreate(&e0));
  GB_CUDA_TRY(cudaEventCreate(&e1));
  double total = 0.0;
  gb_status rc = GB_OK;
  for (int r = 0; r < warmup + reps && rc == GB_OK; ++r) {
    if (d_flush && flush_bytes) cudaMemsetAsync(d_flush, r & 0xff, flush_bytes, s);
    cudaEventRecord(e0, s);
    if (transpose) enq_AT(w, s, w.resid, d_out, F_ALWAYS);
    else enq_A(w, s, d_in, d_out, nullptr, -1, F_ALWAYS);
    cudaEventRecord(e1, s);
    cudaError_t e = cudaEventSynchronize(e1);
    if (e == cudaSuccess) e = cudaGetLastError();
    if (e != cudaSuccess) {
      gb_set_error_message(cudaGetErrorString(e), __FILE__, __LINE__);
      rc = GB_CUDA_ERROR;
      break;
    }
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, e0, e1);
    if (r >= warmup) total += ms;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (rc == GB_OK) *ms_out = (float)(total / reps);
  return rc;
}

extern "C" gb_status gb_cs_operator_apply(const gb_problem *p, int transpose, const float *d_in, float *d_out) {
  if (!p || !d_in || !d_out) return bad("null argument");
  if (p->location != GB_DEVICE) return bad("gb_cs_operator_apply takes device buffers");
  GB_TRY(select_device(0));
  cudaStream_t s = (cudaStream_t)p->stream;
  DeviceBuffers db;
  GbWork w;
  memset(&w, 0, sizeof(w));
  GB_TRY(setup_problem(db, w, *p, s, 1, 0, false));
  GbState st0;
  memset(&st0, 0, sizeof(st0));
  st0.active = 1;
  st0.flags[F_ALWAYS] = 1;
  GB_CUDA_TRY(cudaMemcpyAsync(w.st, &st0, sizeof(st0), cudaMemcpyHostToDevice, s));
  if (transpose) {
    // the operator reads its m-vector input from an lda-padded buffer
    GB_CUDA_TRY(cudaMemcpyAsync(w.resid, d_in, sizeof(float) * p->m, cudaMemcpyDeviceToDevice, s));
    enq_AT(w, s, w.resid, d_out, F_ALWAYS);
  } else {
    if (w.op.kind == GB_OP_DENSE) enq_support_of_nonzeros(w, s, d_in, p->n);
    enq_A(w, s, d_in, w.ru, nullptr, -1, F_ALWAYS);
    GB_CUDA_TRY(cudaMemcpyAsync(d_out, w.ru, sizeof(float) * p->m, cudaMemcpyDeviceToDevice, s));
  }
  GB_CUDA_TRY(cudaGetLastError());
  GB_CUDA_TRY(cudaStreamSynchronize(s));
  return GB_OK;
}

// l0 step on column-grouped rows: scores, then the residual scatter in column order
__global__ void k_l0_scores_component(const float *__restrict__ res, float *__restrict__ x, float *__restrict__ upd,
                                      const int *__restrict__ rows, int n, int d, int thresh, int shift,
                                      int *found) {
  const float EPS = 0.000001f;
  for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
    const size_t idx = (size_t)d * j;
    float score = 0.0f, u = 0.0f;
    const float omega = res[rows[idx + shift]];
    if (fabsf(omega) > EPS) {
      for (int i = 0; i < d; ++i) {
        const float ri = res[rows[idx + i]];
        if (fabsf(__fsub_rn(ri, omega)) <= EPS) score += 1.0f;
        if (fabsf(ri) <= EPS) score -= 1.0f;
      }
      if (score > (float)thresh) {
        *found = 1;
        x[j] = __fadd_rn(x[j], omega);
        u = omega;
      }
    }
    upd[j] = u;
  }
}

__global__ void k_l0_update_component(float *__restrict__ res, const int *__restrict__ ptr,
                                      const int *__restrict__ col, const float *__restrict__ upd, int m) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < m; i += gridDim.x * blockDim.x) {
    float r = res[i];
    for (int e = ptr[i]; e < ptr[i + 1]; ++e) {
      const float u = upd[col[e]];
      if (fabsf(u) > 0.0f) r = __fadd_rn(r, -u);
    }
    res[i] = r;
  }
}

extern "C" gb_status gb_cs_l0_step(float *d_res, float *d_x, float *d_updates, const int *d_rows, int m, int n, int d,
                                   int thresh, int shift, int *found, void *stream) {
  if (!d_res || !d_x || !d_updates || !d_rows || m < 1 || n < 1 || d < 1 || shift < 0 || shift >= d)
    return bad("bad l0 step arguments");
  cudaStream_t s = (cudaStream_t)stream;
  // CSR of the pattern (built on the host once per call)
  const size_t nz = (size_t)n * d;
  std::vector<int> rows(nz);
  GB_CUDA_TRY(cudaMemcpy(rows.data(), d_rows, sizeof(int) * nz, cudaMemcpyDeviceToHost));
  std::vector<int> ptr(m + 1, 0), col(nz);
  for (size_t e = 0; e < nz; ++e) {
    if (rows[e] < 0 || rows[e] >= m) return bad("row index out of range");
    ptr[rows[e] + 1]++;
  }
  for (int i = 0; i < m; ++i) ptr[i + 1] += ptr[i];
  std::vector<int> fill(ptr.begin(), ptr.end() - 1);
  for (size_t e = 0; e < nz; ++e) col[fill[rows[e]]++] = (int)(e / d);
  DeviceBuffers db;
  int *dptr, *dcol, *dfound;
  GB_TRY(db.alloc(&dptr, m + 1, false));
  GB_TRY(db.alloc(&dcol, nz, false));
  GB_TRY(db.alloc(&dfound, 1, true));
  GB_CUDA_TRY(cudaMemcpyAsync(dptr, ptr.data(), sizeof(int) * (m + 1), cudaMemcpyHostToDevice, s));
  GB_CUDA_TRY(cudaMemcpyAsync(dcol, col.data(), sizeof(int) * nz, cudaMemcpyHostToDevice, s));
  k_l0_scores_component<<<std::min((n + 255) / 256, 4096), 256, 0, s>>>(d_res, d_x, d_updates, d_rows, n, d, thresh,
                                                                         shift, dfound);
  k_l0_update_component<<<std::min((m + 255) / 256, 4096), 256, 0, s>>>(d_res, dptr, dcol, d_updates, m);
  int h = 0;
  GB_CUDA_TRY(cudaMemcpyAsync(&h, dfound, sizeof(int), cudaMemcpyDeviceToHost, s));
  GB_CUDA_TRY(cudaStreamSynchronize(s));
  if (found) *found = h;
  return GB_OK;
}
