// gb_batch.cu -- batched multi-trial form.
//
// The reference solves one trial per gaga_cs call: allocate, generate, run a host loop
// with ~20 launches and ~6 device->host round trips per iteration, free.  Here a batch
// of independent dense trials is served by B "slots".  Each slot owns a workspace sized
// for the largest trial of the batch and one CUDA graph, launched once on its own
// stream:
//
//     fetch a trial from a device-side queue
//     WHILE (a trial was fetched)
//         draw A, x0 on the device from (seed + trial id); y = A x0
//         the solver's prologue, then WHILE (stopping rules) { one iteration }
//         write the trial's iterations / relative error / verdict; fetch the next trial
//
// The solver kernels are the plain path's (gb_ops.cu, gb_solver.cu) reading the current
// trial's m, n, k from the slot's device state, so one captured graph serves trials of
// every size.  Large trials run their kernels over the whole GPU; small ones overlap
// across slots.  No host work, allocation or graph build happens per trial.
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <map>
#include <mutex>
#include <vector>

#include "gb_ctrl.cuh"
#include "gb_internal.cuh"
#include "gb_philox.cuh"
#include "gb_resident.h"

__global__ void k_hist(const GbState *st, int pf, const float *__restrict__ v, int *__restrict__ bins,
                       int *__restrict__ bins_prev, int *__restrict__ counters, int n);
__global__ void k_kbin(GbState *st, int pf, const int *__restrict__ counters, int k);
__global__ void k_thresh_count(GbState *st, int pf, float *__restrict__ v, const int *__restrict__ bins,
                               const int *__restrict__ bins_prev, int n, int *__restrict__ tile_cnt);
__global__ void k_compact(GbState *st, int pf, const int *__restrict__ bins, int n, const int *__restrict__ tile_cnt,
                          int *__restrict__ S, unsigned *__restrict__ bm);

namespace {

struct BatchParams {
  int T;
  unsigned int seed;
  float tol_rel;
  int maxiter, alg;
  const int *n, *m, *k;
  const unsigned int *tid;
  const int *order;
  int *queue;
  int *iters;
  float *err;
  int *ok;
  double *bytes;
  int learned;  // learned warm start (CGIHT)
  int *fb;      // per trial: the warm start was abandoned (solve again from zero)
  int gfmt;     // the A^T r operand (GB_GRAD_*)
  const unsigned char *gfmts;  // per trial, or null: gfmt for every trial
  int rec_every;  // CGIHT residual recurrence (GbState::rec_every)
};

using gbgen::KEY_HI;
enum { ST_MATRIX = gbgen::ST_MATRIX, ST_VALUES = gbgen::ST_VALUES, ST_SUPPORT = gbgen::ST_SUPPORT };
__device__ __forceinline__ void philox_d(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3, uint32_t k0,
                                         uint32_t k1, uint32_t out[4]) {
  gbgen::philox(c0, c1, c2, c3, k0, k1, out);
}
__device__ __forceinline__ float u01d(uint32_t x) { return gbgen::u01(x); }

__device__ __forceinline__ uint32_t trial_key(const BatchParams *bp, const GbState *st) {
  return bp->seed + (bp->tid ? bp->tid[st->trial] : (uint32_t)st->trial);
}

// set the slot's state for trial q of the queue order, or end the slot's trial loop
__device__ void load_trial(GbState *st, const BatchParams *bp, int q, cudaGraphConditionalHandle h_trial) {
  if (q >= bp->T) {
    st->active = 0;
    st->trial = -1;
    cudaGraphSetConditional(h_trial, 0u);
    return;
  }
  const int t = bp->order[q];
  batch_trial_fields(st, t, bp->m[t], bp->n[t], bp->k[t], bp->maxiter, bp->alg);
  st->gfmt = bp->gfmts ? bp->gfmts[t] : bp->gfmt;
  st->rec_every = bp->rec_every;
  cudaGraphSetConditional(h_trial, 1u);
}

__global__ void k_b_fetch(GbState *st, const BatchParams *bp, cudaGraphConditionalHandle h_trial) {
  if (threadIdx.x || blockIdx.x) return;
  load_trial(st, bp, atomicAdd(bp->queue, 1), h_trial);
}

// A of the current trial: the element stream of k_gen_dense (gb_api.cu) keyed by seed + trial id
// A, and with the trial's compact A^T r operand (st->gfmt A24 / BF16) its high parts (and low
// bytes) rounded from the drawn values as they are written (rows m..lda-1 of the copy zero)
__global__ void k_b_gen_A(const GbState *st, const BatchParams *bp, float *A, unsigned short *hi, unsigned char *lo) {
  if (!st->active) return;
  const int m = st->m, n = st->n, lda = st->lda;
  const uint32_t key = trial_key(bp, st);
  const int lane = threadIdx.x & 31;
  const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, nw = (gridDim.x * blockDim.x) >> 5;
  const int gfmt = hi ? st->gfmt : GB_GRAD_FP32;
  if (gfmt == GB_GRAD_FP32) {
    for (int j = gw; j < n; j += nw) gbgen::gen_dense_column(A + (size_t)j * lda, j, m, key, 0u, 1, lane, 32);
    return;
  }
  const bool has_lo = gfmt == GB_GRAD_A24;
  for (int j = gw; j < n; j += nw) {
    const size_t c = (size_t)j * lda;
    unsigned short *h = hi + c;
    unsigned char *l = has_lo ? lo + c : nullptr;
    gbgen::gen_dense_column_emit(A + c, j, m, key, 0u, 1, lane, 32, [&](int i, float a) {
      const uint32_t b = round_top_bits(__float_as_uint(a), has_lo ? 8 : 16);
      h[i] = (unsigned short)(b >> 16);
      if (has_lo) l[i] = (unsigned char)(b >> 8);
    });
    for (int i = m + lane; i < lda; i += 32) {
      h[i] = 0;
      if (has_lo) l[i] = 0;
    }
  }
}

// x0 values (+-1) and support keys of createVector (GAGA/gaga/createVector.cu:207-300);
// max key into red[R_XMAX]; clears the n-bin key histogram
__global__ void k_b_gen_x(GbState *st, const BatchParams *bp, float *vals, float *keys, int *hist, float *rp,
                          unsigned int *tk) {
  if (!st->active) return;
  const int n = st->n;
  const uint32_t key = trial_key(bp, st);
  float mx = 0.0f;
  for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
    uint32_t o[4];
    philox_d((uint32_t)(j >> 2), 0u, ST_VALUES, 0u, key, KEY_HI, o);
    vals[j] = signbit(u01d(o[j & 3]) - 0.5f) ? -1.0f : 1.0f;
    philox_d((uint32_t)(j >> 2), 0u, ST_SUPPORT, 0u, key, KEY_HI, o);
    const float u = u01d(o[j & 3]);
    keys[j] = u;
    mx = fmaxf(mx, u);
    hist[j] = 0;
  }
  grid_reduce_publish<1>(mx, R_XMAX, st, rp, tk);
}

// generation bookkeeping (single thread)
enum { B_KEYS = 0, B_X0 = 1, B_INIT = 2, B_RESULT = 3 };
__global__ void k_b_ctrl(GbState *st, const BatchParams *bp, int phase, cudaGraphConditionalHandle h_trial) {
  if (threadIdx.x || blockIdx.x) return;
  if (phase == B_KEYS) {
    if (!st->active) return;
    // n linear bins over the keys, every key counted (createVector.cu:236-248)
    st->max_value = (float)st->red[R_XMAX];
    st->slope = ((float)(st->n - 1) / st->max_value);
    st->max_bin = st->n;
    st->alpha_bin = 0.25f;
    st->flags[F_DOBIN] = 1;
  } else if (phase == B_X0) {
    if (!st->active) return;
    st->k = st->sum;  // |support| >= k, the k the solver is given
  } else if (phase == B_INIT) {
    if (!st->active) return;
    batch_solver_init(st, bp->tol_rel, bp->learned);
  } else {
    // verdict of the finished trial (results.cu:468-475), then the next trial
    if (st->trial >= 0) {
      const int t = st->trial;
      const float rel = (float)(sqrt(st->red[R_DOT1]) / sqrt(st->red[R_DOT2]));
      bp->iters[t] = st->iter;
      bp->err[t] = rel;
      bp->ok[t] = rel <= 1e-3f ? 1 : 0;
      if (bp->fb) bp->fb[t] = st->fell_back;
      atomicAdd(bp->bytes, st->bytes);
    }
    load_trial(st, bp, atomicAdd(bp->queue, 1), h_trial);
  }
}

// ||x - x0||^2 and ||x0||^2
__global__ void k_b_err(GbState *st, const float *__restrict__ x, const float *__restrict__ x0, float *rp,
                        unsigned int *tk) {
  if (st->trial < 0) return;
  const int n = st->n;
  float e2 = 0.0f, x2 = 0.0f;
  for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
    const float d = x0[j] - x[j];
    e2 = fmaf(d, d, e2);
    x2 = fmaf(x0[j], x0[j], x2);
  }
  grid_reduce_publish<0>(e2, R_DOT1, st, rp, tk);
  grid_reduce_publish<0>(x2, R_DOT2, st, rp, tk);
}

struct Slot {
  GbWork w;
  std::vector<void *> bufs;
  float *x0 = nullptr;
  int *hist = nullptr;
  cudaStream_t stream = nullptr;
  cudaGraphExec_t exec = nullptr;
};

struct Engine {
  int dev = -1, alg = -1, n_cap = 0, m_cap = 0, t_cap = 0, slots = 0, learned = 0, sm_share = 0, gfmt = 0,
      av_rows = 0;
  float *ml_params = nullptr;  // the warm-start MLP parameters (copied in by every call)
  int *dfb = nullptr;
  unsigned char *dgfmt = nullptr;  // per-trial A^T r operand formats
  std::vector<Slot> slot;
  char *table = nullptr;
  BatchParams *d_params = nullptr;
  int *dn = nullptr, *dm = nullptr, *dk = nullptr, *dorder = nullptr, *dqueue = nullptr, *diters = nullptr,
      *dok = nullptr;
  unsigned *dtid = nullptr;
  float *derr = nullptr;
  double *dbytes = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  std::vector<cudaEvent_t> done;
};
std::map<int, Engine> g_engines;  // key: device * 2 + learned

gb_status dalloc(std::vector<void *> &bufs, void **p, size_t bytes) {
  GB_CUDA_TRY(cudaMalloc(p, std::max<size_t>(bytes, 4)));
  bufs.push_back(*p);
  GB_CUDA_TRY(cudaMemset(*p, 0, std::max<size_t>(bytes, 4)));
  return GB_OK;
}

void release(Engine &E) {
  for (auto &s : E.slot) {
    if (s.exec) cudaGraphExecDestroy(s.exec);
    for (void *p : s.bufs) cudaFree(p);
    if (s.stream) cudaStreamDestroy(s.stream);
  }
  for (auto e : E.done) cudaEventDestroy(e);
  if (E.table) cudaFree(E.table);
  if (E.e0) cudaEventDestroy(E.e0);
  if (E.e1) cudaEventDestroy(E.e1);
  E = Engine();
}

gb_status build_slot_graph(Engine &E, Slot &S) {
  GbWork &w = S.w;
  cudaStream_t s0, s1, s2, s3;
  GB_CUDA_TRY(cudaStreamCreateWithFlags(&s0, cudaStreamNonBlocking));
  GB_CUDA_TRY(cudaStreamCreateWithFlags(&s1, cudaStreamNonBlocking));
  GB_CUDA_TRY(cudaStreamCreateWithFlags(&s2, cudaStreamNonBlocking));
  GB_CUDA_TRY(cudaStreamCreateWithFlags(&s3, cudaStreamNonBlocking));
  SolvePlan P{&w, E.alg, 0, 0};
  cudaGraph_t graph;
  GB_CUDA_TRY(cudaStreamBeginCapture(s0, cudaStreamCaptureModeThreadLocal));
  cudaGraphConditionalHandle h_trial = 0, h_iter = 0, h_cg = 0;
  GB_TRY(gb_make_handle(s0, &h_trial));
  k_b_fetch<<<1, 32, 0, s0>>>(w.st, E.d_params, h_trial);
  GB_TRY(gb_open_while(s0, s1, h_trial));
  {
    // ---- draw the trial on the device
    k_b_gen_A<<<w.num_sms * 8, 256, 0, s1>>>(w.st, E.d_params, const_cast<float *>(w.op.A),
                                             const_cast<unsigned short *>(w.op.A_hi),
                                             const_cast<unsigned char *>(w.op.A_lo));
    k_b_gen_x<<<w.red_blocks, 256, 0, s1>>>(w.st, E.d_params, S.x0, w.xt, S.hist, w.red_part, w.tickets);
    k_b_ctrl<<<1, 32, 0, s1>>>(w.st, E.d_params, B_KEYS, 0);
    // support of x0: keys in n linear bins, the top bins holding >= k keys
    k_hist<<<w.red_blocks, 256, 0, s1>>>(w.st, F_ALWAYS, w.xt, w.bins, nullptr, S.hist, D_N);
    k_kbin<<<1, 1024, 0, s1>>>(w.st, F_ALWAYS, S.hist, D_K);
    k_b_ctrl<<<1, 32, 0, s1>>>(w.st, E.d_params, B_X0, 0);
    const int tiles = (w.op.n + GB_TILE - 1) / GB_TILE;
    k_thresh_count<<<tiles, 256, 0, s1>>>(w.st, F_ALWAYS, S.x0, w.bins, nullptr, D_N, w.tile_cnt);
    k_compact<<<tiles, 256, 0, s1>>>(w.st, F_DOBIN, w.bins, D_N, w.tile_cnt, w.S, nullptr);
    // y = A x0 and ||y||
    enq_A(w, s1, S.x0, w.y, nullptr, R_RES, F_ALWAYS);
    k_b_ctrl<<<1, 32, 0, s1>>>(w.st, E.d_params, B_INIT, 0);
    // ---- solve
    GB_TRY(gb_make_handle(s1, &h_iter));
    enq_prologue(P, s1, h_iter);
    GB_TRY(gb_open_while(s1, s2, h_iter));
    enq_body(P, s2, h_iter);
    if (E.alg == GB_ALG_HTP) {
      GB_TRY(gb_make_handle(s2, &h_cg));
      enq_ctrl_phase(w, s2, GB_PHASE_HTP_CGINIT, h_cg);
      GB_TRY(gb_open_while(s2, s3, h_cg));
      enq_cg_body(P, s3, h_cg);
      GB_TRY(gb_close_while(s3));
      enq_ctrl_phase(w, s2, GB_PHASE_HTP_STOP, h_iter);
    }
    GB_TRY(gb_close_while(s2));
    // ---- verdict, next trial
    k_b_err<<<w.red_blocks, 256, 0, s1>>>(w.st, w.x, S.x0, w.red_part, w.tickets);
    k_b_ctrl<<<1, 32, 0, s1>>>(w.st, E.d_params, B_RESULT, h_trial);
  }
  GB_TRY(gb_close_while(s1));
  GB_CUDA_TRY(cudaStreamEndCapture(s0, &graph));
  cudaError_t e = cudaGraphInstantiate(&S.exec, graph, 0);
  cudaGraphDestroy(graph);
  cudaStreamDestroy(s0);
  cudaStreamDestroy(s1);
  cudaStreamDestroy(s2);
  cudaStreamDestroy(s3);
  GB_CUDA_TRY(e);
  return GB_OK;
}

gb_status setup_engine(Engine &E, int dev, int alg, int n_cap, int m_cap, int T, int slots, int learned,
                       int sm_share, int gfmt, int av_rows) {
  if (E.dev == dev && E.alg == alg && E.n_cap >= n_cap && E.m_cap >= m_cap && E.t_cap >= T && E.slots == slots &&
      E.learned == learned && E.sm_share == sm_share && E.gfmt == gfmt && E.av_rows == av_rows)
    return GB_OK;
  release(E);
  E.gfmt = gfmt;
  E.av_rows = av_rows;
  E.learned = learned;
  E.sm_share = sm_share;
  E.dev = dev;
  E.alg = alg;
  E.n_cap = n_cap;
  E.m_cap = m_cap;
  E.t_cap = std::max(T, 1024);
  E.slots = slots;
  const size_t tb = (size_t)E.t_cap * 4;
  const size_t bytes = 12 * (tb + 256) + sizeof(BatchParams) + 2048 + (size_t)gb_ml_num_params() * 4 + 256;
  GB_CUDA_TRY(cudaMalloc(&E.table, bytes));
  GB_CUDA_TRY(cudaMemset(E.table, 0, bytes));
  char *p = E.table;
  auto take = [&](size_t b) {
    char *q = p;
    p += (b + 255) & ~(size_t)255;
    return q;
  };
  E.dn = (int *)take(tb); E.dm = (int *)take(tb); E.dk = (int *)take(tb); E.dtid = (unsigned *)take(tb);
  E.dorder = (int *)take(tb); E.diters = (int *)take(tb); E.derr = (float *)take(tb); E.dok = (int *)take(tb);
  E.dqueue = (int *)take(256); E.dbytes = (double *)take(256);
  E.dfb = (int *)take(tb);
  E.dgfmt = (unsigned char *)take((size_t)E.t_cap);
  E.ml_params = (float *)take((size_t)gb_ml_num_params() * 4);
  E.d_params = (BatchParams *)take(sizeof(BatchParams));
  int sms = 0;
  GB_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  const int lda = (m_cap + 31) / 32 * 32;
  E.slot.resize(slots);
  for (int i = 0; i < slots; ++i) {
    Slot &S = E.slot[i];
    GbWork &w = S.w;
    memset(&w, 0, sizeof(w));
    w.dyn = 1;
    w.num_sms = sms;
    // slots run concurrently: each slot's kernels are shaped for sm_share SMs
    w.red_blocks = std::max(1, std::min(GB_MAXRB, sm_share));
    w.wide_blocks = sm_share * 4;
    GbOp &op = w.op;
    op.kind = GB_OP_DENSE;
    op.m = m_cap;
    op.n = n_cap;
    op.lda = lda;
    op.vec4 = 1;
    auto A = [&](void **q, size_t b) { return dalloc(S.bufs, q, b); };
    float *Abuf = nullptr;
    GB_TRY(A((void **)&Abuf, (size_t)lda * n_cap * 4));
    op.A = Abuf;
    op.gfmt = gfmt;
    if (gfmt != GB_GRAD_FP32) {
      unsigned short *hi = nullptr;
      GB_TRY(A((void **)&hi, (size_t)lda * n_cap * 2));
      op.A_hi = hi;
      if (gfmt == GB_GRAD_A24) {
        unsigned char *lo = nullptr;
        GB_TRY(A((void **)&lo, (size_t)lda * n_cap));
        op.A_lo = lo;
      }
    }
    GB_TRY(A((void **)&w.st, sizeof(GbState)));
    GB_TRY(A((void **)&w.red_part, (size_t)GB_NSLOT * GB_MAXRB * 4));
    GB_TRY(A((void **)&w.tickets, GB_NSLOT * 4));
    for (float **v : {&w.x, &w.xt, &w.grad, &w.gp, &w.gpt, &w.upd, &S.x0}) GB_TRY(A((void **)v, (size_t)n_cap * 4));
    for (float **v : {&w.y, &w.resid, &w.ru}) GB_TRY(A((void **)v, (size_t)lda * 4));
    for (int **v : {&w.bins, &w.bins_prev, &w.S, &S.hist}) GB_TRY(A((void **)v, (size_t)n_cap * 4));
    GB_TRY(A((void **)&w.counters, (size_t)std::max(n_cap / 20, 1000) * 4));
    GB_TRY(A((void **)&w.tile_cnt, (size_t)((n_cap + GB_TILE - 1) / GB_TILE) * 4));
    gb_dense_av_shape(m_cap, sm_share, true, &w.av_ntile, &w.av_nsplit, &w.av_rows, av_rows);
    w.part_cap = gb_dense_part_floats_av(w.av_ntile, w.av_nsplit, w.av_rows);
    GB_TRY(A((void **)&w.part, 2 * w.part_cap * 4));
    w.part_two = 1;
    GB_TRY(A((void **)&w.av_tickets, (size_t)w.av_ntile * 4));
    if (learned) {
      w.ml_params = E.ml_params;
      GB_TRY(A((void **)&w.ml_counts, (size_t)gb_ml_rank_bins() * 4));
      GB_TRY(A((void **)&w.ml_cum, (size_t)gb_ml_rank_bins() * 4));
    }
    GbState st0;
    memset(&st0, 0, sizeof(st0));
    st0.lda = lda;
    st0.trial = -1;
    GB_CUDA_TRY(cudaMemcpy(w.st, &st0, sizeof(st0), cudaMemcpyHostToDevice));
    GB_CUDA_TRY(cudaStreamCreateWithFlags(&S.stream, cudaStreamNonBlocking));
    cudaEvent_t ev;
    GB_CUDA_TRY(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
    E.done.push_back(ev);
  }
  for (auto &S : E.slot) GB_TRY(build_slot_graph(E, S));
  GB_CUDA_TRY(cudaEventCreate(&E.e0));
  GB_CUDA_TRY(cudaEventCreate(&E.e1));
  return GB_OK;
}

// Number of slots: the requested count (default 16: enough concurrency for small trials),
// within 60% of free memory.
int slots_for(int n_cap, int m_cap, size_t free_bytes, int T, int requested, int gfmt) {
  int s = requested > 0 ? requested : 16;
  if (const char *e = getenv("GB_CS_BATCH_SLOTS")) s = std::max(1, atoi(e));
  const double eb = 4.0 + (gfmt == GB_GRAD_A24 ? 3.0 : gfmt == GB_GRAD_BF16 ? 2.0 : 0.0);  // bytes per entry of A
  const double per = (double)((m_cap + 31) / 32 * 32) * n_cap * eb * 1.05 + 64.0 * n_cap + (1 << 24);
  while (s > 1 && s * per > 0.6 * (double)free_bytes) s--;
  return std::max(1, std::min(s, T));
}

}  // namespace

static thread_local double g_last_bytes = 0.0;
static thread_local float g_last_kernel_ms = 0.0f;

// The engines (slot graphs, resident buffers) are per device and shared by every caller, so
// calls from several host threads run one at a time; recursive because the learned warm
// start's fallback pass calls back in.
std::recursive_mutex &gb_batch_mutex() {
  static std::recursive_mutex mu;
  return mu;
}

extern "C" gb_status gb_cs_solve_batch(const gb_batch *b, int *iters_out, float *rel_err_out, int *success_out,
                                       int *num_success) {
  if (!b || b->ntrials < 0 || (b->ntrials > 0 && (!b->n || !b->m || !b->k))) {
    gb_set_error_message("bad batch arguments", __FILE__, __LINE__);
    return GB_BAD_ARG;
  }
  if (b->alg != GB_ALG_NIHT && b->alg != GB_ALG_CGIHT && b->alg != GB_ALG_HTP) {
    gb_set_error_message("batched form supports NIHT, HTP and CGIHT", __FILE__, __LINE__);
    return GB_BAD_ARG;
  }
  if (b->use_learned && (b->alg != GB_ALG_CGIHT || !b->learned_params)) {
    gb_set_error_message("use_learned needs CGIHT and learned_params", __FILE__, __LINE__);
    return GB_BAD_ARG;
  }
  if (b->maxiter < 0) {
    gb_set_error_message("maxiter must be >= 0", __FILE__, __LINE__);
    return GB_BAD_ARG;
  }
  if (b->av_rows != 0 && b->av_rows != 128 && b->av_rows != 256) {
    gb_set_error_message("av_rows: 0, 128 or 256", __FILE__, __LINE__);
    return GB_BAD_ARG;
  }
  if (b->grad_format < GB_GRAD_FP32 || b->grad_format > GB_GRAD_BF16 ||
      (b->grad_format != GB_GRAD_FP32 && b->alg == GB_ALG_HTP)) {
    gb_set_error_message("grad_format: 0, 1 or 2, and FP32 for HTP (its CG projection needs A^T A)", __FILE__,
                         __LINE__);
    return GB_BAD_ARG;
  }
  // the operand format of the engines' buffers: per-trial formats are A24 or BF16 (A24's
  // buffers hold both)
  int gfmt = b->grad_format;
  if (b->grad_formats && b->ntrials > 0) {
    if (b->alg == GB_ALG_HTP) {
      gb_set_error_message("grad_formats: HTP keeps FP32", __FILE__, __LINE__);
      return GB_BAD_ARG;
    }
    gfmt = GB_GRAD_BF16;
    for (int t = 0; t < b->ntrials; ++t) {
      const int f = b->grad_formats[t];
      if (f != GB_GRAD_A24 && f != GB_GRAD_BF16) {
        gb_set_error_message("grad_formats: every entry GB_GRAD_A24 or GB_GRAD_BF16", __FILE__, __LINE__);
        return GB_BAD_ARG;
      }
      if (f == GB_GRAD_A24) gfmt = GB_GRAD_A24;
    }
  }
  std::lock_guard<std::recursive_mutex> lock(gb_batch_mutex());
  const int T = b->ntrials;
  int n_cap = 16, m_cap = 1;
  for (int t = 0; t < T; ++t) {
    if (b->n[t] < 16 || b->m[t] < 1 || b->k[t] < 1 || b->m[t] > b->n[t] || b->n[t] > (1 << 22)) {
      gb_set_error_message("trial sizes must satisfy 1 <= k, 1 <= m <= n, 16 <= n <= 2^22", __FILE__, __LINE__);
      return GB_BAD_ARG;
    }
  }
  // NIHT trials with n <= resident_n go to the cluster-resident kernel (gb_resident.cu),
  // the others to the slot graphs; both run at the same time
  int rn = b->resident_n;
  if (rn == 0) {
    rn = GB_RESIDENT_N_DEFAULT;
    if (const char *e = getenv("GB_CS_RESIDENT_N")) rn = atoi(e);
  }
  if (b->alg != GB_ALG_NIHT && b->alg != GB_ALG_CGIHT && b->alg != GB_ALG_HTP) rn = -1;
  std::vector<char> resident(T, 0);
  int rn_cap = 16, rm_cap = 1, n_res = 0;
  for (int t = 0; t < T; ++t)
    if (rn > 0 && b->n[t] <= rn) {
      resident[t] = 1;
      rn_cap = std::max(rn_cap, b->n[t]);
      rm_cap = std::max(rm_cap, b->m[t]);
      n_res++;
    }
  if (n_res > 0 && gb_resident_pick_cluster(rn_cap, rm_cap, b->cluster, b->alg, b->use_learned ? 1 : 0) <= 0) {
    if (b->cluster > 0 || b->resident_n > 0) {
      gb_set_error_message("resident form: the requested cluster size does not fit these trials", __FILE__,
                           __LINE__);
      return GB_BAD_ARG;
    }
    std::fill(resident.begin(), resident.end(), 0);
    n_res = 0;
  }
  for (int t = 0; t < T; ++t)
    if (!resident[t]) {
      n_cap = std::max(n_cap, b->n[t]);
      m_cap = std::max(m_cap, b->m[t]);
    }
  if (num_success) *num_success = 0;
  if (T == 0) return GB_OK;
  int dev = 0;
  GB_CUDA_TRY(cudaGetDevice(&dev));
  const int learned = b->use_learned ? 1 : 0;
  Engine &E = g_engines[dev * 2 + learned];
  int sms = 0;
  GB_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  const int sm_share = b->sm_share > 0 ? std::min(b->sm_share, sms) : std::max(1, sms / 2);
  const bool reuse = E.dev == dev && E.alg == b->alg && E.n_cap >= n_cap && E.m_cap >= m_cap && E.t_cap >= T &&
                     E.sm_share == sm_share && (b->slots <= 0 || E.slots == b->slots) && E.gfmt == gfmt &&
                     E.av_rows == b->av_rows;
  if (!reuse) {
    release(E);
    size_t free_b = 0, total_b = 0;
    GB_CUDA_TRY(cudaMemGetInfo(&free_b, &total_b));
    GB_TRY(setup_engine(E, dev, b->alg, n_cap, m_cap, T,
                        slots_for(n_cap, m_cap, free_b, std::max(T, 16), b->slots, gfmt), learned, sm_share,
                        gfmt, b->av_rows));
  }
  cudaStream_t s = (cudaStream_t)b->stream;
  // trial table, longest (m*n) first
  std::vector<int> order, rorder;
  for (int t = 0; t < T; ++t) (resident[t] ? rorder : order).push_back(t);
  auto larger = [&](int x, int y) { return (double)b->m[x] * b->n[x] > (double)b->m[y] * b->n[y]; };
  std::stable_sort(order.begin(), order.end(), larger);
  std::stable_sort(rorder.begin(), rorder.end(), larger);
  const int T_slot = (int)order.size();
  std::vector<unsigned> tid(T);
  for (int t = 0; t < T; ++t) tid[t] = b->trial_id ? b->trial_id[t] : (unsigned)t;
  BatchParams bp;
  bp.T = T_slot; bp.seed = b->seed; bp.tol_rel = b->tol_rel; bp.maxiter = b->maxiter; bp.alg = b->alg;
  bp.n = E.dn; bp.m = E.dm; bp.k = E.dk; bp.tid = E.dtid; bp.order = E.dorder; bp.queue = E.dqueue;
  bp.iters = E.diters; bp.err = E.derr; bp.ok = E.dok; bp.bytes = E.dbytes;
  bp.learned = learned;
  bp.fb = learned ? E.dfb : nullptr;
  bp.gfmt = gfmt;
  bp.gfmts = b->grad_formats ? E.dgfmt : nullptr;
  if (b->grad_formats)
    GB_CUDA_TRY(cudaMemcpyAsync(E.dgfmt, b->grad_formats, (size_t)T, cudaMemcpyHostToDevice, s));
  bp.rec_every = b->alg == GB_ALG_CGIHT ? std::max(0, b->residual_refresh) : 0;
  if (learned)
    GB_CUDA_TRY(cudaMemcpyAsync(E.ml_params, b->learned_params, sizeof(float) * gb_ml_num_params(),
                                cudaMemcpyDeviceToDevice, s));
  GB_CUDA_TRY(cudaMemcpyAsync(E.dn, b->n, (size_t)T * 4, cudaMemcpyHostToDevice, s));
  GB_CUDA_TRY(cudaMemcpyAsync(E.dm, b->m, (size_t)T * 4, cudaMemcpyHostToDevice, s));
  GB_CUDA_TRY(cudaMemcpyAsync(E.dk, b->k, (size_t)T * 4, cudaMemcpyHostToDevice, s));
  GB_CUDA_TRY(cudaMemcpyAsync(E.dtid, tid.data(), (size_t)T * 4, cudaMemcpyHostToDevice, s));
  if (T_slot > 0)
    GB_CUDA_TRY(cudaMemcpyAsync(E.dorder, order.data(), (size_t)T_slot * 4, cudaMemcpyHostToDevice, s));
  GB_CUDA_TRY(cudaMemcpyAsync(E.d_params, &bp, sizeof(bp), cudaMemcpyHostToDevice, s));
  GB_CUDA_TRY(cudaMemsetAsync(E.dqueue, 0, 4, s));
  GB_CUDA_TRY(cudaMemsetAsync(E.dbytes, 0, 8, s));
  GB_CUDA_TRY(cudaEventRecord(E.e0, s));
  const size_t nslot = T_slot > 0 ? E.slot.size() : 0;
  for (size_t i = 0; i < nslot; ++i) {
    Slot &S = E.slot[i];
    GB_CUDA_TRY(cudaStreamWaitEvent(S.stream, E.e0, 0));
    GB_CUDA_TRY(cudaGraphLaunch(S.exec, S.stream));
    GB_CUDA_TRY(cudaEventRecord(E.done[i], S.stream));
  }
  if (n_res > 0) {
    GbResidentArgs ra;
    ra.count = n_res;
    ra.order = rorder.data();
    ra.n = E.dn; ra.m = E.dm; ra.k = E.dk; ra.tid = E.dtid;
    ra.seed = b->seed; ra.tol_rel = b->tol_rel; ra.maxiter = b->maxiter;
    ra.iters = E.diters; ra.err = E.derr; ra.ok = E.dok; ra.bytes = E.dbytes;
    ra.n_cap = rn_cap; ra.m_cap = rm_cap; ra.cluster = b->cluster; ra.alg = b->alg;
    ra.ml_params = learned ? E.ml_params : nullptr;
    ra.fb = learned ? E.dfb : nullptr;
    ra.gfmt = gfmt;
    ra.gfmts = bp.gfmts;
    ra.rec_every = bp.rec_every;
    GB_TRY(gb_resident_enqueue(ra, s));
  }
  for (size_t i = 0; i < nslot; ++i) GB_CUDA_TRY(cudaStreamWaitEvent(s, E.done[i], 0));
  GB_CUDA_TRY(cudaEventRecord(E.e1, s));
  std::vector<int> hit(T), hok(T), hfb(T, 0);
  std::vector<float> herr(T);
  double hbytes = 0.0;
  if (learned) GB_CUDA_TRY(cudaMemcpyAsync(hfb.data(), E.dfb, (size_t)T * 4, cudaMemcpyDeviceToHost, s));
  GB_CUDA_TRY(cudaMemcpyAsync(hit.data(), E.diters, (size_t)T * 4, cudaMemcpyDeviceToHost, s));
  GB_CUDA_TRY(cudaMemcpyAsync(herr.data(), E.derr, (size_t)T * 4, cudaMemcpyDeviceToHost, s));
  GB_CUDA_TRY(cudaMemcpyAsync(hok.data(), E.dok, (size_t)T * 4, cudaMemcpyDeviceToHost, s));
  GB_CUDA_TRY(cudaMemcpyAsync(&hbytes, E.dbytes, 8, cudaMemcpyDeviceToHost, s));
  GB_CUDA_TRY(cudaStreamSynchronize(s));
  if (n_res > 0) GB_TRY(gb_resident_check());
  cudaEventElapsedTime(&g_last_kernel_ms, E.e0, E.e1);
  g_last_bytes = hbytes;
  if (learned) {
    // trials whose warm start was abandoned: plain zero-initialised CGIHT decides
    std::vector<int> sn, sm, sk, idx;
    std::vector<unsigned> stid;
    std::vector<unsigned char> sfmt;
    for (int t = 0; t < T; ++t)
      if (hfb[t]) {
        idx.push_back(t);
        sn.push_back(b->n[t]);
        sm.push_back(b->m[t]);
        sk.push_back(b->k[t]);
        stid.push_back(tid[t]);
        if (b->grad_formats) sfmt.push_back(b->grad_formats[t]);
      }
    if (!idx.empty()) {
      const float ms1 = g_last_kernel_ms;
      const double by1 = g_last_bytes;
      gb_batch pb = *b;
      pb.ntrials = (int)idx.size();
      pb.n = sn.data();
      pb.m = sm.data();
      pb.k = sk.data();
      pb.trial_id = stid.data();
      pb.grad_formats = b->grad_formats ? sfmt.data() : nullptr;
      pb.use_learned = 0;
      pb.learned_params = nullptr;
      const int F = (int)idx.size();
      std::vector<int> pit(F), pok(F);
      std::vector<float> perr(F);
      GB_TRY(gb_cs_solve_batch(&pb, pit.data(), perr.data(), pok.data(), nullptr));
      for (int q = 0; q < F; ++q) {
        const int t = idx[q];
        hit[t] += pit[q];
        herr[t] = perr[q];
        hok[t] = pok[q];
      }
      g_last_kernel_ms += ms1;
      g_last_bytes += by1;
    }
  }
  int ns = 0;
  for (int t = 0; t < T; ++t) {
    if (iters_out) iters_out[t] = hit[t];
    if (rel_err_out) rel_err_out[t] = herr[t];
    if (success_out) success_out[t] = hok[t];
    ns += hok[t];
  }
  if (num_success) *num_success = ns;
  return GB_OK;
}

extern "C" void gb_cs_batch_last_stats(double *bytes, float *kernel_ms) {
  if (bytes) *bytes = g_last_bytes;
  if (kernel_ms) *kernel_ms = g_last_kernel_ms;
}

extern "C" int gb_cs_batch_last_cluster(void) { return gb_resident_last_cluster(); }
