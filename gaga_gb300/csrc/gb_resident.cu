// gb_resident.cu -- the cluster-resident solver: one thread-block cluster per trial, whole
// solves inside one persistent launch, for the batched form's trials with n <= 8192 and for
// the drop-in's small dense solves.
//
// The slot graphs of gb_batch.cu and the single-trial graph run about a dozen kernels per
// iteration; for problems of a few MB that is bound by kernel dispatch, not by HBM.  Here
// each trial is solved start to finish by one cluster of C CTAs (one CTA per SM):
//
//   * CTA r owns a contiguous range of columns: its slab of A (generated in place for the
//     batched trials, rows padded with zeros to lda = roundup(m, 32); the caller's A for a
//     single solve) and its entries of x, grad, bins and x0 (CGIHT and HTP: also
//     grad_previous, its restriction and the previous bins), which live in shared memory.
//     Every CTA keeps the whole residual (m floats).
//   * A^T r: each CTA over its own columns (lane groups per column, float4 streams).
//   * A v_S: each CTA over its own support columns into a partial m-vector; the partials
//     are summed in rank order through distributed shared memory, each CTA summing its
//     share of the rows, then every CTA gathers the rows it needs.
//   * Every CTA keeps its own copy of the solver state and runs the control phases of the
//     single-trial solver (gb_ctrl.cuh) itself.  The reductions those phases read are
//     combined from the CTAs' partials in rank order, and the bin counts are exact
//     integers, so every copy holds the same bits and every CTA takes the same branches
//     (and so meets the same cluster barriers).
//
// The algorithms (a template parameter, one kernel instance each) are NIHT_S_gen, HTP_S_gen
// and CGIHT_S_gen (GAGA/gaga/algorithms.cu:1274-1441, 2491-2716, 3689-3942), and CGIHT from
// the learned warm start (gb_learned.cu), with the same steps and control as the graph path
// (enq_prologue / enq_body / enq_cg_body in gb_solver.cu); only the order of floating-point
// sums differs.  A batched trial is the problem gb_cs_generate_and_solve draws with
// seed + trial id (Gaussian A, +-1 signal on the createVector support).
#include <cooperative_groups.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <map>
#include <vector>

#include "gb_ctrl.cuh"
#include "gb_internal.cuh"
#include "gb_mlp.cuh"
#include "gb_philox.cuh"
#include "gb_resident.h"

namespace cg = cooperative_groups;

#define RS_THREADS 512
#define RS_WARPS (RS_THREADS / 32)
#define RS_NPUB 16

// algorithms of the resident kernel (RS_CGIHT_ML: CGIHT from the learned warm start)
enum { RS_NIHT = 0, RS_CGIHT = 1, RS_CGIHT_ML = 2, RS_HTP = 3 };

namespace {

struct RsParams {
  int T;  // resident trials (entries of order)
  unsigned int seed;
  float tol_rel;
  int maxiter;
  const int *n, *m, *k;
  const unsigned int *tid;
  const int *order;  // resident trials, largest first
  int *queue;
  int *iters;
  float *err;
  int *ok;
  double *bytes;
  float *A;        // per cluster: a_stride floats
  size_t a_stride;
  int *xhist;      // per cluster: n_cap key bins
  int n_cap, m_cap, nb_cap;
  // single given-data solve (the drop-in): A (column-major, lda_u, m % 4 == 0), y, the
  // initial state in st_io (written back at the end), x out; one cluster, T = 1
  int single;
  const float *Ag;
  int lda_u;
  const float *yg;
  float *xg;
  GbState *st_io;
  // learned warm start (RS_CGIHT_ML): the MLP parameters; per trial whether it fell back
  const float *ml_params;
  int *fb;
  // batched trials: the A^T r operand (GB_GRAD_*) and, when compact, its per-cluster copies
  // (a_stride entries each, indexed like A)
  int gfmt;
  const unsigned char *gfmts;  // per trial (device, indexed like n, m, k), or null: gfmt for all
  unsigned short *Ah;
  unsigned char *Al;
  int rec_every;  // batched CGIHT: residual recurrence (GbState::rec_every)
};

// Shared-memory layout of one CTA (the same on host and device).
struct RsLayout {
  int nc_cap, lda_cap, rc4_cap, nb_cap;
  size_t o_st, o_pub, o_x, o_grad, o_x0, o_bins, o_sidx, o_r, o_part, o_rowp, o_ypart, o_cnt, o_cntf, o_gscr;
  size_t o_gp, o_gpt, o_binsp, o_rowa, o_rowb;  // CGIHT only (zero bytes for NIHT)
  size_t o_mlh, o_mlc;                         // learned warm start only
  size_t bytes;
};

__host__ __device__ inline size_t rs_take(size_t &o, size_t b) {
  const size_t r = o;
  o += (b + 15) / 16 * 16;
  return r;
}

// the batched trials' bin count, max(n / 20, 1000) (batch_trial_fields)
__host__ __device__ inline int rs_default_bins(int n_cap) { return n_cap / 20 > 1000 ? n_cap / 20 : 1000; }

__host__ __device__ inline RsLayout rs_layout(int n_cap, int m_cap, int C, int nb, int alg = RS_NIHT) {
  RsLayout L;
  L.nc_cap = ((n_cap + C - 1) / C + 3) / 4 * 4;
  L.lda_cap = (m_cap + 31) / 32 * 32;
  L.rc4_cap = (L.lda_cap / 4 + C - 1) / C;
  L.nb_cap = (nb + 3) / 4 * 4;
  size_t o = 0;
  L.o_st = rs_take(o, sizeof(GbState));
  L.o_pub = rs_take(o, RS_NPUB * 8);  // RS_NPUB floats, then RS_NPUB ints
  L.o_x = rs_take(o, (size_t)L.nc_cap * 4);
  L.o_grad = rs_take(o, (size_t)L.nc_cap * 4);
  L.o_x0 = rs_take(o, (size_t)L.nc_cap * 4);
  L.o_bins = rs_take(o, (size_t)L.nc_cap * 4);
  L.o_sidx = rs_take(o, (size_t)L.nc_cap * 4);
  L.o_r = rs_take(o, (size_t)L.lda_cap * 4);
  L.o_part = rs_take(o, (size_t)L.lda_cap * 4);
  L.o_rowp = rs_take(o, (size_t)L.rc4_cap * 16);
  L.o_ypart = rs_take(o, (size_t)L.rc4_cap * 16);
  L.o_cnt = rs_take(o, (size_t)L.nb_cap * 4);
  L.o_cntf = rs_take(o, (size_t)L.nb_cap * 4);
  L.o_gscr = rs_take(o, (size_t)RS_THREADS * 16);
  const size_t cg = alg == RS_CGIHT || alg == RS_CGIHT_ML || alg == RS_HTP ? 1 : 0;
  L.o_gp = rs_take(o, cg * L.nc_cap * 4);      // grad_previous (own columns)
  L.o_gpt = rs_take(o, cg * L.nc_cap * 4);     // grad_prev_thres
  L.o_binsp = rs_take(o, cg * L.nc_cap * 4);   // bins before the last binning
  L.o_rowa = rs_take(o, cg * L.rc4_cap * 16);  // own rows of A grad_prev_thres, then of A gp
  L.o_rowb = rs_take(o, cg * L.rc4_cap * 16);  // own rows of A x_thres
  const size_t ml = alg == RS_CGIHT_ML ? 1 : 0;
  // (32 KB: more shared memory leaves the SM's L1 too small; a 66 KB layout measured 12%
  // slower over the whole solve)
  L.o_mlh = rs_take(o, ml * ML_RANK_BINS * 4);  // the CTA's |g| rank histogram
  L.o_mlc = rs_take(o, ml * ML_RANK_BINS * 4);  // the cluster's: 2 * exclusive prefix + count
  L.bytes = o;
  return L;
}

template <class T>
__device__ __forceinline__ T *peer(cg::cluster_group &cl, T *p, int rank) {
  return cl.map_shared_rank(p, rank);
}

__device__ __forceinline__ float4 f4zero() { return make_float4(0.0f, 0.0f, 0.0f, 0.0f); }

// st->red[slot] = sum (rank order, in double) / max of the CTAs' published partials
__device__ double combine_sum(cg::cluster_group &cl, int C, float *pub, int slot) {
  double a = 0.0;
  for (int c = 0; c < C; ++c) a += (double)peer(cl, pub, c)[slot];
  return a;
}
__device__ float combine_max(cg::cluster_group &cl, int C, float *pub, int slot) {
  float a = 0.0f;
  for (int c = 0; c < C; ++c) a = fmaxf(a, peer(cl, pub, c)[slot]);
  return a;
}

// sum and max of the CTA's threads in one pass (thread 0 gets both)
__device__ __forceinline__ void block_reduce_sum_max(float s, float m, float *red32, float *out_s, float *out_m) {
  s = warp_sum(s);
  m = warp_max(m);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) { red32[wid] = s; red32[16 + wid] = m; }
  __syncthreads();
  if (wid == 0) {
    float a = lane < RS_WARPS ? red32[lane] : 0.0f;
    float b = lane < RS_WARPS ? red32[16 + lane] : 0.0f;
    a = warp_sum(a);
    b = warp_max(b);
    if (lane == 0) { *out_s = a; *out_m = b; }
  }
}

// out[c] = A[:, c0 + c] . r for the CTA's columns.  G lanes per column, each lane keeping
// U x V float4 loads in flight over V adjacent columns (one SM streams about as many bytes
// per second as it has in flight per memory latency).  r is the full residual in shared
// memory, zero in the padding rows (as A is).
template <int G, int U, int V>
__device__ void at_own_t(const float *A, int lda, int q4, int c0, int nc, const float *r, float *out) {
  constexpr int PW = 32 / G;
  constexpr int STEP = RS_WARPS * PW * V;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int gl = lane % G, gsub = lane / G;
  const float4 *r4 = reinterpret_cast<const float4 *>(r);
  for (int base = 0; base < nc; base += STEP) {
    const int col0 = base + (wid * PW + gsub) * V;
    float acc[V];
#pragma unroll
    for (int v = 0; v < V; ++v) acc[v] = 0.0f;
    for (int i0 = gl; i0 < q4; i0 += U * G) {
      float4 a[V][U];
#pragma unroll
      for (int v = 0; v < V; ++v) {
        const float4 *a4 = reinterpret_cast<const float4 *>(A + (size_t)(c0 + col0 + v) * lda);
#pragma unroll
        for (int u = 0; u < U; ++u) {
          const int i = i0 + u * G;
          a[v][u] = (col0 + v < nc && i < q4) ? __ldcg(a4 + i) : f4zero();
        }
      }
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const int i = i0 + u * G;
        if (i < q4) {
          const float4 rr = r4[i];
#pragma unroll
          for (int v = 0; v < V; ++v) {
            acc[v] = fmaf(a[v][u].x, rr.x, acc[v]);
            acc[v] = fmaf(a[v][u].y, rr.y, acc[v]);
            acc[v] = fmaf(a[v][u].z, rr.z, acc[v]);
            acc[v] = fmaf(a[v][u].w, rr.w, acc[v]);
          }
        }
      }
    }
#pragma unroll
    for (int v = 0; v < V; ++v) {
      float s = acc[v];
#pragma unroll
      for (int o = G >> 1; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
      if (gl == 0 && col0 + v < nc) out[col0 + v] = s;
    }
  }
}

// DEEP: 16 float4 loads in flight per lane (one cluster alone on the GPU, reading from L2);
// otherwise 8 (every SM streaming from HBM: more requests in flight measured slower)
template <bool DEEP>
__device__ void at_own(const float *A, int lda, int q4, int c0, int nc, const float *r, float *out) {
  if (DEEP) {
    if (q4 >= 512) at_own_t<32, 16, 1>(A, lda, q4, c0, nc, r, out);
    else if (q4 >= 256) at_own_t<32, 8, 2>(A, lda, q4, c0, nc, r, out);
    else if (q4 >= 128) at_own_t<32, 4, 4>(A, lda, q4, c0, nc, r, out);
    else if (q4 >= 64) at_own_t<32, 2, 8>(A, lda, q4, c0, nc, r, out);
    else if (q4 >= 32) at_own_t<16, 2, 8>(A, lda, q4, c0, nc, r, out);
    else at_own_t<8, 4, 4>(A, lda, q4, c0, nc, r, out);
  } else {
    if (q4 >= 256) at_own_t<32, 8, 1>(A, lda, q4, c0, nc, r, out);
    else if (q4 >= 128) at_own_t<32, 4, 2>(A, lda, q4, c0, nc, r, out);
    else if (q4 >= 64) at_own_t<32, 2, 4>(A, lda, q4, c0, nc, r, out);
    else if (q4 >= 32) at_own_t<16, 2, 4>(A, lda, q4, c0, nc, r, out);
    else at_own_t<8, 4, 2>(A, lda, q4, c0, nc, r, out);
  }
}

// at_own_t over the compact operand (GB_GRAD_A24 with LO, GB_GRAD_BF16 without): groups of
// 8 rows (16 bytes of high parts, 8 of low bytes), q8 = lda / 8 groups
template <int G, int U, int V, int LO>
__device__ void at_own_c_t(const unsigned short *Ah, const unsigned char *Al, int lda, int q8, int c0, int nc,
                           const float *r, float *out) {
  constexpr int PW = 32 / G;
  constexpr int STEP = RS_WARPS * PW * V;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int gl = lane % G, gsub = lane / G;
  const float4 *r4 = reinterpret_cast<const float4 *>(r);
  for (int base = 0; base < nc; base += STEP) {
    const int col0 = base + (wid * PW + gsub) * V;
    float acc[V];
#pragma unroll
    for (int v = 0; v < V; ++v) acc[v] = 0.0f;
    for (int i0 = gl; i0 < q8; i0 += U * G) {
      uint4 h[V][U];
      uint2 l[V][U];
#pragma unroll
      for (int v = 0; v < V; ++v) {
        const size_t e = (size_t)(c0 + col0 + v) * lda;
        const uint4 *h4 = reinterpret_cast<const uint4 *>(Ah + e);
        const uint2 *l2 = reinterpret_cast<const uint2 *>(Al + e);
#pragma unroll
        for (int u = 0; u < U; ++u) {
          const int i = i0 + u * G;
          const bool ok = col0 + v < nc && i < q8;
          h[v][u] = ok ? __ldcg(h4 + i) : make_uint4(0u, 0u, 0u, 0u);
          l[v][u] = (LO && ok) ? __ldcg(l2 + i) : make_uint2(0u, 0u);
        }
      }
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const int i = i0 + u * G;
        if (i < q8) {
          const float4 ra = r4[2 * i], rb = r4[2 * i + 1];
#pragma unroll
          for (int v = 0; v < V; ++v) {
            float a[8];
            dec8(h[v][u], l[v][u], a, LO);
            acc[v] = fmaf(a[0], ra.x, acc[v]);
            acc[v] = fmaf(a[1], ra.y, acc[v]);
            acc[v] = fmaf(a[2], ra.z, acc[v]);
            acc[v] = fmaf(a[3], ra.w, acc[v]);
            acc[v] = fmaf(a[4], rb.x, acc[v]);
            acc[v] = fmaf(a[5], rb.y, acc[v]);
            acc[v] = fmaf(a[6], rb.z, acc[v]);
            acc[v] = fmaf(a[7], rb.w, acc[v]);
          }
        }
      }
    }
#pragma unroll
    for (int v = 0; v < V; ++v) {
      float s = acc[v];
#pragma unroll
      for (int o = G >> 1; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
      if (gl == 0 && col0 + v < nc) out[col0 + v] = s;
    }
  }
}

template <int LO>
__device__ void at_own_c(const unsigned short *Ah, const unsigned char *Al, int lda, int q8, int c0, int nc,
                         const float *r, float *out) {
  if (q8 >= 256) at_own_c_t<32, 8, 1, LO>(Ah, Al, lda, q8, c0, nc, r, out);
  else if (q8 >= 128) at_own_c_t<32, 4, 2, LO>(Ah, Al, lda, q8, c0, nc, r, out);
  else if (q8 >= 64) at_own_c_t<32, 2, 4, LO>(Ah, Al, lda, q8, c0, nc, r, out);
  else if (q8 >= 32) at_own_c_t<16, 2, 4, LO>(Ah, Al, lda, q8, c0, nc, r, out);
  else at_own_c_t<8, 4, 2, LO>(Ah, Al, lda, q8, c0, nc, r, out);
}

// A^T r for the trial's own columns in the trial's operand format (gfmt)
template <bool DEEP>
__device__ __forceinline__ void at_trial(int gfmt, const float *A, const unsigned short *Ah,
                                         const unsigned char *Al, int lda, int q4, int c0, int nc, const float *r,
                                         float *out) {
  if (gfmt == GB_GRAD_A24) at_own_c<1>(Ah, Al, lda, q4 / 2, c0, nc, r, out);
  else if (gfmt == GB_GRAD_BF16) at_own_c<0>(Ah, Al, lda, q4 / 2, c0, nc, r, out);
  else at_own<DEEP>(A, lda, q4, c0, nc, r, out);
}

// part (lda floats) = sum over the CTA's support entries e (ascending) of
// A[:, c0 + sidx[e]] * v[sidx[e]].  Up to 512 row quads: one pass of the CTA, entries split
// over P = 512 / TG thread groups whose partial vectors are then summed in group order.
// NV = 2 also forms part2 from v2 with the same column loads (the unrestricted CG step's
// A x and A p), each product summed in the order of its own NV = 1 call.
template <int NV>
__device__ void av_own_partial_t(const float *A, int lda, int q4, int c0, const int *sidx, int s_own,
                                 const float *v, const float *v2, float *part, float *part2, float4 *gscr) {
  float4 *pv[2] = {reinterpret_cast<float4 *>(part), reinterpret_cast<float4 *>(part2)};
  const float *vv[2] = {v, v2};
  const int tg = q4 >= RS_THREADS ? RS_THREADS : (q4 + 31) / 32 * 32;
  const int P = RS_THREADS / tg;
  auto fma4 = [](float4 &acc, const float4 &l, float w) {
    acc.x = fmaf(l.x, w, acc.x); acc.y = fmaf(l.y, w, acc.y);
    acc.z = fmaf(l.z, w, acc.z); acc.w = fmaf(l.w, w, acc.w);
  };
  if (P == 1) {
    // rows t, t + 512, t + 1024, t + 1536 (q4 <= 2048)
    const int t = threadIdx.x;
    float4 acc[NV][4];
#pragma unroll
    for (int p = 0; p < NV; ++p)
#pragma unroll
      for (int q = 0; q < 4; ++q) acc[p][q] = f4zero();
    int e = 0;
    for (; e + 1 < s_own; e += 2) {
      const int ca = sidx[e], cb = sidx[e + 1];
      const float4 *aa = reinterpret_cast<const float4 *>(A + (size_t)(c0 + ca) * lda);
      const float4 *ab = reinterpret_cast<const float4 *>(A + (size_t)(c0 + cb) * lda);
      float4 la[4], lb[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const int i = t + q * RS_THREADS;
        la[q] = i < q4 ? __ldcg(aa + i) : f4zero();
        lb[q] = i < q4 ? __ldcg(ab + i) : f4zero();
      }
#pragma unroll
      for (int p = 0; p < NV; ++p) {
        const float wa = vv[p][ca], wb = vv[p][cb];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          fma4(acc[p][q], la[q], wa);
          fma4(acc[p][q], lb[q], wb);
        }
      }
    }
    if (e < s_own) {
      const int ca = sidx[e];
      const float4 *aa = reinterpret_cast<const float4 *>(A + (size_t)(c0 + ca) * lda);
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const int i = t + q * RS_THREADS;
        const float4 la = i < q4 ? __ldcg(aa + i) : f4zero();
#pragma unroll
        for (int p = 0; p < NV; ++p) fma4(acc[p][q], la, vv[p][ca]);
      }
    }
#pragma unroll
    for (int p = 0; p < NV; ++p)
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const int i = t + q * RS_THREADS;
        if (i < q4) pv[p][i] = acc[p][q];
      }
  } else {
    // one row quad per thread; group p takes entries p, p + P, ... four at a time
    const int g = threadIdx.x / tg, t = threadIdx.x % tg;
    float4 acc[NV];
#pragma unroll
    for (int p = 0; p < NV; ++p) acc[p] = f4zero();
    if (g < P && t < q4) {
      int e = g;
      for (; e + 3 * P < s_own; e += 4 * P) {
        float4 l[4];
        int cc[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          cc[u] = sidx[e + u * P];
          l[u] = __ldcg(reinterpret_cast<const float4 *>(A + (size_t)(c0 + cc[u]) * lda) + t);
        }
#pragma unroll
        for (int p = 0; p < NV; ++p)
#pragma unroll
          for (int u = 0; u < 4; ++u) fma4(acc[p], l[u], vv[p][cc[u]]);
      }
      for (; e < s_own; e += P) {
        const int c = sidx[e];
        const float4 l = __ldcg(reinterpret_cast<const float4 *>(A + (size_t)(c0 + c) * lda) + t);
#pragma unroll
        for (int p = 0; p < NV; ++p) fma4(acc[p], l, vv[p][c]);
      }
    }
    // group partials summed in group order, one product at a time through gscr
#pragma unroll
    for (int p = 0; p < NV; ++p) {
      if (p > 0) __syncthreads();
      if (g < P && t < q4) gscr[g * tg + t] = acc[p];
      __syncthreads();
      for (int i = threadIdx.x; i < q4; i += RS_THREADS) {
        float4 s = gscr[i];
        for (int pp = 1; pp < P; ++pp) {
          const float4 h = gscr[pp * tg + i];
          s.x += h.x; s.y += h.y; s.z += h.z; s.w += h.w;
        }
        pv[p][i] = s;
      }
    }
  }
}

__device__ void av_own_partial(const float *A, int lda, int q4, int c0, const int *sidx, int s_own,
                               const float *v, float *part, float4 *gscr) {
  av_own_partial_t<1>(A, lda, q4, c0, sidx, s_own, v, nullptr, part, nullptr, gscr);
}

// Rows [rr0, rr1) (row quads) of the cluster sum of the CTAs' partials (rank order); with
// sub_y the result is y - sum.  Stored in rowp (and ycopy) when given; returns this thread's
// sum of squares.
__device__ float reduce_rows(cg::cluster_group &cl, int C, float *part, int rr0, int rr1, const float *ypart,
                             float *rowp, float *ycopy) {
  float s2 = 0.0f;
  const float4 *y4 = reinterpret_cast<const float4 *>(ypart);
  float4 *o4 = reinterpret_cast<float4 *>(rowp);
  float4 *c4 = reinterpret_cast<float4 *>(ycopy);
  for (int i = rr0 + threadIdx.x; i < rr1; i += RS_THREADS) {
    float4 s = f4zero();
    for (int c = 0; c < C; ++c) {
      const float4 p = reinterpret_cast<const float4 *>(peer(cl, part, c))[i];
      s.x += p.x; s.y += p.y; s.z += p.z; s.w += p.w;
    }
    if (ypart) {
      const float4 yy = y4[i - rr0];
      s.x = yy.x - s.x; s.y = yy.y - s.y; s.z = yy.z - s.z; s.w = yy.w - s.w;
    }
    if (rowp) o4[i - rr0] = s;
    if (ycopy) c4[i - rr0] = s;
    s2 = fmaf(s.x, s.x, s2);
    s2 = fmaf(s.y, s.y, s2);
    s2 = fmaf(s.z, s.z, s2);
    s2 = fmaf(s.w, s.w, s2);
  }
  return s2;
}

// r (all q4 row quads) from the CTAs' row shares
__device__ void gather_rows(cg::cluster_group &cl, int C, int q4, int RB, float *rowp, float *r) {
  float4 *r4 = reinterpret_cast<float4 *>(r);
  for (int c = 0; c < C; ++c) {
    const int a = min(q4, c * RB), b = min(q4, a + RB);
    const float4 *src = reinterpret_cast<const float4 *>(peer(cl, rowp, c));
    for (int i = a + threadIdx.x; i < b; i += RS_THREADS) r4[i] = src[i - a];
  }
}

// the k-th bin scan of k_kbin (gb_solver.cu) over counters cnt[0, max_bin) (shared memory,
// or the cluster's global key histogram read at L2), same results, by warp 0 alone: lane l
// sums a contiguous chunk, a shuffle scan finds the lane whose chunk reaches k, that lane
// walks its chunk.  One CTA barrier at the end publishes the state.
template <bool GLOBAL>
__device__ void block_kbin(GbState *st, const int *cnt, int k) {
  if (threadIdx.x < 32) {
    const int lane = threadIdx.x;
    const int max_bin = st->max_bin;
    const int CH = (max_bin + 31) / 32;
    const int b0 = min(lane * CH, max_bin), b1 = min(b0 + CH, max_bin);
    auto ld = [&](int b) { return GLOBAL ? __ldcg(cnt + b) : cnt[b]; };
    int csum = 0;
    for (int b = b0; b < b1; ++b) csum += ld(b);
    int incl = csum;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int v = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += v;
    }
    const int total = __shfl_sync(0xffffffffu, incl, 31);
    const int excl = incl - csum;
    const unsigned hit = __ballot_sync(0xffffffffu, k > 0 && excl < k && incl >= k);
    int res_kbin = -2, res_sum = 0;
    if (hit) {
      const int owner = __ffs(hit) - 1;
      if (lane == owner) {
        int s2 = excl;
        for (int b = b0; b < b1; ++b) {
          s2 += ld(b);
          if (s2 >= k) { res_kbin = b; res_sum = s2; break; }
        }
      }
      res_kbin = __shfl_sync(0xffffffffu, res_kbin, owner);
      res_sum = __shfl_sync(0xffffffffu, res_sum, owner);
    }
    if (lane == 0) {
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
      st->k_bin = k_bin;
      st->sum = sum;
    }
  }
  __syncthreads();
}

// sidx = ascending { c < nc : bins[c] <= kb }; returns the count (every thread)
__device__ int compact_own(const int *bins, int nc, int kb, int *sidx, int *wcnt) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  int running = 0;
  for (int base = 0; base < nc; base += RS_THREADS) {
    const int c = base + threadIdx.x;
    const bool in = c < nc && bins[c] <= kb;
    const unsigned bal = __ballot_sync(0xffffffffu, in);
    if (lane == 0) wcnt[wid] = __popc(bal);
    __syncthreads();
    int wb = 0, tot = 0;
    for (int w = 0; w < RS_WARPS; ++w) {
      const int cw = wcnt[w];
      if (w < wid) wb += cw;
      tot += cw;
    }
    if (in) sidx[running + wb + __popc(bal & ((1u << lane) - 1u))] = c;
    running += tot;
    __syncthreads();
  }
  return running;
}

// LinearBinning of the CTA's entries of v into bins and the CTA's counters (k_hist)
__device__ void hist_own(const GbState *st, const float *v, int *bins, int nc, int *cnt, int *gcnt) {
  const float intercept = st->max_value;
  const float slope = st->slope;
  const float small_f = __double2float_rd((double)intercept * 0.000001);
  const int max_bin = st->max_bin;
  for (int c = threadIdx.x; c < nc; c += RS_THREADS) {
    bool counted;
    const int b = lin_bin(v[c], slope, intercept, small_f, counted);
    bins[c] = b;
    if (counted && b < max_bin) {
      const unsigned act = __activemask();
      const unsigned same = __match_any_sync(act, b);
      if ((int)(threadIdx.x & 31) == __ffs(same) - 1) {
        if (gcnt) atomicAdd(&gcnt[b], __popc(same));
        else atomicAdd(&cnt[b], __popc(same));
      }
    }
  }
}

// ml_forward1 (gb_mlp.cuh) with the weights read from global memory (cached) and rounded to
// BF16 at every use: the same arithmetic, no shared memory
__device__ __forceinline__ float ml_w(const float *__restrict__ p, int i) { return ml_bf16(__ldg(p + i)); }
__device__ float ml_forward1_g(const float *__restrict__ p, const float f[ML_IN]) {
  float h1[ML_H];
#pragma unroll
  for (int j = 0; j < ML_H; ++j) {
    float a = ml_w(p, ML_OFF_B1 + j);
#pragma unroll
    for (int q = 0; q < ML_IN; ++q) a = fmaf(ml_w(p, ML_OFF_W1 + j * ML_IN + q), f[q], a);
    h1[j] = ml_gelu(a);
  }
  float out = ml_w(p, ML_OFF_B3);
  for (int j = 0; j < ML_H; ++j) {
    float a = ml_w(p, ML_OFF_B2 + j);
#pragma unroll
    for (int i = 0; i < ML_H; ++i) a = fmaf(ml_w(p, ML_OFF_W2 + j * ML_H + i), h1[i], a);
    out = fmaf(ml_w(p, ML_OFF_W3 + j), ml_gelu(a), out);
  }
  return out;
}

// x_c = g_c * net(features_c) over the CTA's columns (g in x; bins: each entry's rank bin;
// mlc: 2 * exclusive prefix + count per bin); returns the thread's max |x|.  Not inlined: the
// network's registers stay out of the solver loop's allocation.
__device__ __noinline__ float ml_warm_own(float *x, const int *bins, int nc, int n, float mx, float delta, float rho,
                                          const int *mlc, const float *__restrict__ p) {
  float mxx = 0.0f;
  for (int c = threadIdx.x; c < nc; c += RS_THREADS) {
    const float gi = x[c];
    const int b = bins[c];
    float f[ML_IN];
    f[0] = mx > 0.0f ? fabsf(gi) / mx : 0.0f;
    f[1] = (0.5f * (float)mlc[b]) / (float)n;  // (cum[b] + counts[b] / 2) / n, exact
    f[2] = delta;
    f[3] = rho;
    const float v = gi * ml_forward1_g(p, f);
    x[c] = v;
    mxx = fmaxf(mxx, fabsf(v));
  }
  return mxx;
}

// set by a launch whose dynamic shared memory is smaller than the layout its parameters imply
// (every CTA then returns before touching memory); read and cleared by gb_resident_check
__device__ int g_rs_guard;

// DEEP: the single given-data solve's deeper A^T r pipeline (a separate instance, so the
// batched kernel keeps its own register allocation).  ALG: RS_NIHT or RS_CGIHT.
template <bool DEEP, int ALG>
__global__ void __launch_bounds__(RS_THREADS, 1) k_resident(const RsParams P) {
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ int s_q;
  __shared__ float red32[32];
  __shared__ int wcnt[RS_WARPS];
  cg::cluster_group cl = cg::this_cluster();
  const int C = (int)cl.num_blocks(), rank = (int)cl.block_rank();
  const int cid = blockIdx.x / C;
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  const RsLayout L = rs_layout(P.n_cap, P.m_cap, C, P.nb_cap, ALG);
  {
    unsigned int dsmem;
    asm volatile("mov.u32 %0, %%dynamic_smem_size;" : "=r"(dsmem));
    if ((size_t)dsmem < L.bytes) {  // the same for every CTA of the launch
      if (threadIdx.x == 0) atomicExch(&g_rs_guard, 1);
      return;
    }
  }
  GbState *st = reinterpret_cast<GbState *>(smem + L.o_st);
  float *pub = reinterpret_cast<float *>(smem + L.o_pub);
  int *ipub = reinterpret_cast<int *>(pub + RS_NPUB);
  float *x = reinterpret_cast<float *>(smem + L.o_x);
  float *grad = reinterpret_cast<float *>(smem + L.o_grad);
  float *x0 = reinterpret_cast<float *>(smem + L.o_x0);
  int *bins = reinterpret_cast<int *>(smem + L.o_bins);
  int *sidx = reinterpret_cast<int *>(smem + L.o_sidx);
  float *r = reinterpret_cast<float *>(smem + L.o_r);
  float *part = reinterpret_cast<float *>(smem + L.o_part);
  float *rowp = reinterpret_cast<float *>(smem + L.o_rowp);
  float *ypart = reinterpret_cast<float *>(smem + L.o_ypart);
  int *cnt = reinterpret_cast<int *>(smem + L.o_cnt);
  int *cntf = reinterpret_cast<int *>(smem + L.o_cntf);
  float4 *gscr = reinterpret_cast<float4 *>(smem + L.o_gscr);
  float *gp = reinterpret_cast<float *>(smem + L.o_gp);
  float *gpt = reinterpret_cast<float *>(smem + L.o_gpt);
  int *binsp = reinterpret_cast<int *>(smem + L.o_binsp);
  float *rowa = reinterpret_cast<float *>(smem + L.o_rowa);
  float *rowb = reinterpret_cast<float *>(smem + L.o_rowb);
  int *mlh = reinterpret_cast<int *>(smem + L.o_mlh);
  int *mlc = reinterpret_cast<int *>(smem + L.o_mlc);
  constexpr bool IS_CG = ALG == RS_CGIHT || ALG == RS_CGIHT_ML;
  float *A = P.single ? const_cast<float *>(P.Ag) : P.A + (size_t)cid * P.a_stride;
  unsigned short *Ah = P.Ah ? P.Ah + (size_t)cid * P.a_stride : nullptr;
  unsigned char *Al = P.Al ? P.Al + (size_t)cid * P.a_stride : nullptr;
  int *xh = P.single ? nullptr : P.xhist + (size_t)cid * P.n_cap;
  {
    unsigned int *w = reinterpret_cast<unsigned int *>(st);
    for (int i = tid; i < (int)(sizeof(GbState) / 4); i += RS_THREADS) w[i] = 0u;
  }
  __syncthreads();
  for (int pass = 0;; ++pass) {
    // ---- next trial: rank 0 takes it from the queue, the others read it from rank 0 (the
    // single given-data solve has one trial and no queue)
    int q = pass;
    if (!P.single) {
      if (rank == 0 && tid == 0) s_q = atomicAdd(P.queue, 1);
      cl.sync();
      q = *peer(cl, &s_q, 0);
    }
    if (q >= P.T) break;
    const int t = P.single ? 0 : P.order[q];
    const int m = P.single ? P.m_cap : P.m[t], n = P.single ? P.n_cap : P.n[t];
    const int lda = P.single ? P.lda_u : (m + 31) / 32 * 32, q4 = P.single ? m / 4 : lda / 4;
    const int CH = (n + C - 1) / C;
    const int c0 = min(n, rank * CH), nc = min(n, c0 + CH) - c0;
    const int RB = (q4 + C - 1) / C;
    const int rr0 = min(q4, rank * RB), rr1 = min(q4, rr0 + RB);
    int s_own = 0;
    if (P.single) {
      // ---- the caller's problem: initial state, y (whole in r, own rows in ypart), ||y||^2
      if (tid == 0) {
        const unsigned int *src = reinterpret_cast<const unsigned int *>(P.st_io);
        unsigned int *dst = reinterpret_cast<unsigned int *>(st);
        for (int i = 0; i < (int)(sizeof(GbState) / 4); ++i) dst[i] = src[i];
      }
      const float4 *y4 = reinterpret_cast<const float4 *>(P.yg);
      float4 *r4 = reinterpret_cast<float4 *>(r);
      float4 *yp4 = reinterpret_cast<float4 *>(ypart);
      for (int i = tid; i < q4; i += RS_THREADS) r4[i] = __ldcg(y4 + i);
      float s2 = 0.0f;
      for (int i = rr0 + tid; i < rr1; i += RS_THREADS) {
        const float4 v = __ldcg(y4 + i);
        yp4[i - rr0] = v;
        s2 = fmaf(v.x, v.x, s2); s2 = fmaf(v.y, v.y, s2); s2 = fmaf(v.z, v.z, s2); s2 = fmaf(v.w, v.w, s2);
      }
      const float b = block_reduce<0>(s2, red32);
      if (tid == 0) pub[R_RES] = b;
      cl.sync();
      if (tid == 0) {
        st->red[R_RES] = combine_sum(cl, C, pub, R_RES);
        // NIHT prologue (algorithms.cu:1296-1354): resid = y; err = ||y||
        ctrl_phase(st, C_INIT0, 0);
      }
      __syncthreads();
    } else {
    const uint32_t key = P.seed + (P.tid ? P.tid[t] : (uint32_t)t);
    if (tid == 0) {
      batch_trial_fields(st, t, m, n, P.k[t], P.maxiter,
                         IS_CG ? GB_ALG_CGIHT : ALG == RS_HTP ? GB_ALG_HTP : GB_ALG_NIHT);
      st->lda = lda;
      st->gfmt = P.gfmts ? P.gfmts[t] : P.gfmt;
      st->rec_every = P.rec_every;
    }
    const int gfmt_t = P.gfmts ? P.gfmts[t] : P.gfmt;  // this trial's A^T r operand
    // ---- draw the trial (k_b_gen_A, k_b_gen_x, key bins, y = A x0 of gb_batch.cu)
    for (int col = wid; col < nc; col += RS_WARPS) {
      const int j = c0 + col;
      float *cp = A + (size_t)j * lda;
      if (gfmt_t == GB_GRAD_FP32) {
        gbgen::gen_dense_column(cp, j, m, key, 0u, 1, lane, 32);
        for (int i = m + lane; i < lda; i += 32) cp[i] = 0.0f;
      } else {
        // the compact A^T r operand, rounded from the drawn values as they are written
        const bool has_lo = gfmt_t == GB_GRAD_A24;
        unsigned short *h = Ah + (size_t)j * lda;
        unsigned char *l = has_lo ? Al + (size_t)j * lda : nullptr;
        gbgen::gen_dense_column_emit(cp, j, m, key, 0u, 1, lane, 32, [&](int i, float a) {
          const uint32_t b = round_top_bits(__float_as_uint(a), has_lo ? 8 : 16);
          h[i] = (unsigned short)(b >> 16);
          if (has_lo) l[i] = (unsigned char)(b >> 8);
        });
        for (int i = m + lane; i < lda; i += 32) {
          cp[i] = 0.0f;
          h[i] = 0;
          if (has_lo) l[i] = 0;
        }
      }
    }
    float mx = 0.0f;
    for (int c = tid; c < nc; c += RS_THREADS) {
      const int j = c0 + c;
      uint32_t o[4];
      gbgen::philox((uint32_t)(j >> 2), 0u, gbgen::ST_VALUES, 0u, key, gbgen::KEY_HI, o);
      x0[c] = signbit(gbgen::u01(o[j & 3]) - 0.5f) ? -1.0f : 1.0f;
      gbgen::philox((uint32_t)(j >> 2), 0u, gbgen::ST_SUPPORT, 0u, key, gbgen::KEY_HI, o);
      const float u = gbgen::u01(o[j & 3]);
      grad[c] = u;  // the support keys, until the solve starts
      mx = fmaxf(mx, u);
      __stcg(xh + j, 0);
    }
    {
      const float b = block_reduce<1>(mx, red32);
      if (tid == 0) pub[R_XMAX] = b;
    }
    __threadfence();
    cl.sync();
    if (tid == 0) {
      // n linear bins over the keys (createVector.cu:236-248)
      st->red[R_XMAX] = (double)combine_max(cl, C, pub, R_XMAX);
      st->max_value = (float)st->red[R_XMAX];
      st->slope = ((float)(st->n - 1) / st->max_value);
      st->max_bin = st->n;
      st->alpha_bin = 0.25f;
      st->flags[F_DOBIN] = 1;
    }
    __syncthreads();
    hist_own(st, grad, bins, nc, nullptr, xh);
    __threadfence();
    cl.sync();
    block_kbin<true>(st, xh, st->k);
    // the counts came through global memory: every CTA takes rank 0's scan result, so the
    // copies of the state stay identical whatever each CTA read
    cl.sync();
    if (tid == 0) {
      if (rank != 0) {
        const GbState *s0 = peer(cl, st, 0);
        st->k_bin = s0->k_bin;
        st->sum = s0->sum;
        st->min_val = s0->min_val;
        st->alpha_bin = s0->alpha_bin;
        st->max_bin = s0->max_bin;
      }
      st->k = st->sum;  // |support| >= k, the k the solver is given
    }
    __syncthreads();
    {
      const int kb = st->k_bin;
      for (int c = tid; c < nc; c += RS_THREADS)
        if (bins[c] > kb) x0[c] = 0.0f;
    }
    s_own = compact_own(bins, nc, st->k_bin, sidx, wcnt);
    av_own_partial(A, lda, q4, c0, sidx, s_own, x0, part, gscr);
    cl.sync();
    {
      const float s2 = reduce_rows(cl, C, part, rr0, rr1, nullptr, rowp, ypart);
      const float b = block_reduce<0>(s2, red32);
      if (tid == 0) pub[R_RES] = b;
    }
    cl.sync();
    gather_rows(cl, C, q4, RB, rowp, r);
    if (tid == 0) {
      st->red[R_RES] = combine_sum(cl, C, pub, R_RES);
      batch_solver_init(st, P.tol_rel, ALG == RS_CGIHT_ML ? 1 : 0);
      // NIHT prologue (algorithms.cu:1296-1354): resid = y; err = ||y||
      ctrl_phase(st, C_INIT0, 0);
    }
    __syncthreads();
    }
    // A learned warm start abandoned after 10 iterations (C_CGIHT_STOP) is solved again from
    // zero by plain CGIHT on the same cluster, its slab of A still in place, and the
    // iterations add up (the batched form's fallback, gb_cs_solve_batch)
    int warm_iters = 0;
    double warm_bytes = 0.0;
    const double y2 = st->red[R_RES];
    for (int attempt = 0;; ++attempt) {
      if (attempt > 0) {
        warm_iters = st->iter;
        warm_bytes = st->bytes;
        __syncthreads();  // every thread has read the state before thread 0 resets it
        if (tid == 0) {
          st->red[R_RES] = y2;
          st->active = 1;
          batch_solver_init(st, P.tol_rel, 0);
          ctrl_phase(st, C_INIT0, 0);
        }
        gather_rows(cl, C, q4, RB, ypart, r);  // r = y again (every CTA's rows of y are unchanged)
        __syncthreads();
      }
      // x = A^T y ; max|x| ; FindSupportSet ; Threshold
      at_trial<DEEP>(st->gfmt, A, Ah, Al, lda, q4, c0, nc, r, x);
      __syncthreads();
      {
        float mxx = 0.0f;
        for (int c = tid; c < nc; c += RS_THREADS) mxx = fmaxf(mxx, fabsf(x[c]));
        for (int b = tid; b < L.nb_cap; b += RS_THREADS) cnt[b] = 0;
        const float b = block_reduce<1>(mxx, red32);
        if (tid == 0) pub[R_XMAX] = b;
      }
      cl.sync();
      if (tid == 0) st->red[R_XMAX] = (double)combine_max(cl, C, pub, R_XMAX);
      __syncthreads();
      if (ALG == RS_CGIHT_ML && st->learned) {
        // learned warm start (enq_learned_warm, gb_learned.cu): x_i = g_i * net(features_i) with
        // g = A^T y in x; the rank feature from the cluster's 4096-bin histogram of |g|
        const float mx = (float)st->red[R_XMAX];
        const float slope = mx > 0.0f ? (float)(ML_RANK_BINS - 1) / mx : 0.0f;
        for (int b = tid; b < ML_RANK_BINS; b += RS_THREADS) mlh[b] = 0;
        __syncthreads();
        for (int c = tid; c < nc; c += RS_THREADS) {
          int b = (int)((mx - fabsf(x[c])) * slope);
          b = min(max(b, 0), ML_RANK_BINS - 1);
          bins[c] = b;
          atomicAdd(&mlh[b], 1);
        }
        cl.sync();
        {
          // the cluster's counts (rank order) and, in place, 2 * exclusive prefix + count:
          // rank feature (cum + count / 2) / n exactly as ml_features computes it
          constexpr int PER = ML_RANK_BINS / RS_THREADS;
          int loc[PER], tot = 0;
#pragma unroll
          for (int q = 0; q < PER; ++q) {
            const int b = tid * PER + q;
            int sum = 0;
            for (int c = 0; c < C; ++c) sum += peer(cl, mlh, c)[b];
            loc[q] = sum;
            tot += sum;
          }
          int incl = tot;
#pragma unroll
          for (int o = 1; o < 32; o <<= 1) {
            const int v = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += v;
          }
          if (lane == 31) wcnt[wid] = incl;
          __syncthreads();
          int run = incl - tot;
          for (int w2 = 0; w2 < wid; ++w2) run += wcnt[w2];
#pragma unroll
          for (int q = 0; q < PER; ++q) {
            mlc[tid * PER + q] = 2 * run + loc[q];
            run += loc[q];
          }
        }
        __syncthreads();
        const float delta = (float)st->m / (float)st->n, rho = (float)st->k / (float)st->m;
        const float mxx = ml_warm_own(x, bins, nc, n, mx, delta, rho, mlc, P.ml_params);
        const float b = block_reduce<1>(mxx, red32);
        if (tid == 0) pub[R_XMAX] = b;
        cl.sync();
        if (tid == 0) st->red[R_XMAX] = (double)combine_max(cl, C, pub, R_XMAX);
        __syncthreads();
      }
      if (tid == 0) ctrl_phase(st, C_INIT_BINPREP, 0);
      __syncthreads();
      // the support step (enq_support): bins and the k-th bin when binning, threshold always;
      // with save_prev (CGIHT) the previous bins are kept and a support entry that left is
      // flagged (checkSupportEvolution, GAGA/gaga/kernels.cu:178-193) in st->changed
      auto support = [&](bool save_prev) {
        const bool dobin = st->flags[F_DOBIN] != 0;
        if (dobin) {
          if (save_prev)
            for (int c = tid; c < nc; c += RS_THREADS) binsp[c] = bins[c];  // the same thread bins c next
          hist_own(st, x, bins, nc, cnt, nullptr);
          cl.sync();
          const int mb = st->max_bin;
          for (int b = tid; b < mb; b += RS_THREADS) {
            int s = 0;
            for (int c = 0; c < C; ++c) s += peer(cl, cnt, c)[b];
            cntf[b] = s;
          }
          __syncthreads();
          block_kbin<false>(st, cntf, st->k);
        }
        const int kb = st->k_bin, kbp = st->k_bin_prev;
        int chg = 0;
        for (int c = tid; c < nc; c += RS_THREADS) {
          if (bins[c] > kb) x[c] = 0.0f;
          if (save_prev && dobin && binsp[c] <= kbp && bins[c] > kb) chg = 1;
        }
        if (dobin) s_own = compact_own(bins, nc, kb, sidx, wcnt);
        if (save_prev && dobin) {
          const int any = __syncthreads_or(chg);
          if (tid == 0) {
            ipub[1] = any;
            ipub[2] = s_own;
          }
          cl.sync();
          if (tid == 0) {
            int a = 0, sc = 0;
            for (int c = 0; c < C; ++c) {
              a |= peer(cl, ipub, c)[1];
              sc += peer(cl, ipub, c)[2];
            }
            st->changed = a;
            st->s_cnt = sc;  // the new support's size (C_CGIHT_POST compares it)
          }
        }
        __syncthreads();
      };
      support(false);
      if ((ALG == RS_NIHT || ALG == RS_HTP) && tid == 0) ctrl_phase(st, C_INIT_DONE, 0);
      __syncthreads();
      // ---- NIHT iterations (RestrictedSD, GAGA/gaga/functions.cu:659-745, then the support)
      while ((ALG == RS_NIHT || ALG == RS_HTP) && st->active) {
        // resid = y - A x_S ; ||resid||^2
        av_own_partial(A, lda, q4, c0, sidx, s_own, x, part, gscr);
        if (tid == 0) ipub[0] = s_own;
        cl.sync();
        {
          const float s2 = reduce_rows(cl, C, part, rr0, rr1, ypart, rowp, nullptr);
          const float b = block_reduce<0>(s2, red32);
          if (tid == 0) pub[R_RES] = b;
        }
        cl.sync();
        gather_rows(cl, C, q4, RB, rowp, r);
        if (tid == 0) {
          st->red[R_RES] = combine_sum(cl, C, pub, R_RES);
          int sc = 0;
          for (int c = 0; c < C; ++c) sc += peer(cl, ipub, c)[0];
          st->s_cnt = sc;
          ctrl_phase(st, C_PUSH_RES, 0);
        }
        __syncthreads();
        // grad = A^T resid ; ||grad on the support||^2 ; max|grad|
        at_trial<DEEP>(st->gfmt, A, Ah, Al, lda, q4, c0, nc, r, grad);
        __syncthreads();
        {
          const int kb = st->k_bin;
          float s2 = 0.0f, gm = 0.0f;
          for (int c = tid; c < nc; c += RS_THREADS) {
            const float g = grad[c];
            const float o = bins[c] <= kb ? g : 0.0f;
            s2 = fmaf(o, o, s2);
            gm = fmaxf(gm, fabsf(g));
          }
          // published now, combined after the next two cluster barriers with ||A x_thres||^2
          block_reduce_sum_max(s2, gm, red32, &pub[R_XT], &pub[R_GMAX]);
        }
        // ||A x_thres||^2 (x_thres = grad on the support)
        av_own_partial(A, lda, q4, c0, sidx, s_own, grad, part, gscr);
        cl.sync();
        {
          const float s2 = reduce_rows(cl, C, part, rr0, rr1, nullptr, nullptr, nullptr);
          const float b = block_reduce<0>(s2, red32);
          if (tid == 0) pub[R_AXT] = b;
        }
        cl.sync();
        if (tid == 0) {
          st->red[R_XT] = combine_sum(cl, C, pub, R_XT);
          st->red[R_GMAX] = (double)combine_max(cl, C, pub, R_GMAX);
          st->red[R_AXT] = combine_sum(cl, C, pub, R_AXT);
          ctrl_phase(st, C_SD_MU, 0);
        }
        __syncthreads();
        // x += mu grad ; max|x| ; counters cleared
        {
          const float mu = st->mu;
          float mxx = 0.0f;
          for (int c = tid; c < nc; c += RS_THREADS) {
            const float o = fmaf(mu, grad[c], x[c]);
            x[c] = o;
            mxx = fmaxf(mxx, fabsf(o));
          }
          for (int b = tid; b < L.nb_cap; b += RS_THREADS) cnt[b] = 0;
          const float b = block_reduce<1>(mxx, red32);
          if (tid == 0) pub[R_XMAX] = b;
        }
        cl.sync();
        if (tid == 0) {
          st->red[R_XMAX] = (double)combine_max(cl, C, pub, R_XMAX);
          ctrl_phase(st, C_BINPREP, 0);
        }
        __syncthreads();
        support(false);
        if (ALG == RS_HTP) {
          // CG projection on the support (GAGA/gaga/algorithms.cu:2588-2669), then up to 15
          // RestrictedCG steps (functions.cu:922-1000), as enq_body / enq_cg_body run them
          auto av_rows = [&](const float *v, bool sub_y, float *rows, float *full, int slot) {
            av_own_partial(A, lda, q4, c0, sidx, s_own, v, part, gscr);
            cl.sync();
            const float s2 = reduce_rows(cl, C, part, rr0, rr1, sub_y ? ypart : nullptr, rows, nullptr);
            const float b = block_reduce<0>(s2, red32);
            if (tid == 0 && slot >= 0) pub[slot] = b;
            cl.sync();
            if (full) gather_rows(cl, C, q4, RB, rows, full);
          };
          av_rows(x, true, rowp, r, R_RES);  // resid = y - A x_S
          if (tid == 0) st->red[R_RES] = combine_sum(cl, C, pub, R_RES);
          __syncthreads();
          at_own<DEEP>(A, lda, q4, c0, nc, r, grad);  // grad = (A^T resid) on the support; gp = grad
          __syncthreads();
          {
            const int kb = st->k_bin;
            float s2 = 0.0f;
            for (int c = tid; c < nc; c += RS_THREADS) {
              const float g = bins[c] > kb ? 0.0f : grad[c];
              grad[c] = g;
              gp[c] = g;
              s2 = fmaf(g, g, s2);
            }
            const float b = block_reduce<0>(s2, red32);
            if (tid == 0) pub[R_DOT1] = b;
          }
          cl.sync();
          if (tid == 0) {
            st->red[R_DOT1] = combine_sum(cl, C, pub, R_DOT1);
            ctrl_phase(st, C_HTP_CGINIT, 0);
          }
          __syncthreads();
          while (st->flags[F_CG] && st->active) {
            av_rows(grad, false, rowp, r, R_CG);  // resid = A grad_S
            if (tid == 0) {
              st->red[R_CG] = combine_sum(cl, C, pub, R_CG);
              ctrl_phase(st, C_HTP_CG1, 0);
            }
            __syncthreads();
            const float alpha = st->cg_alpha;
            for (int c = tid; c < nc; c += RS_THREADS) x[c] = fmaf(alpha, grad[c], x[c]);
            at_own<DEEP>(A, lda, q4, c0, nc, r, gpt);  // x_thres = (A^T A grad_S) on the support
            __syncthreads();
            {
              const int kb = st->k_bin;
              float s3 = 0.0f;
              for (int c = tid; c < nc; c += RS_THREADS) {
                const float xtv = bins[c] > kb ? 0.0f : gpt[c];
                const float o = fmaf(-alpha, xtv, gp[c]);
                gp[c] = o;
                s3 = fmaf(o, o, s3);
              }
              const float b = block_reduce<0>(s3, red32);
              if (tid == 0) pub[R_DOT3] = b;
            }
            cl.sync();
            if (tid == 0) {
              st->red[R_DOT3] = combine_sum(cl, C, pub, R_DOT3);
              ctrl_phase(st, C_HTP_CG2, 0);
            }
            __syncthreads();
            {
              const float beta = st->cg_beta;
              for (int c = tid; c < nc; c += RS_THREADS) grad[c] = fmaf(1.0f, gp[c], beta * grad[c]);
            }
            av_rows(x, true, rowa, nullptr, R_RES);  // ||y - A x_S||^2
            if (tid == 0) {
              st->red[R_RES] = combine_sum(cl, C, pub, R_RES);
              ctrl_phase(st, C_HTP_CG3, 0);
            }
            __syncthreads();
          }
          if (tid == 0) ctrl_phase(st, C_HTP_STOP, 0);
        } else {
          if (tid == 0) ctrl_phase(st, C_NIHT_STOP, 0);
        }
        __syncthreads();
      }
      if (IS_CG) {
        // A v_S of the own support into an m-vector (2 cluster barriers): own rows into rows,
        // y - A v_S with sub_y; every row gathered into full when given; the CTA's partial of
        // the squared norm into pub[slot], combined by the caller before its next barrier
        auto av_rows = [&](const float *v, bool sub_y, float *rows, float *full, int slot) {
          av_own_partial(A, lda, q4, c0, sidx, s_own, v, part, gscr);
          if (tid == 0) ipub[0] = s_own;
          cl.sync();
          const float s2 = reduce_rows(cl, C, part, rr0, rr1, sub_y ? ypart : nullptr, rows, nullptr);
          const float b = block_reduce<0>(s2, red32);
          if (tid == 0 && slot >= 0) pub[slot] = b;
          cl.sync();
          if (full) gather_rows(cl, C, q4, RB, rows, full);
        };
        // prologue tail (GAGA/gaga/algorithms.cu:3776-3808): r0 = y - A x, grad_previous =
        // A^T r0, grad_prev_thres
        av_rows(x, true, rowp, r, R_RES);
        if (tid == 0) st->red[R_RES] = combine_sum(cl, C, pub, R_RES);
        __syncthreads();
        at_trial<DEEP>(st->gfmt, A, Ah, Al, lda, q4, c0, nc, r, gp);
        __syncthreads();
        {
          const int kb = st->k_bin;
          for (int c = tid; c < nc; c += RS_THREADS) gpt[c] = bins[c] <= kb ? gp[c] : 0.0f;
        }
        if (tid == 0) ctrl_phase(st, C_CGIHT_INIT, 0);
        __syncthreads();
        // ---- CGIHT iterations: RestrictedCGwithSupportEvolution (F_RCG,
        // GAGA/gaga/functions.cu:1004-1102) or UnrestrictedCG (F_UCG, :1107-1220), then
        // x += alpha p and the support (algorithms.cu:3849-3899)
        while (st->active) {
          const bool rcg = st->flags[F_RCG] != 0;
          if (st->flags[F_RESR]) {
            // r = r - alpha A p over the own rows (A p from the last restricted step), then
            // every CTA gathers the rows
            const float alpha = st->cg_alpha;
            float4 *rp4 = reinterpret_cast<float4 *>(rowp);
            const float4 *ra4 = reinterpret_cast<const float4 *>(rowa);
            float s2 = 0.0f;
            for (int i = tid; i < rr1 - rr0; i += RS_THREADS) {
              float4 v = rp4[i];
              const float4 a = ra4[i];
              v.x = fmaf(-alpha, a.x, v.x); v.y = fmaf(-alpha, a.y, v.y);
              v.z = fmaf(-alpha, a.z, v.z); v.w = fmaf(-alpha, a.w, v.w);
              rp4[i] = v;
              s2 = fmaf(v.x, v.x, s2); s2 = fmaf(v.y, v.y, s2); s2 = fmaf(v.z, v.z, s2); s2 = fmaf(v.w, v.w, s2);
            }
            const float b = block_reduce<0>(s2, red32);
            if (tid == 0) {
              pub[R_RES] = b;
              ipub[0] = s_own;
            }
            cl.sync();
            gather_rows(cl, C, q4, RB, rowp, r);
          } else if (rcg) {
            av_rows(x, true, rowp, r, R_RES);  // r = y - A x_S
          } else {
            // unrestricted step: r = y - A x_S and the own rows of A grad_prev_thres from one
            // pass over the support columns; the second partial sits in r, which the gather
            // overwrites only after the cluster barrier that ends the reads of it
            av_own_partial_t<2>(A, lda, q4, c0, sidx, s_own, x, gpt, part, r, gscr);
            if (tid == 0) ipub[0] = s_own;
            cl.sync();
            const float s2 = reduce_rows(cl, C, part, rr0, rr1, ypart, rowp, nullptr);
            reduce_rows(cl, C, r, rr0, rr1, nullptr, rowa, nullptr);
            const float b = block_reduce<0>(s2, red32);
            if (tid == 0) pub[R_RES] = b;
            cl.sync();
            gather_rows(cl, C, q4, RB, rowp, r);
          }
          if (tid == 0) {
            st->red[R_RES] = combine_sum(cl, C, pub, R_RES);
            int sc = 0;
            for (int c = 0; c < C; ++c) sc += peer(cl, ipub, c)[0];
            st->s_cnt = sc;
            ctrl_phase(st, C_PUSH_RES, 0);
          }
          __syncthreads();
          at_trial<DEEP>(st->gfmt, A, Ah, Al, lda, q4, c0, nc, r, grad);  // grad = A^T r; x_thres = grad on the support
          __syncthreads();
          const int kb = st->k_bin;
          float sxt = 0.0f;
          for (int c = tid; c < nc; c += RS_THREADS) {
            const float o = bins[c] <= kb ? grad[c] : 0.0f;
            sxt = fmaf(o, o, sxt);
          }
          if (rcg) {
            {
              const float b = block_reduce<0>(sxt, red32);
              if (tid == 0) pub[R_XT] = b;
            }
            cl.sync();
            if (tid == 0) {
              st->red[R_XT] = combine_sum(cl, C, pub, R_XT);
              ctrl_phase(st, C_RCG_BETA, 0);
            }
            __syncthreads();
            {
              const float beta = st->cg_beta;
              float gm = 0.0f;
              for (int c = tid; c < nc; c += RS_THREADS) {
                const float g = fmaf(1.0f, grad[c], beta * gp[c]);  // k_scale_add
                gp[c] = g;
                gpt[c] = bins[c] <= kb ? g : 0.0f;
                gm = fmaxf(gm, fabsf(g));
              }
              const float b = block_reduce<1>(gm, red32);
              if (tid == 0) pub[R_GMAX] = b;  // combined after the next product
            }
            av_rows(gpt, false, rowa, nullptr, R_AXT);  // ||A grad_prev_thres||^2
            if (tid == 0) {
              st->red[R_GMAX] = (double)combine_max(cl, C, pub, R_GMAX);
              st->red[R_AXT] = combine_sum(cl, C, pub, R_AXT);
              ctrl_phase(st, C_RCG_ALPHA, 0);
            }
            __syncthreads();
          } else {
            {
              const float b = block_reduce<0>(sxt, red32);
              if (tid == 0) pub[R_XT] = b;  // combined with the dot products below
            }
            // (the own rows of A grad_prev_thres came with the residual's pass)
            av_rows(grad, false, rowb, nullptr, -1);  // own rows of A x_thres
            {
              const float4 *a4 = reinterpret_cast<const float4 *>(rowa);
              const float4 *b4 = reinterpret_cast<const float4 *>(rowb);
              float d1 = 0.0f, d2 = 0.0f;
              for (int i = tid; i < rr1 - rr0; i += RS_THREADS) {
                const float4 a = a4[i], bb = b4[i];
                d1 = fmaf(a.x, bb.x, d1); d1 = fmaf(a.y, bb.y, d1); d1 = fmaf(a.z, bb.z, d1); d1 = fmaf(a.w, bb.w, d1);
                d2 = fmaf(a.x, a.x, d2); d2 = fmaf(a.y, a.y, d2); d2 = fmaf(a.z, a.z, d2); d2 = fmaf(a.w, a.w, d2);
              }
              const float b1 = block_reduce<0>(d1, red32);
              if (tid == 0) pub[R_DOT1] = b1;
              const float b2 = block_reduce<0>(d2, red32);
              if (tid == 0) pub[R_DOT2] = b2;
            }
            cl.sync();
            if (tid == 0) {
              st->red[R_XT] = combine_sum(cl, C, pub, R_XT);
              st->red[R_DOT1] = combine_sum(cl, C, pub, R_DOT1);
              st->red[R_DOT2] = combine_sum(cl, C, pub, R_DOT2);
              ctrl_phase(st, C_UCG_BETA, 0);
            }
            __syncthreads();
            {
              const float beta = st->cg_beta;
              float gm = 0.0f, d3 = 0.0f, d4 = 0.0f;
              for (int c = tid; c < nc; c += RS_THREADS) {
                const float g = fmaf(1.0f, grad[c], beta * gp[c]);  // k_scale_add
                gp[c] = g;
                const bool in = bins[c] <= kb;
                const float pt = in ? g : 0.0f;
                gpt[c] = pt;
                gm = fmaxf(gm, fabsf(g));
                d3 = fmaf(pt, in ? grad[c] : 0.0f, d3);  // <grad_prev_thres, x_thres>
              }
              float4 *a4 = reinterpret_cast<float4 *>(rowa);
              const float4 *b4 = reinterpret_cast<const float4 *>(rowb);
              for (int i = tid; i < rr1 - rr0; i += RS_THREADS) {  // A p = A x_thres + beta A p_prev
                float4 a = a4[i];
                const float4 bb = b4[i];
                a.x = fmaf(1.0f, bb.x, beta * a.x); a.y = fmaf(1.0f, bb.y, beta * a.y);
                a.z = fmaf(1.0f, bb.z, beta * a.z); a.w = fmaf(1.0f, bb.w, beta * a.w);
                a4[i] = a;
                d4 = fmaf(a.x, a.x, d4); d4 = fmaf(a.y, a.y, d4); d4 = fmaf(a.z, a.z, d4); d4 = fmaf(a.w, a.w, d4);
              }
              block_reduce_sum_max(d3, gm, red32, &pub[R_DOT3], &pub[R_GMAX]);
              const float b4s = block_reduce<0>(d4, red32);
              if (tid == 0) pub[R_DOT4] = b4s;
            }
            cl.sync();
            if (tid == 0) {
              st->red[R_DOT3] = combine_sum(cl, C, pub, R_DOT3);
              st->red[R_DOT4] = combine_sum(cl, C, pub, R_DOT4);
              st->red[R_GMAX] = (double)combine_max(cl, C, pub, R_GMAX);
              ctrl_phase(st, C_UCG_ALPHA, 0);
            }
            __syncthreads();
          }
          // x += alpha grad_previous ; max|x| ; counters cleared
          {
            const float alpha = st->cg_alpha;
            float mxx = 0.0f;
            for (int c = tid; c < nc; c += RS_THREADS) {
              const float o = fmaf(alpha, gp[c], x[c]);
              x[c] = o;
              mxx = fmaxf(mxx, fabsf(o));
            }
            for (int b = tid; b < L.nb_cap; b += RS_THREADS) cnt[b] = 0;
            const float b = block_reduce<1>(mxx, red32);
            if (tid == 0) pub[R_XMAX] = b;
          }
          cl.sync();
          if (tid == 0) {
            st->red[R_XMAX] = (double)combine_max(cl, C, pub, R_XMAX);
            ctrl_phase(st, C_CGIHT_BINDEC, 0);
            ctrl_phase(st, C_BINPREP, 0);
          }
          __syncthreads();
          support(true);
          if (tid == 0) ctrl_phase(st, C_CGIHT_POST, 0);
          __syncthreads();
          if (st->flags[F_REMASK]) {
            const int kb2 = st->k_bin;
            for (int c = tid; c < nc; c += RS_THREADS) gpt[c] = bins[c] <= kb2 ? gp[c] : 0.0f;
          }
          if (tid == 0) ctrl_phase(st, C_CGIHT_STOP, 0);
          __syncthreads();
        }
      }
      if (!(ALG == RS_CGIHT_ML && !P.single && attempt == 0 && st->fell_back)) break;
    }
    if (P.single) {
      // ---- x and the final state back to the caller's workspace
      for (int c = tid; c < nc; c += RS_THREADS) P.xg[c0 + c] = x[c];
      if (rank == 0 && tid == 0) {
        const unsigned int *src = reinterpret_cast<const unsigned int *>(st);
        unsigned int *dst = reinterpret_cast<unsigned int *>(P.st_io);
        for (int i = 0; i < (int)(sizeof(GbState) / 4); ++i) dst[i] = src[i];
      }
      continue;
    }
    // ---- verdict (k_b_err and the result phase of gb_batch.cu)
    {
      float e2 = 0.0f, x2 = 0.0f;
      for (int c = tid; c < nc; c += RS_THREADS) {
        const float d = x0[c] - x[c];
        e2 = fmaf(d, d, e2);
        x2 = fmaf(x0[c], x0[c], x2);
      }
      const float b1 = block_reduce<0>(e2, red32);
      if (tid == 0) pub[R_DOT1] = b1;
      const float b2 = block_reduce<0>(x2, red32);
      if (tid == 0) pub[R_DOT2] = b2;
    }
    cl.sync();
    if (rank == 0 && tid == 0) {
      const double e2 = combine_sum(cl, C, pub, R_DOT1), x2 = combine_sum(cl, C, pub, R_DOT2);
      const float rel = (float)(sqrt(e2) / sqrt(x2));
      P.iters[t] = warm_iters + st->iter;
      P.err[t] = rel;
      P.ok[t] = rel <= 1e-3f ? 1 : 0;
      if (P.fb) P.fb[t] = 0;  // an abandoned warm start was solved again above
      atomicAdd(P.bytes, warm_bytes + st->bytes);
    }
  }
  cl.sync();  // no CTA leaves while a peer may still read its shared memory
}

struct ResEngine {
  int dev = -1, n_cap = 0, m_cap = 0, C = 0, ncl = 0, t_cap = 0, gfmt = 0;
  size_t smem = 0, a_stride = 0;
  float *A = nullptr;
  unsigned short *Ah = nullptr;  // compact A^T r operand (gfmt != GB_GRAD_FP32)
  unsigned char *Al = nullptr;
  int *xhist = nullptr;
  int *order = nullptr, *queue = nullptr;
};
std::map<int, ResEngine> g_res;

void res_release(ResEngine &R) {
  if (R.A) cudaFree(R.A);
  if (R.Ah) cudaFree(R.Ah);
  if (R.Al) cudaFree(R.Al);
  if (R.xhist) cudaFree(R.xhist);
  if (R.order) cudaFree(R.order);
  R = ResEngine();
}

// the kernel instance for (single given-data solve or batched trials, algorithm), with its
// attributes set once per device: dynamic shared memory up to the opt-in maximum and
// clusters of up to 16 CTAs
using RsKernel = void (*)(const RsParams);
RsKernel rs_kernel(bool deep, int alg) {
  if (deep)
    return alg == RS_CGIHT_ML ? k_resident<true, RS_CGIHT_ML>
           : alg == RS_CGIHT  ? k_resident<true, RS_CGIHT>
           : alg == RS_HTP    ? k_resident<true, RS_HTP>
                              : k_resident<true, RS_NIHT>;
  return alg == RS_CGIHT_ML ? k_resident<false, RS_CGIHT_ML>
         : alg == RS_CGIHT  ? k_resident<false, RS_CGIHT>
         : alg == RS_HTP    ? k_resident<false, RS_HTP>
                            : k_resident<false, RS_NIHT>;
}
std::atomic<unsigned long long> g_attr_done[8];

}  // namespace

int gb_resident_max_smem();

static gb_status rs_attrs(bool deep, int alg) {
  const int cap = gb_resident_max_smem();
  return gb_once_per_device(g_attr_done[(deep ? 4 : 0) + alg], [&]() -> gb_status {
    const void *fn = (const void *)rs_kernel(deep, alg);
    GB_CUDA_TRY(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, cap));
    GB_CUDA_TRY(cudaFuncSetAttribute(fn, cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
    return GB_OK;
  });
}

// the resident algorithm of a library algorithm id (learned: CGIHT from the warm start)
int gb_resident_alg(int gb_alg, int learned) {
  if (gb_alg == GB_ALG_CGIHT) return learned ? RS_CGIHT_ML : RS_CGIHT;
  if (learned) return -1;
  return gb_alg == GB_ALG_NIHT ? RS_NIHT : gb_alg == GB_ALG_HTP ? RS_HTP : -1;
}

int gb_resident_max_smem() {
  int dev = 0, optin = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 0;
  if (cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess) return 0;
  cudaFuncAttributes fa;
  if (cudaFuncGetAttributes(&fa, (const void *)k_resident<false, RS_NIHT>) != cudaSuccess) return 0;
  return optin - (int)fa.sharedSizeBytes;
}

size_t gb_resident_smem(int n_cap, int m_cap, int C, int gb_alg, int learned) {
  return rs_layout(n_cap, m_cap, C, rs_default_bins(n_cap), gb_resident_alg(gb_alg, learned)).bytes;
}

int gb_resident_pick_cluster(int n_cap, int m_cap, int requested, int gb_alg, int learned) {
  const int cap = gb_resident_max_smem();
  if (m_cap > 8192 || n_cap > 20000 || cap <= 0 || gb_resident_alg(gb_alg, learned) < 0) return 0;
  auto fits = [&](int C) {
    return (long long)gb_resident_smem(n_cap, m_cap, C, gb_alg, learned) <= (long long)cap;
  };
  if (requested > 0) return (requested <= 16 && fits(requested)) ? requested : 0;
  // four CTAs per trial measured best over the sweep's mix (n = 1024 ... 8192) on GB300
  int C = 4;
  while (C < 16 && !fits(C)) C *= 2;
  return fits(C) ? C : 0;
}

gb_status gb_resident_enqueue(const GbResidentArgs &a, cudaStream_t s) {
  int dev = 0;
  GB_CUDA_TRY(cudaGetDevice(&dev));
  const int alg = gb_resident_alg(a.alg, a.ml_params != nullptr);
  const int C = gb_resident_pick_cluster(a.n_cap, a.m_cap, a.cluster, a.alg, a.ml_params != nullptr);
  if (C <= 0 || alg < 0) {
    gb_set_error_message("resident form: no cluster size fits the trial sizes", __FILE__, __LINE__);
    return GB_BAD_ARG;
  }
  GB_TRY(rs_attrs(false, alg));
  const RsKernel kern = rs_kernel(false, alg);
  ResEngine &R = g_res[dev * 4 + alg];
  const int learned = a.ml_params != nullptr;
  // the kernel lays out shared memory for the engine's capacities, which a reused engine can
  // have above this call's sizes: the launch provides that layout's size, and an engine whose
  // layout no longer fits is rebuilt for this call
  const bool reuse = R.dev == dev && R.n_cap >= a.n_cap && R.m_cap >= a.m_cap && R.C == C &&
                     R.t_cap >= a.count && R.gfmt == a.gfmt &&
                     (long long)gb_resident_smem(R.n_cap, R.m_cap, C, a.alg, learned) <= gb_resident_max_smem();
  const size_t smem = gb_resident_smem(a.n_cap, a.m_cap, C, a.alg, learned);
  cudaLaunchConfig_t cfg;
  memset(&cfg, 0, sizeof(cfg));
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = C;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.blockDim = dim3(RS_THREADS, 1, 1);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  if (!reuse) {
    res_release(R);
    int sms = 0;
    GB_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    cfg.gridDim = dim3(sms / C * C, 1, 1);
    int ncl = 0;
    GB_CUDA_TRY(cudaOccupancyMaxActiveClusters(&ncl, (void *)kern, &cfg));
    if (ncl <= 0) {
      gb_set_error_message("resident form: no cluster can be resident", __FILE__, __LINE__);
      return GB_CUDA_ERROR;
    }
    const size_t a_stride = (size_t)((a.m_cap + 31) / 32 * 32) * a.n_cap;
    size_t free_b = 0, total_b = 0;
    GB_CUDA_TRY(cudaMemGetInfo(&free_b, &total_b));
    const double eb = 4.0 + (a.gfmt == GB_GRAD_A24 ? 3.0 : a.gfmt == GB_GRAD_BF16 ? 2.0 : 0.0);
    while (ncl > 1 && (double)ncl * a_stride * eb > 0.5 * (double)free_b) ncl--;
    R.dev = dev;
    R.gfmt = a.gfmt;
    R.n_cap = a.n_cap;
    R.m_cap = a.m_cap;
    R.C = C;
    R.ncl = ncl;
    R.smem = smem;
    R.a_stride = a_stride;
    R.t_cap = std::max(a.count, 1024);
    GB_CUDA_TRY(cudaMalloc(&R.A, (size_t)ncl * a_stride * 4));
    if (a.gfmt != GB_GRAD_FP32) GB_CUDA_TRY(cudaMalloc(&R.Ah, (size_t)ncl * a_stride * 2));
    if (a.gfmt == GB_GRAD_A24) GB_CUDA_TRY(cudaMalloc(&R.Al, (size_t)ncl * a_stride));
    GB_CUDA_TRY(cudaMalloc(&R.xhist, (size_t)ncl * a.n_cap * 4));
    GB_CUDA_TRY(cudaMalloc(&R.order, (size_t)(R.t_cap + 64) * 4));
    R.queue = R.order + R.t_cap;
  }
  GB_CUDA_TRY(cudaMemcpyAsync(R.order, a.order, (size_t)a.count * 4, cudaMemcpyHostToDevice, s));
  GB_CUDA_TRY(cudaMemsetAsync(R.queue, 0, 4, s));
  RsParams P;
  P.T = a.count;
  P.seed = a.seed;
  P.tol_rel = a.tol_rel;
  P.maxiter = a.maxiter;
  P.n = a.n;
  P.m = a.m;
  P.k = a.k;
  P.tid = a.tid;
  P.order = R.order;
  P.queue = R.queue;
  P.iters = a.iters;
  P.err = a.err;
  P.ok = a.ok;
  P.bytes = a.bytes;
  P.A = R.A;
  P.a_stride = R.a_stride;
  P.xhist = R.xhist;
  P.n_cap = R.n_cap;
  P.m_cap = R.m_cap;
  P.nb_cap = rs_default_bins(R.n_cap);
  P.single = 0;
  P.Ag = nullptr;
  P.lda_u = 0;
  P.yg = nullptr;
  P.xg = nullptr;
  P.st_io = nullptr;
  P.ml_params = a.ml_params;
  P.fb = a.fb;
  P.gfmt = a.gfmt;
  P.gfmts = a.gfmts;
  P.Ah = R.Ah;
  P.Al = R.Al;
  P.rec_every = a.rec_every;
  cfg.gridDim = dim3(R.ncl * C, 1, 1);
  cfg.dynamicSmemBytes = gb_resident_smem(R.n_cap, R.m_cap, C, a.alg, learned);
  GB_CUDA_TRY(cudaLaunchKernelEx(&cfg, kern, P));
  return GB_OK;
}

int gb_resident_last_cluster() {
  std::lock_guard<std::recursive_mutex> lock(gb_batch_mutex());
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 0;
  auto it = g_res.find(dev);
  return it == g_res.end() ? 0 : it->second.C;
}

// The drop-in's dense NIHT, HTP or CGIHT on one cluster (the caller checked that no timing
// variant is asked for; with w.ml_params CGIHT runs the learned warm-start instance).  The cluster takes up to 16 CTAs with at
// least 128 columns each; *used = 0 when the problem does not fit (the graph path solves it).
gb_status gb_resident_solve_single(GbWork &w, int gb_alg, int num_bins, cudaStream_t s, int *used) {
  *used = 0;
  const int alg = gb_resident_alg(gb_alg, w.ml_params != nullptr);
  if (alg < 0) return GB_OK;
  const GbOp &op = w.op;
  if (op.kind != GB_OP_DENSE || !op.vec4 || (op.m % 4) || op.m > 8192 || op.n > 20000 || w.dyn) return GB_OK;
  // 16 SMs stream a 48 MB matrix in about the time the per-step kernels take over the whole
  // GPU; larger ones are faster there
  if (4.0 * op.m * op.n > 48e6) return GB_OK;
  const int cap = gb_resident_max_smem();
  if (cap <= 0) return GB_OK;
  GB_TRY(rs_attrs(true, alg));
  const RsKernel kern = rs_kernel(true, alg);
  cudaLaunchConfig_t cfg;
  memset(&cfg, 0, sizeof(cfg));
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.blockDim = dim3(RS_THREADS, 1, 1);
  cfg.stream = s;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  // up to 16 CTAs with at least 128 columns each, halved while the GPU cannot place such a
  // cluster; fewer CTAs need more shared memory each, so a size that does not fit ends it
  int C = 16;
  while (C > 1 && op.n / C < 128) C /= 2;
  if (const char *e = getenv("GB_CS_SINGLE_CLUSTER")) C = std::max(1, std::min(16, atoi(e)));
  for (;;) {
    const size_t smem = rs_layout(op.n, op.m, C, num_bins, alg).bytes;
    if ((long long)smem > cap) return GB_OK;
    attr[0].val.clusterDim.x = C;
    cfg.gridDim = dim3(C, 1, 1);
    cfg.dynamicSmemBytes = smem;
    int ncl = 0;
    if (cudaOccupancyMaxActiveClusters(&ncl, (void *)kern, &cfg) == cudaSuccess && ncl > 0) break;
    cudaGetLastError();
    if (C == 1) return GB_OK;
    C /= 2;
  }
  RsParams P;
  memset(&P, 0, sizeof(P));
  P.T = 1;
  P.n_cap = op.n;
  P.m_cap = op.m;
  P.nb_cap = num_bins;
  P.single = 1;
  P.Ag = op.A;
  P.lda_u = op.lda;
  P.yg = w.y;
  P.xg = w.x;
  P.st_io = w.st;
  P.ml_params = w.ml_params;
  GB_CUDA_TRY(cudaLaunchKernelEx(&cfg, kern, P));
  *used = 1;
  return GB_OK;
}

gb_status gb_resident_check() {
  int v = 0;
  GB_CUDA_TRY(cudaMemcpyFromSymbol(&v, g_rs_guard, sizeof(int)));
  if (v) {
    const int zero = 0;
    cudaMemcpyToSymbol(g_rs_guard, &zero, sizeof(int));
    gb_set_error_message("resident kernel launched with less shared memory than its layout", __FILE__, __LINE__);
    return GB_CUDA_ERROR;
  }
  return GB_OK;
}

