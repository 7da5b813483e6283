// gb_gemm.cu -- BF16 "TN" GEMM with FP32 accumulation for the shared-matrix batched form.
//
//     Ct[N x M] = [Y -] (A[M x K] . B[N x K]^T)^T
//
// A and B are K-major (row-major with K contiguous), the output is written transposed
// (one contiguous vector of M values per column n = per trial), optionally as Y - A B^T
// and optionally also as BF16.  In the shared-matrix form A is the measurement matrix
// (or its transpose) and B holds one trial's vector per row.
//
// This file holds the warp-level tensor-core kernel (mma.sync m16n8k16, 3-stage cp.async
// pipeline, 128x128x32 CTA tile) and the dispatch.  The mma.sync kernel is the baseline the
// tcgen05 kernel (gb_gemm_tc.cu) is validated against; gb_gemm runs the tcgen05 kernel
// whenever the shape allows (N % 256, K % 64) unless GB_CS_GEMM=mma.
#include <cuda_bf16.h>

#include <stdlib.h>
#include <string.h>

#include "gb_internal.cuh"

#define GT_M 128
#define GT_N 128
#define GT_K 32
#define GT_STAGES 3
#define GT_LD (GT_K + 8)  // padded row (halves) to avoid ldmatrix bank conflicts

__device__ __forceinline__ void cp_async16(void *smem, const void *gmem) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(s), "l"(gmem));
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;" ::"n"(N));
}

__device__ __forceinline__ void ldmatrix_x4(unsigned &r0, unsigned &r1, unsigned &r2, unsigned &r3, const void *p) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(p);
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];"
               : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3)
               : "r"(s));
}

__device__ __forceinline__ void mma_bf16(float *d, const unsigned *a, const unsigned *b) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

// M % 128 == 0, N % 128 == 0, K % 32 == 0 (the caller pads).
// Grid: x = M/128 row tiles; y = (N/128 column tiles) x s_max K splits.  With a column map
// the live column count is read on the device, tiles past it exit at once, and the K
// split S is chosen from the live tile count so that about two CTAs per SM run; partial
// tiles then go to a workspace and the last CTA of a tile to arrive sums them in split
// order (deterministic) and runs the epilogue.
__global__ void __launch_bounds__(256) k_gemm_tn_mma(GbGemm g, GbGemmWs ws, int s_max) {
  extern __shared__ __align__(16) __nv_bfloat16 gsm[];
  __nv_bfloat16 *As = gsm;                                  // [stage][128][GT_LD]
  __nv_bfloat16 *Bs = gsm + GT_STAGES * GT_M * GT_LD;       // [stage][128][GT_LD]
  const __nv_bfloat16 *__restrict__ A = (const __nv_bfloat16 *)g.A;
  const __nv_bfloat16 *__restrict__ B = (const __nv_bfloat16 *)g.B;
  const int M = g.M, lda = g.lda, ldb = g.ldb;
  const int *__restrict__ nmap = g.nmap;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int wm = warp >> 2, wn = warp & 3;  // 2 x 4 warps, warp tile 64 x 32
  const int mt = blockIdx.x, mtiles = gridDim.x;
  const int nti = blockIdx.y / s_max, sp = blockIdx.y % s_max;
  const int m0 = mt * GT_M, n0 = nti * GT_N;
  const int nk = g.K / GT_K;
  // with a column map, tile columns c < *ncount are B rows / Ct columns nmap[c]
  const int cnt = g.ncount ? *g.ncount : g.N;
  if (n0 >= cnt) return;
  int S = 1;
  if (s_max > 1) {
    const int tiles = mtiles * ((cnt + GT_N - 1) / GT_N);
    S = max(1, min(min(s_max, nk), (2 * ws.num_sms) / tiles));
    if (S * tiles > ws.part_tiles) S = 1;
  }
  if (sp >= S) return;
  const int kb = (int)((long long)sp * nk / S), ke = (int)((long long)(sp + 1) * nk / S);
  const int br0 = nmap ? nmap[min(n0 + (tid >> 2), cnt - 1)] : n0 + (tid >> 2);
  const int br1 = nmap ? nmap[min(n0 + (tid >> 2) + 64, cnt - 1)] : n0 + (tid >> 2) + 64;
  float acc[4][4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[i][j][0] = acc[i][j][1] = acc[i][j][2] = acc[i][j][3] = 0.0f;

  auto load_stage = [&](int st, int kt) {
    const int k0 = kt * GT_K;
#pragma unroll
    for (int c = 0; c < 2; ++c) {
      const int q = tid + c * 256;  // 512 chunks of 16 bytes per operand
      const int row = q >> 2, col = (q & 3) * 8;
      cp_async16(As + (st * GT_M + row) * GT_LD + col, A + (size_t)(m0 + row) * lda + k0 + col);
      cp_async16(Bs + (st * GT_N + row) * GT_LD + col, B + (size_t)(c ? br1 : br0) * ldb + k0 + col);
    }
  };

  const int nkl = ke - kb;
  for (int s = 0; s < GT_STAGES - 1; ++s) {
    if (s < nkl) load_stage(s, kb + s);
    cp_async_commit();
  }
  for (int it = 0; it < nkl; ++it) {
    cp_async_wait<GT_STAGES - 2>();
    __syncthreads();
    const int nxt = it + GT_STAGES - 1;
    if (nxt < nkl) load_stage(nxt % GT_STAGES, kb + nxt);
    cp_async_commit();
    const int st = it % GT_STAGES;
    const __nv_bfloat16 *as = As + st * GT_M * GT_LD;
    const __nv_bfloat16 *bs = Bs + st * GT_N * GT_LD;
#pragma unroll
    for (int kk = 0; kk < GT_K; kk += 16) {
      unsigned af[4][4], bf[4][2];
#pragma unroll
      for (int mi = 0; mi < 4; ++mi) {
        const int r = wm * 64 + mi * 16 + (lane & 15);
        const int c = kk + (lane >> 4) * 8;
        ldmatrix_x4(af[mi][0], af[mi][1], af[mi][2], af[mi][3], as + r * GT_LD + c);
      }
#pragma unroll
      for (int nj = 0; nj < 2; ++nj) {
        const int r = wn * 32 + nj * 16 + (lane & 7) + ((lane >> 4) << 3);
        const int c = kk + ((lane >> 3) & 1) * 8;
        unsigned r0, r1, r2, r3;
        ldmatrix_x4(r0, r1, r2, r3, bs + r * GT_LD + c);
        bf[2 * nj][0] = r0;
        bf[2 * nj][1] = r1;
        bf[2 * nj + 1][0] = r2;
        bf[2 * nj + 1][1] = r3;
      }
#pragma unroll
      for (int mi = 0; mi < 4; ++mi)
#pragma unroll
        for (int ni = 0; ni < 4; ++ni) mma_bf16(acc[mi][ni], af[mi], bf[ni]);
    }
  }
  cp_async_wait<0>();
  if (S > 1) {
    // publish this split's partial tile (fragment-major: element e of thread tid at e*256+tid)
    __shared__ int last;
    float *mine = ws.part + ((size_t)(nti * S + sp) * mtiles + mt) * (GT_M * GT_N);
#pragma unroll
    for (int mi = 0; mi < 4; ++mi)
#pragma unroll
      for (int ni = 0; ni < 4; ++ni)
#pragma unroll
        for (int e = 0; e < 4; ++e) __stcg(mine + ((mi * 4 + ni) * 4 + e) * 256 + tid, acc[mi][ni][e]);
    __threadfence();
    __syncthreads();
    if (tid == 0) last = atomicAdd(&ws.tickets[nti * mtiles + mt], 1u) == (unsigned)(S - 1);
    __syncthreads();
    if (!last) return;
    __threadfence();
#pragma unroll
    for (int mi = 0; mi < 4; ++mi)
#pragma unroll
      for (int ni = 0; ni < 4; ++ni)
#pragma unroll
        for (int e = 0; e < 4; ++e) acc[mi][ni][e] = 0.0f;
    for (int s2 = 0; s2 < S; ++s2) {
      const float *src = ws.part + ((size_t)(nti * S + s2) * mtiles + mt) * (GT_M * GT_N);
#pragma unroll
      for (int mi = 0; mi < 4; ++mi)
#pragma unroll
        for (int ni = 0; ni < 4; ++ni)
#pragma unroll
          for (int e = 0; e < 4; ++e) acc[mi][ni][e] += __ldcg(src + ((mi * 4 + ni) * 4 + e) * 256 + tid);
    }
    if (tid == 0) ws.tickets[nti * mtiles + mt] = 0u;
  }
  // epilogue: element (row, col) of C goes to Ct[col * M + row]
  const int gq = lane >> 2, tq = lane & 3;
  __nv_bfloat16 *Cb = (__nv_bfloat16 *)g.Cb;
#pragma unroll
  for (int mi = 0; mi < 4; ++mi)
#pragma unroll
    for (int ni = 0; ni < 4; ++ni)
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        const int row = m0 + wm * 64 + mi * 16 + gq + (e >> 1) * 8;
        int col = n0 + wn * 32 + ni * 8 + tq * 2 + (e & 1);
        if (col >= cnt) continue;
        if (nmap) col = nmap[col];
        const size_t o = (size_t)col * M + row;
        const float v = g.Y ? g.Y[o] - acc[mi][ni][e] : acc[mi][ni][e];
        g.Ct[o] = v;
        if (Cb) {
          const __nv_bfloat16 hi = __float2bfloat16_rn(v);
          if (g.cb_split) {  // column of 3M: [hi ; hi ; lo]
            const size_t q = (size_t)col * 3 * M + row;
            Cb[q] = hi;
            Cb[q + M] = hi;
            Cb[q + 2 * (size_t)M] = __float2bfloat16_rn(v - __bfloat162float(hi));
          } else {
            Cb[o] = hi;
          }
        }
      }
}

int gb_gemm_use_tc() {
  const char *e = getenv("GB_CS_GEMM");
  return !(e && strcmp(e, "mma") == 0);
}

gb_status gb_gemm(const GbGemm &g, cudaStream_t s) {
  if (g.M % GT_M || g.N % GT_N || g.K % GT_K || g.M <= 0 || g.N <= 0 || g.K <= 0 || g.lda < g.K || g.ldb < g.K ||
      g.lda % 8 || g.ldb % 8) {
    gb_set_error_message("GEMM sizes must be multiples of 128 (M, N) and 32 (K); strides multiples of 8", __FILE__,
                         __LINE__);
    return GB_BAD_ARG;
  }
  const bool aligned = ((uintptr_t)g.A & 15) == 0 && ((uintptr_t)g.B & 15) == 0;
  if (gb_gemm_use_tc() && g.N % 256 == 0 && g.K % 64 == 0 && aligned &&
      (!g.nmap || (g.ws && g.ws->gather)))
    return gb_gemm_tc(g, s);
  GbGemmWs ws = {};
  int s_max = 1;
  if (g.ws && g.ws->part && g.ws->tickets && (g.M / GT_M) * (g.N / GT_N) <= g.ws->ticket_count) {
    ws = *g.ws;
    s_max = GB_GEMM_SPLIT_MAX;
  }
  const int smem = GT_STAGES * (GT_M + GT_N) * GT_LD * 2;
  static std::atomic<unsigned long long> attr_done{0};
  GB_TRY(gb_once_per_device(attr_done, [&]() -> gb_status {
    GB_CUDA_TRY(cudaFuncSetAttribute(k_gemm_tn_mma, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
    return GB_OK;
  }));
  dim3 grid(g.M / GT_M, (g.N / GT_N) * s_max);
  k_gemm_tn_mma<<<grid, 256, smem, s>>>(g, ws, s_max);
  GB_CUDA_TRY(cudaGetLastError());
  return GB_OK;
}

extern "C" gb_status gb_cs_gemm_bf16_tn(const void *d_A, const void *d_B, float *d_Ct, int M, int N, int K,
                                        const float *d_Y, void *d_Cb, void *stream) {
  if (!d_A || !d_B || !d_Ct) {
    gb_set_error_message("gb_cs_gemm_bf16_tn: null buffer", __FILE__, __LINE__);
    return GB_BAD_ARG;
  }
  GbGemm g = {};
  g.A = d_A; g.B = d_B; g.Ct = d_Ct; g.M = M; g.N = N; g.K = K; g.lda = K; g.ldb = K; g.Y = d_Y; g.Cb = d_Cb;
  return gb_gemm(g, (cudaStream_t)stream);
}
