// gb_gemm_tc.cu -- the shared-matrix GEMM on the 5th-generation tensor cores (tcgen05).
//
//     Ct[N x M] = [Y -] (A[M x K] . B[N x K]^T)^T        A, B BF16, K-major; FP32 accumulate
//
// Two instances of one kernel, each CTA holding a 128 x 256 tile of C (M x N) in tensor memory:
//   pair (M % 256 == 0, the default): a cluster of two CTAs computes a 256 x 256 tile with
//               tcgen05.mma.cta_group::2 (M = 256, N = 256, K = 16).  Each CTA stages its
//               own 128 rows of A and one half (128 rows) of the B tile, 32 KB per k-block,
//               in a 7-stage ring; both CTAs' copies complete on the even CTA's stage
//               barrier, the even CTA issues the MMAs and its commits arrive on both CTAs'
//               barriers (multicast).  Per k-block an SM receives 32 KB instead of 48 KB.
//   single:     one CTA, tcgen05.mma.cta_group::1 (M = 128, N = 256), 128 x 64 (A) and
//               256 x 64 (B) boxes in a 4-stage ring of 48 KB stages.
// With a column map, a tile whose live columns number at most 64 (128) issues MMAs of
// N = 64 (128): the pair's CTAs load B from the tile's first column plus half that width,
// and the epilogue reads that many TMEM columns.
// Roles in each CTA:
//   warp 0      TMA producer: 128B-swizzled boxes into the ring, completion counted on a
//               per-stage mbarrier (expect_tx by the issuing CTA of the MMAs)
//   warp 1      allocates 256 TMEM columns; one elected lane issues the MMAs (4 per stage)
//               and frees each stage with tcgen05.commit
//   warps 2-5   epilogue: tcgen05.ld of their TMEM lane quarter (32 rows each), FP32
//               [Y -] epilogue, optional BF16 / split-BF16 copies, or a split-K partial
// Every mbarrier wait is bounded by the global timer; on a timeout the CTA records an
// error word, drains what it issued and returns, so a fault never hangs the GPU.
//
// With a column map (the active trials of the batched form) the live B rows are first
// gathered into a contiguous buffer, so the TMA boxes stay plain tiles; the epilogue
// writes column c to Ct column nmap[c].
#include <cuda.h>
#include <cuda_bf16.h>
#include <cudaTypedefs.h>

#include <cstdlib>
#include <mutex>

#include "gb_internal.cuh"

#define TC_BM 128  // rows of C per CTA
#define TC_BN 256  // columns of C per tile
#define TC_BK 64   // 64 BF16 = 128 bytes = one swizzle row
#define TC_THREADS 192  // producer, MMA issuer, four epilogue warps
#define TC_EPI_THREADS 128
#define TC_A_BYTES (TC_BM * TC_BK * 2)
#define TC_TMEM_COLS 256

// ring geometry of the two instances (PAIR: B rows per CTA are half the tile's columns)
template <int PAIR>
struct TcCfg {
  static constexpr int B_ROWS = PAIR ? TC_BN / 2 : TC_BN;
  static constexpr int STAGES = PAIR ? 7 : 4;
  static constexpr int B_BYTES = B_ROWS * TC_BK * 2;
  static constexpr int STAGE_BYTES = TC_A_BYTES + B_BYTES;
  static constexpr int SMEM = STAGES * STAGE_BYTES + 1024;
};
static_assert(TcCfg<1>::SMEM <= 230400, "pair ring must fit 227 KB with the static barriers");
#define TC_WAIT_NS 4000000000ull  // 4 s: far beyond any wait of a correct launch

__device__ int g_tc_error = 0;  // first failure code of any tcgen05 GEMM launch

namespace {

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ uint64_t global_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}

__device__ __forceinline__ bool mbar_test(uint64_t *bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// Wait for the phase with the given parity; false on timeout or when another role of the
// CTA has already given up (abort flag), after recording `code`.
__device__ bool mbar_wait(uint64_t *bar, uint32_t parity, volatile int *abort_flag, int code) {
  const uint64_t t0 = global_ns();
  for (uint32_t i = 0;; ++i) {
    if (mbar_test(bar, parity)) return true;
    if ((i & 63) == 63) {
      if (*abort_flag) return false;
      if (global_ns() - t0 > TC_WAIT_NS) {
        *abort_flag = 1;
        atomicCAS(&g_tc_error, 0, code);
        return false;
      }
    }
  }
}

__device__ __forceinline__ void tma_load_2d(void *dst, const CUtensorMap *map, uint64_t *bar, int x, int y) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4}], [%2];" ::
          "r"(smem_u32(dst)),
      "l"((uint64_t)map), "r"(smem_u32(bar)), "r"(x), "r"(y)
      : "memory");
}

// The pair form: the box lands in this CTA's shared memory, its bytes complete on the mbarrier
// at cluster address bar_cluster (the even CTA's stage barrier)
__device__ __forceinline__ void tma_load_2d_pair(void *dst, const CUtensorMap *map, uint32_t bar_cluster, int x,
                                                 int y) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes.cta_group::2 [%0], [%1, {%3, "
      "%4}], [%2];" ::"r"(smem_u32(dst)),
      "l"((uint64_t)map), "r"(bar_cluster), "r"(x), "r"(y)
      : "memory");
}

// shared::cluster address of the same shared-memory location in cluster CTA `rank`
__device__ __forceinline__ uint32_t cluster_addr(const void *p, uint32_t rank) {
  uint32_t r;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(smem_u32(p)), "r"(rank));
  return r;
}

__device__ __forceinline__ uint32_t cluster_rank() {
  uint32_t r;
  asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
  return r;
}

__device__ __forceinline__ void cluster_sync_all() {
  asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}

// Shared-memory matrix descriptor: K-major operand, 128-byte swizzle, 8-row groups 1024 B
// apart (the layout the TMA boxes above produce).
__device__ __forceinline__ uint64_t sw128_desc(uint32_t saddr) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr & 0x3FFFFu) >> 4);  // start address
  d |= (uint64_t)1 << 16;                    // leading byte offset (unused for swizzled K-major)
  d |= (uint64_t)(1024 >> 4) << 32;          // stride byte offset: next 8-row group
  d |= (uint64_t)1 << 46;                    // descriptor version
  d |= (uint64_t)2 << 61;                    // 128-byte swizzle
  return d;
}

// Instruction descriptor, kind::f16: D FP32, A and B BF16, both K-major, M = 128 per CTA (256
// for the pair), N = n columns (64, 128 or 256: a multiple of 16 for either M)
template <int PAIR>
__host__ __device__ constexpr uint32_t tc_idesc(int n) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) |
         ((uint32_t)((TC_BM << PAIR) >> 4) << 24);
}

template <int PAIR>
__device__ __forceinline__ void umma(uint32_t tmem_d, uint64_t da, uint64_t db, uint32_t idesc, uint32_t accumulate) {
  if constexpr (PAIR) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::2.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem_d),
        "l"(da), "l"(db), "r"(idesc), "r"(accumulate)
        : "memory");
  } else {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem_d),
        "l"(da), "l"(db), "r"(idesc), "r"(accumulate)
        : "memory");
  }
}

// arrive on `bar` once the MMAs issued so far complete; the pair form arrives on the barrier at
// the same offset in both CTAs
template <int PAIR>
__device__ __forceinline__ void umma_commit(uint64_t *bar) {
  if constexpr (PAIR) {
    asm volatile(
        "tcgen05.commit.cta_group::2.mbarrier::arrive::one.shared::cluster.multicast::cluster.b64 [%0], %1;" ::"r"(
            smem_u32(bar)),
        "h"((uint16_t)3)
        : "memory");
  } else {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
                 : "memory");
  }
}

template <int PAIR>
__device__ __forceinline__ void tmem_alloc(uint32_t *dst) {
  if constexpr (PAIR) {
    asm volatile("tcgen05.alloc.cta_group::2.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(dst)),
                 "r"(TC_TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::2.sync.aligned;" ::: "memory");
  } else {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(dst)),
                 "r"(TC_TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
}

template <int PAIR>
__device__ __forceinline__ void tmem_dealloc(uint32_t tmem) {
  if constexpr (PAIR)
    asm volatile("tcgen05.dealloc.cta_group::2.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TC_TMEM_COLS) : "memory");
  else
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TC_TMEM_COLS) : "memory");
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// 32 consecutive TMEM columns of this warp's 32 lanes: v[j] = column col + j of lane (row)
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float *v) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
      "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
      "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
        "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
        "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int j = 0; j < 32; ++j) v[j] = __uint_as_float(r[j]);
}

__device__ __forceinline__ void epi_bar() { asm volatile("bar.sync 1, %0;" ::"n"(TC_EPI_THREADS) : "memory"); }

struct TcArgs {
  float *Ct;
  int M, N, K;
  const float *Y;
  __nv_bfloat16 *Cb;
  int cb_split;
  const int *nmap, *ncount;
  int s_max;
  int split_rows;
  GbGemmWs ws;
};

template <int PAIR>
__global__ void __launch_bounds__(TC_THREADS, 1)
    k_gemm_tn_tc(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB, TcArgs a) {
  using Cfg = TcCfg<PAIR>;
  constexpr int STAGES = Cfg::STAGES;
  extern __shared__ uint8_t tc_smem_raw[];
  __shared__ __align__(8) uint64_t full_bar[STAGES], empty_bar[STAGES], accum_bar;
  __shared__ uint32_t tmem_base_sh;
  __shared__ int abort_sh, last_sh;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int mtiles = gridDim.x, mt = blockIdx.x;
  const int nti = blockIdx.y / a.s_max, sp = blockIdx.y % a.s_max;
  const int m0 = mt * TC_BM, n0 = nti * TC_BN;
  const int nkb = a.K / TC_BK;
  const int cnt = a.ncount ? *a.ncount : a.N;
  // the pair's two CTAs share blockIdx.y, so they return (or not) together here and below
  if (n0 >= cnt) return;
  const uint32_t rank = PAIR ? cluster_rank() : 0u;  // 0: this CTA issues the MMAs
  int S = 1;
  if (a.s_max > 1) {
    const int tiles = mtiles * ((cnt + TC_BN - 1) / TC_BN);
    S = max(1, min(min(a.s_max, nkb), a.ws.num_sms / (a.split_rows ? mtiles : tiles)));
    if (S * tiles * 2 > a.ws.part_tiles) S = 1;  // a 128 x 256 partial is two 128 x 128 units
  }
  if (sp >= S) return;
  const int kb0 = (int)((long long)sp * nkb / S), kb1 = (int)((long long)(sp + 1) * nkb / S);
  const int nk = kb1 - kb0;
  // MMA width: the tile's live columns rounded up to 64, 128 or 256 (a column map's few live
  // trials do not pay for a full 256-column product); the pair's two CTAs each hold half of
  // those columns' B rows at the start of their B buffer
  const int live = min(TC_BN, cnt - n0);
  const int nrt = live <= 64 ? 64 : live <= 128 ? 128 : TC_BN;

  uint8_t *smem = (uint8_t *)(((uintptr_t)tc_smem_raw + 1023) & ~(uintptr_t)1023);
  if (threadIdx.x == 0) {
    for (int s = 0; s < STAGES; ++s) {
      mbar_init(&full_bar[s], 1);
      mbar_init(&empty_bar[s], 1);
    }
    mbar_init(&accum_bar, 1);
    abort_sh = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) tmem_alloc<PAIR>(&tmem_base_sh);
  tc_fence_before();
  // the pair: the odd CTA's copies complete on the even CTA's barriers, initialised above
  if constexpr (PAIR)
    cluster_sync_all();
  else
    __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tmem_base_sh;
  volatile int *abort_flag = &abort_sh;

  if (warp == 0) {
    // ---------------------------------------------------------------- TMA producer
    if (lane == 0) {
      int issued = 0;
      const int b_row = n0 + (int)rank * (nrt / 2);  // the pair: B rows of this CTA's half
      for (int it = 0; it < nk; ++it) {
        const int s = it % STAGES;
        const uint32_t ph = (uint32_t)(it / STAGES) & 1u;
        if (it >= STAGES && !mbar_wait(&empty_bar[s], ph ^ 1u, abort_flag, 1)) break;
        uint8_t *sa = smem + s * Cfg::STAGE_BYTES;
        const int kx = (kb0 + it) * TC_BK;
        if constexpr (PAIR) {
          if (rank == 0) mbar_expect_tx(&full_bar[s], 2 * Cfg::STAGE_BYTES);
          const uint32_t bar0 = cluster_addr(&full_bar[s], 0);
          tma_load_2d_pair(sa, &tmA, bar0, kx, m0);
          tma_load_2d_pair(sa + TC_A_BYTES, &tmB, bar0, kx, b_row);
        } else {
          mbar_expect_tx(&full_bar[s], Cfg::STAGE_BYTES);
          tma_load_2d(sa, &tmA, &full_bar[s], kx, m0);
          tma_load_2d(sa + TC_A_BYTES, &tmB, &full_bar[s], kx, b_row);
        }
        issued = it + 1;
      }
      // on an abort, wait (bounded) for the copies still in flight into the ring; the odd CTA
      // of a pair has no barrier of its own for them and waits a fixed 1 ms instead
      if (*abort_flag) {
        if (PAIR && rank != 0) {
          const uint64_t t0 = global_ns();
          while (global_ns() - t0 < 1000000ull) {
          }
        } else {
          for (int it = max(0, issued - STAGES); it < issued; ++it) {
            const uint64_t t0 = global_ns();
            while (!mbar_test(&full_bar[it % STAGES], (uint32_t)(it / STAGES) & 1u) && global_ns() - t0 < TC_WAIT_NS) {
            }
          }
        }
      }
    }
  } else if (warp == 1) {
    // ---------------------------------------------------------------- MMA issuer
    // (the pair: the even CTA only; its MMAs read both CTAs' stages at the same offsets)
    if (lane == 0 && rank == 0) {
      for (int it = 0; it < nk; ++it) {
        const int s = it % STAGES;
        const uint32_t ph = (uint32_t)(it / STAGES) & 1u;
        if (!mbar_wait(&full_bar[s], ph, abort_flag, 2)) break;
        tc_fence_after();
        const uint32_t sa = smem_u32(smem + s * Cfg::STAGE_BYTES);
        const uint64_t da = sw128_desc(sa), db = sw128_desc(sa + TC_A_BYTES);
        const uint32_t idesc = tc_idesc<PAIR>(nrt);
#pragma unroll
        for (int k = 0; k < TC_BK / 16; ++k)  // 16 BF16 = 32 bytes = +2 in the descriptor
          umma<PAIR>(tmem, da + 2 * k, db + 2 * k, idesc, (it | k) != 0 ? 1u : 0u);
        umma_commit<PAIR>(&empty_bar[s]);
      }
      umma_commit<PAIR>(&accum_bar);  // also on an abort: completes once every issued MMA has
    }
  } else {
    // ---------------------------------------------------------------- epilogue (warps 2-5)
    const int q = warp & 3;  // TMEM lane quarter this warp may access
    const int row = m0 + 32 * q + lane;
    mbar_wait(&accum_bar, 0, abort_flag, 3);
    epi_bar();
    const bool ok = *abort_flag == 0;  // uniform over the epilogue warps
    tc_fence_after();
    const uint32_t taddr = tmem + ((uint32_t)(32 * q) << 16);
    bool do_store = ok;
    float *part = nullptr;
    if (ok && S > 1) {
      // publish this split's partial tile: element (row r, column c) at c * 128 + r
      part = a.ws.part + ((size_t)(nti * S + sp) * mtiles + mt) * (TC_BM * TC_BN);
      for (int c0 = 0; c0 < nrt; c0 += 32) {
        float v[32];
        tmem_ld32(taddr + c0, v);
#pragma unroll
        for (int j = 0; j < 32; ++j) __stcg(part + (size_t)(c0 + j) * TC_BM + 32 * q + lane, v[j]);
      }
      __threadfence();
      epi_bar();
      if (threadIdx.x == 64)
        last_sh = atomicAdd(&a.ws.tickets[nti * mtiles + mt], 1u) == (unsigned)(S - 1);
      epi_bar();
      do_store = last_sh != 0;
      if (do_store) __threadfence();
    }
    if (do_store) {
      for (int c0 = 0; c0 < nrt; c0 += 32) {
        // the 32 columns' map entries, then their Y values, all issued before any store (the
        // stores may alias Y, so the compiler would otherwise wait out one load per column)
        int colv[32];
#pragma unroll
        for (int j = 0; j < 32; ++j) {
          const int c = n0 + c0 + j;
          colv[j] = c >= cnt ? -1 : (a.nmap ? a.nmap[c] : c);
        }
        float yv[32];
#pragma unroll
        for (int j = 0; j < 32; ++j) yv[j] = (a.Y && colv[j] >= 0) ? a.Y[(size_t)colv[j] * a.M + row] : 0.0f;
        float v[32];
        if (S > 1) {
#pragma unroll
          for (int j = 0; j < 32; ++j) v[j] = 0.0f;
          for (int s2 = 0; s2 < S; ++s2) {
            const float *src = a.ws.part + ((size_t)(nti * S + s2) * mtiles + mt) * (TC_BM * TC_BN);
#pragma unroll
            for (int j = 0; j < 32; ++j) v[j] += __ldcg(src + (size_t)(c0 + j) * TC_BM + 32 * q + lane);
          }
        } else {
          tmem_ld32(taddr + c0, v);
        }
#pragma unroll
        for (int j = 0; j < 32; ++j) {
          const int col = colv[j];
          if (col < 0) continue;
          const size_t o = (size_t)col * a.M + row;
          const float val = a.Y ? yv[j] - v[j] : v[j];
          a.Ct[o] = val;
          if (a.Cb) {
            const __nv_bfloat16 hi = __float2bfloat16_rn(val);
            if (a.cb_split) {
              const size_t qo = (size_t)col * 3 * a.M + row;
              a.Cb[qo] = hi;
              a.Cb[qo + a.M] = hi;
              a.Cb[qo + 2 * (size_t)a.M] = __float2bfloat16_rn(val - __bfloat162float(hi));
            } else {
              a.Cb[o] = hi;
            }
          }
        }
      }
      if (S > 1 && threadIdx.x == 64) a.ws.tickets[nti * mtiles + mt] = 0u;
    }
  }
  tc_fence_before();
  // the pair: neither CTA leaves (or frees tensor memory) while the other's MMAs or copies may
  // still touch its shared memory
  if constexpr (PAIR)
    cluster_sync_all();
  else
    __syncthreads();
  if (warp == 1) {
    tc_fence_after();
    tmem_dealloc<PAIR>(tmem);
  }
}

// B rows nmap[c] (c < *ncount) gathered into a contiguous row-major K-wide buffer
__global__ void k_gather_rows(const __nv_bfloat16 *__restrict__ B, int ldb, int K, const int *__restrict__ nmap,
                              const int *__restrict__ ncount, __nv_bfloat16 *__restrict__ out) {
  const int cnt = *ncount;
  const int per_row = K / 8;  // 16-byte chunks
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < (long long)cnt * per_row;
       q += (long long)gridDim.x * blockDim.x) {
    const int c = (int)(q / per_row), e = (int)(q % per_row) * 8;
    *reinterpret_cast<uint4 *>(out + (size_t)c * K + e) =
        __ldg(reinterpret_cast<const uint4 *>(B + (size_t)nmap[c] * ldb + e));
  }
}

PFN_cuTensorMapEncodeTiled_v12000 g_encode = nullptr;
std::once_flag g_encode_once;

gb_status tensor_map(CUtensorMap *map, const void *base, int rows, int K, int ld, int box_rows) {
  std::call_once(g_encode_once, [] {
    void *fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      g_encode = (PFN_cuTensorMapEncodeTiled_v12000)fn;
  });
  if (!g_encode) {
    gb_set_error_message("cuTensorMapEncodeTiled is not available from the driver", __FILE__, __LINE__);
    return GB_CUDA_ERROR;
  }
  const cuuint64_t dims[2] = {(cuuint64_t)K, (cuuint64_t)rows};
  const cuuint64_t strides[1] = {(cuuint64_t)ld * 2};
  const cuuint32_t box[2] = {TC_BK, (cuuint32_t)box_rows};
  const cuuint32_t estr[2] = {1, 1};
  const CUresult r = g_encode(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void *>(base), dims, strides, box,
                              estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                              CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) {
    gb_set_error_message("cuTensorMapEncodeTiled rejected a GEMM operand", __FILE__, __LINE__);
    return GB_BAD_ARG;
  }
  return GB_OK;
}

}  // namespace

// tcgen05 path of gb_gemm (gb_gemm.cu decides): M % 128, N % 256, K % 64, 16-byte aligned
// operands with row strides that are multiples of 8 elements.
gb_status gb_gemm_tc(const GbGemm &g, cudaStream_t s) {
  static std::atomic<unsigned long long> attr_done{0};
  GB_TRY(gb_once_per_device(attr_done, []() -> gb_status {
    GB_CUDA_TRY(
        cudaFuncSetAttribute(k_gemm_tn_tc<0>, cudaFuncAttributeMaxDynamicSharedMemorySize, TcCfg<0>::SMEM));
    GB_CUDA_TRY(
        cudaFuncSetAttribute(k_gemm_tn_tc<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, TcCfg<1>::SMEM));
    return GB_OK;
  }));
  // the CTA-pair instance unless M is an odd number of 128-row tiles or GB_CS_GEMM_PAIR=0
  const char *pe = getenv("GB_CS_GEMM_PAIR");
  const bool pair = !(pe && atoi(pe) == 0) && g.M % (2 * TC_BM) == 0;
  const void *B = g.B;
  int ldb = g.ldb;
  if (g.nmap) {
    if (!g.ws || !g.ws->gather || g.ws->gather_elems < (size_t)g.N * g.K) {
      gb_set_error_message("tcgen05 GEMM with a column map needs a gather buffer of N x K", __FILE__, __LINE__);
      return GB_BAD_ARG;
    }
    k_gather_rows<<<g.ws->num_sms * 4, 256, 0, s>>>((const __nv_bfloat16 *)g.B, g.ldb, g.K, g.nmap, g.ncount,
                                                     (__nv_bfloat16 *)g.ws->gather);
    GB_CUDA_TRY(cudaGetLastError());
    B = g.ws->gather;
    ldb = g.K;
  }
  CUtensorMap ta, tb;
  GB_TRY(tensor_map(&ta, g.A, g.M, g.K, g.lda, TC_BM));
  GB_TRY(tensor_map(&tb, B, g.N, g.K, ldb, pair ? TcCfg<1>::B_ROWS : TcCfg<0>::B_ROWS));
  TcArgs a = {};
  a.Ct = g.Ct;
  a.M = g.M;
  a.N = g.N;
  a.K = g.K;
  a.Y = g.Y;
  a.Cb = (__nv_bfloat16 *)g.Cb;
  a.cb_split = g.cb_split;
  a.nmap = g.nmap;
  a.ncount = g.ncount;
  a.s_max = 1;
  a.split_rows = g.split_rows;
  if (g.ws && g.ws->part && g.ws->tickets && (g.M / TC_BM) * (g.N / TC_BN) <= g.ws->ticket_count) {
    a.ws = *g.ws;
    a.s_max = GB_GEMM_SPLIT_MAX;
  }
  const dim3 grid(g.M / TC_BM, (g.N / TC_BN) * a.s_max);
  if (!pair) {
    k_gemm_tn_tc<0><<<grid, TC_THREADS, TcCfg<0>::SMEM, s>>>(ta, tb, a);
    GB_CUDA_TRY(cudaGetLastError());
    return GB_OK;
  }
  cudaLaunchConfig_t cfg = {};
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = 2;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.gridDim = grid;
  cfg.blockDim = dim3(TC_THREADS, 1, 1);
  cfg.dynamicSmemBytes = TcCfg<1>::SMEM;
  cfg.stream = s;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  GB_CUDA_TRY(cudaLaunchKernelEx(&cfg, k_gemm_tn_tc<1>, ta, tb, a));
  return GB_OK;
}

// Reads and clears the error word of the tcgen05 GEMM (0: no launch gave up).
gb_status gb_gemm_tc_check() {
  int err = 0;
  GB_CUDA_TRY(cudaMemcpyFromSymbol(&err, g_tc_error, sizeof(int)));
  if (err) {
    const int zero = 0;
    GB_CUDA_TRY(cudaMemcpyToSymbol(g_tc_error, &zero, sizeof(int)));
    gb_set_error_message("tcgen05 GEMM: a pipeline wait timed out", __FILE__, __LINE__);
    return GB_WATCHDOG;
  }
  return GB_OK;
}
