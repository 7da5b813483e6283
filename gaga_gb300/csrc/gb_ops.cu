// gb_ops.cu -- measurement operators on sm_103a.
//
//   dense   A v  : gather of the support columns (coalesced float4 column streams,
//                  split-K over fixed chunks of S, partials reduced in chunk order)
//                  replaces gen_matvec_sparse (GAGA/Matrices/gen_gpu.cu:79-132,141-152)
//           A^T r: one warp per column of the same column-major A (no transposed copy),
//                  replaces gen_matvec on d_AT + matrix_transpose (gen_gpu.cu:33-74,161-171,
//                  GAGA/gaga/kernels.cu:237-246)
//   dct     row-subsampled orthonormal DCT-II and its transpose by Makhoul's reordering
//           and a hand-written two-pass shared-memory radix-2 FFT (n = n1 * n2), replaces
//           the cuFFT path of GAGA/Matrices/dct_gpu.cu:121-353
//   smv     A v  : one thread per row over a column-sorted CSR copy (atomic-free)
//           A^T r: one thread per column over its d nonzeros
//           replaces sparse_matvec / sparse_matvecT (GAGA/Matrices/smv_gpu.cu:29-47)
#include "gb_internal.cuh"

// ------------------------------------------------------------------ dense
#define DG_THREADS 128  // 4 warps
#define DG_ROWS 128     // rows per work item (32 lanes x float4)
#define DG_CHUNK 32     // support columns per work item

size_t gb_dense_part_floats(int m_pad, int n) {
  size_t nch = (size_t)(n + DG_CHUNK - 1) / DG_CHUNK;
  return nch * (size_t)m_pad;
}

// partial[c][i] = sum_{s in chunk c} A[i, S[s]] * v[S[s]]  for rows i of the work item
template <int VEC>
__global__ void __launch_bounds__(DG_THREADS) k_dense_gather(const GbState *__restrict__ st, int pf,
                                                             const float *__restrict__ A, int lda, int m,
                                                             const int *__restrict__ S,
                                                             const float *__restrict__ v,
                                                             float *__restrict__ part) {
  if (!gb_pred(st, pf)) return;
  const int s = st->s_cnt;
  const int nch = (s + DG_CHUNK - 1) / DG_CHUNK;
  const int nrt = (m + DG_ROWS - 1) / DG_ROWS;
  const int items = nrt * nch;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  __shared__ int sj[DG_CHUNK];
  __shared__ float sv[DG_CHUNK];
  __shared__ float4 red[4][32];
  for (int it = blockIdx.x; it < items; it += gridDim.x) {
    const int rt = it % nrt, ch = it / nrt;
    const int c0 = ch * DG_CHUNK;
    const int cn = min(DG_CHUNK, s - c0);
    __syncthreads();
    if (threadIdx.x < cn) {
      int j = S[c0 + threadIdx.x];
      sj[threadIdx.x] = j;
      sv[threadIdx.x] = v[j];
    }
    __syncthreads();
    float a0 = 0.f, a1 = 0.f, a2 = 0.f, a3 = 0.f;
    if (VEC == 4) {
      const int row = rt * DG_ROWS + lane * 4;
      if (row < m) {
#pragma unroll 4
        for (int c = warp; c < cn; c += 4) {
          const float4 a = __ldg(reinterpret_cast<const float4 *>(A + (size_t)sj[c] * lda + row));
          const float vj = sv[c];
          a0 = fmaf(a.x, vj, a0);
          a1 = fmaf(a.y, vj, a1);
          a2 = fmaf(a.z, vj, a2);
          a3 = fmaf(a.w, vj, a3);
        }
      }
    } else {
      const int rbase = rt * DG_ROWS + lane;
#pragma unroll 2
      for (int c = warp; c < cn; c += 4) {
        const float *col = A + (size_t)sj[c] * lda;
        const float vj = sv[c];
        if (rbase < m) a0 = fmaf(__ldg(col + rbase), vj, a0);
        if (rbase + 32 < m) a1 = fmaf(__ldg(col + rbase + 32), vj, a1);
        if (rbase + 64 < m) a2 = fmaf(__ldg(col + rbase + 64), vj, a2);
        if (rbase + 96 < m) a3 = fmaf(__ldg(col + rbase + 96), vj, a3);
      }
    }
    red[warp][lane] = make_float4(a0, a1, a2, a3);
    __syncthreads();
    if (warp == 0) {
      float4 r = red[0][lane];
#pragma unroll
      for (int w2 = 1; w2 < 4; ++w2) {
        float4 q = red[w2][lane];
        r.x += q.x; r.y += q.y; r.z += q.z; r.w += q.w;
      }
      float *dst = part + (size_t)ch * lda;
      if (VEC == 4) {
        const int row = rt * DG_ROWS + lane * 4;
        if (row < m) *reinterpret_cast<float4 *>(dst + row) = r;
      } else {
        const int rbase = rt * DG_ROWS + lane;
        if (rbase < m) dst[rbase] = r.x;
        if (rbase + 32 < m) dst[rbase + 32] = r.y;
        if (rbase + 64 < m) dst[rbase + 64] = r.z;
        if (rbase + 96 < m) dst[rbase + 96] = r.w;
      }
    }
  }
}

// out_i = [y_i -] sum_c partial[c][i]; optional ||out||^2 into st->red[slot]
__global__ void k_dense_finish(GbState *st, int pf, const float *__restrict__ part, int lda, int m,
                               const float *__restrict__ y, float *__restrict__ out, int slot,
                               float *red_part, unsigned int *tickets) {
  if (!gb_pred(st, pf)) return;
  const int nch = (st->s_cnt + DG_CHUNK - 1) / DG_CHUNK;
  float acc2 = 0.0f;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < m; i += gridDim.x * blockDim.x) {
    float sum = 0.0f;
    for (int c = 0; c < nch; ++c) sum += part[(size_t)c * lda + i];
    float o = y ? y[i] - sum : sum;
    out[i] = o;
    acc2 = fmaf(o, o, acc2);
  }
  if (slot >= 0) grid_reduce_publish<0>(acc2, slot, st, red_part, tickets);
}

// g_j = sum_i A[i, j] r_i, one warp per column
template <int VEC>
__global__ void __launch_bounds__(256) k_dense_at(const GbState *__restrict__ st, int pf,
                                                  const float *__restrict__ A, int lda, int m, int n,
                                                  const float *__restrict__ r, float *__restrict__ g) {
  if (!gb_pred(st, pf)) return;
  const int lane = threadIdx.x & 31;
  const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int nw = (gridDim.x * blockDim.x) >> 5;
  for (int j = gw; j < n; j += nw) {
    const float *col = A + (size_t)j * lda;
    float a0 = 0.f, a1 = 0.f, a2 = 0.f, a3 = 0.f;
    if (VEC == 4) {
      int i = lane * 4;
      // full float4 groups (rows i..i+3 all < m)
      const int mfull = m & ~3;
#pragma unroll 4
      for (; i < mfull; i += 128) {
        const float4 a = __ldg(reinterpret_cast<const float4 *>(col + i));
        const float4 b = __ldg(reinterpret_cast<const float4 *>(r + i));
        a0 = fmaf(a.x, b.x, a0);
        a1 = fmaf(a.y, b.y, a1);
        a2 = fmaf(a.z, b.z, a2);
        a3 = fmaf(a.w, b.w, a3);
      }
      if (i < m) {  // ragged tail inside one float4 group
        if (i < m) a0 = fmaf(__ldg(col + i), __ldg(r + i), a0);
        if (i + 1 < m) a1 = fmaf(__ldg(col + i + 1), __ldg(r + i + 1), a1);
        if (i + 2 < m) a2 = fmaf(__ldg(col + i + 2), __ldg(r + i + 2), a2);
      }
    } else {
#pragma unroll 4
      for (int i = lane; i < m; i += 32) a0 = fmaf(__ldg(col + i), __ldg(r + i), a0);
    }
    float t = (a0 + a1) + (a2 + a3);
    t = warp_sum(t);
    if (lane == 0) g[j] = t;
  }
}

// ------------------------------------------------------------------ DCT
// Two-pass FFT: n = n1 * n2, index j = j1*n2 + j2, frequency k = k1 + n1*k2.
//   pass 1: for each j2, an n1-point FFT over j1 (stride n2), times exp(-+2 pi i j2 k1 / n),
//           stored at k1*n2 + j2
//   pass 2: for each k1, an n2-point FFT over j2 (contiguous), stored at k1 + n1*k2
// Each block transforms FFT_ELEMS / L sequences of length L in shared memory.
#define FFT_ELEMS 4096
#define FFT_THREADS 512

enum { LOAD_MAKHOUL = 0, LOAD_FREQ = 1, LOAD_CPLX = 2 };
enum { STORE_CPLX_T = 0, STORE_CPLX_NAT = 1, STORE_MAKHOUL_REAL = 2 };

__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
  return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

// exp(sgn * i * pi * num / den) for exact integer num, power-of-two den
__device__ __forceinline__ float2 cis_pi(float sgn, float num_over_den) {
  float s, c;
  sincospif(num_over_den, &s, &c);
  return make_float2(c, sgn * s);
}

template <int INV, int LOAD, int STORE>
__global__ void __launch_bounds__(FFT_THREADS) k_fft_pass(const GbState *__restrict__ st, int pf, int pass,
                                                          int logL, int log1, int log2,
                                                          const float *__restrict__ vin,
                                                          const float2 *__restrict__ cin,
                                                          float2 *__restrict__ cout,
                                                          float *__restrict__ rout) {
  if (!gb_pred(st, pf)) return;
  extern __shared__ float2 sm[];
  const int L = 1 << logL;
  const int B = FFT_ELEMS / L;  // sequences per block (L <= FFT_ELEMS)
  float2 *buf = sm;             // B * L
  float2 *tw = sm + FFT_ELEMS;  // L / 2 twiddles exp(-+2 pi i t / L)
  const int n1 = 1 << log1, n2 = 1 << log2;
  const int N = n1 * n2;
  const int nseq = pass == 1 ? n2 : n1;
  const float sgn = INV ? 1.0f : -1.0f;
  for (int t = threadIdx.x; t < L / 2; t += blockDim.x) tw[t] = cis_pi(sgn, (2.0f * t) / (float)L);
  const float wn0 = sqrtf(1.0f / (float)N), wn = sqrtf(2.0f / (float)N);
  for (int seq0 = blockIdx.x * B; seq0 < nseq; seq0 += gridDim.x * B) {
    __syncthreads();
    // load: element e of local sequence b, bit-reversed into shared memory
    for (int q = threadIdx.x; q < B * L; q += blockDim.x) {
      int b, e;
      if (pass == 1) { b = q % B; e = q / B; }  // consecutive threads -> consecutive j2
      else { b = q / L; e = q % L; }            // consecutive threads -> contiguous row
      const int sq = seq0 + b;
      float2 val = make_float2(0.f, 0.f);
      if (sq < nseq) {
        if (pass == 1) {
          const int idx = e * n2 + sq;  // natural index j1*n2 + j2
          if (LOAD == LOAD_MAKHOUL) {
            // Makhoul reordering: w[j] = x[2j] (j < N/2), w[N-1-j'] = x[2j'+1]
            const int src = idx < N / 2 ? 2 * idx : 2 * (N - 1 - idx) + 1;
            val = make_float2(vin[src], 0.f);
          } else if (LOAD == LOAD_FREQ) {
            const float xv = vin[idx];
            if (xv != 0.0f) {
              const float wgt = idx == 0 ? wn0 : wn;
              const float2 c = cis_pi(1.0f, (float)idx / (float)(2 * N));
              val = make_float2(wgt * xv * c.x, wgt * xv * c.y);
            }
          } else {
            val = cin[idx];
          }
        } else {
          val = cin[(size_t)sq * n2 + e];
        }
      }
      const int pos = (int)(__brev((unsigned)e) >> (32 - logL));
      buf[b * L + pos] = val;
    }
    __syncthreads();
    // radix-2 decimation-in-time stages
    for (int s = 1; s <= logL; ++s) {
      const int half = 1 << (s - 1);
      for (int u = threadIdx.x; u < B * L / 2; u += blockDim.x) {
        const int b = u >> (logL - 1);
        const int q = u & (L / 2 - 1);
        const int pos = q & (half - 1);
        const int i0 = b * L + ((q >> (s - 1)) << s) + pos;
        const int i1 = i0 + half;
        const float2 w = tw[pos << (logL - s)];
        const float2 a = buf[i0];
        const float2 bb = cmul(buf[i1], w);
        buf[i0] = make_float2(a.x + bb.x, a.y + bb.y);
        buf[i1] = make_float2(a.x - bb.x, a.y - bb.y);
      }
      __syncthreads();
    }
    // store
    for (int q = threadIdx.x; q < B * L; q += blockDim.x) {
      int b, e;
      if (pass == 1) { b = q % B; e = q / B; }
      else { b = q % B; e = q / B; }  // pass 2 stores k1 + n1*k2: consecutive b contiguous
      const int sq = seq0 + b;
      if (sq >= nseq) continue;
      float2 val = buf[b * L + e];
      if (pass == 1) {
        // twiddle exp(-+2 pi i j2 k1 / N), j2 = sq, k1 = e
        const int prod = (int)(((long long)sq * e) & (N - 1));
        val = cmul(val, cis_pi(sgn, (2.0f * prod) / (float)N));
        cout[(size_t)e * n2 + sq] = val;
      } else {
        const int kk = sq + n1 * e;  // natural frequency / time index
        if (STORE == STORE_CPLX_NAT) {
          cout[kk] = val;
        } else {
          // inverse Makhoul: x[2m] = v[m], x[2m+1] = v[N-1-m]
          const int dst = kk < N / 2 ? 2 * kk : 2 * (N - 1 - kk) + 1;
          rout[dst] = val.x;
        }
      }
    }
  }
}

// forward post-processing at the sampled rows: X_k = w_k Re(W_k exp(-i pi k / 2N))
__global__ void k_dct_select(GbState *st, int pf, const float2 *__restrict__ W, const int *__restrict__ rows,
                             int m, int N, const float *__restrict__ y, float *__restrict__ out, int slot,
                             float *red_part, unsigned int *tickets) {
  if (!gb_pred(st, pf)) return;
  const float wn0 = sqrtf(1.0f / (float)N), wn = sqrtf(2.0f / (float)N);
  float acc2 = 0.0f;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < m; i += gridDim.x * blockDim.x) {
    const int k = rows[i];
    const float2 Wk = W[k];
    float s, c;
    sincospif((float)k / (float)(2 * N), &s, &c);
    const float X = (k == 0 ? wn0 : wn) * (Wk.x * c + Wk.y * s);
    const float o = y ? y[i] - X : X;
    out[i] = o;
    acc2 = fmaf(o, o, acc2);
  }
  if (slot >= 0) grid_reduce_publish<0>(acc2, slot, st, red_part, tickets);
}

// inverse pre-processing: frequency image at the sampled rows
__global__ void k_dct_scatter(const GbState *st, int pf, const int *__restrict__ rows, int m,
                              const float *__restrict__ r, float *__restrict__ freq) {
  if (!gb_pred(st, pf)) return;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < m; i += gridDim.x * blockDim.x) freq[rows[i]] = r[i];
}

// ------------------------------------------------------------------ smv
__global__ void k_smv_A(GbState *st, int pf, const int *__restrict__ ptr, const int *__restrict__ col,
                        const float *__restrict__ val, int m, const float *__restrict__ v,
                        const float *__restrict__ y, float *__restrict__ out, int slot, float *red_part,
                        unsigned int *tickets) {
  if (!gb_pred(st, pf)) return;
  float acc2 = 0.0f;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < m; i += gridDim.x * blockDim.x) {
    float sum = 0.0f;
    const int e1 = ptr[i + 1];
    for (int e = ptr[i]; e < e1; ++e) sum = __fadd_rn(sum, __fmul_rn(val[e], v[col[e]]));
    const float o = y ? __fsub_rn(y[i], sum) : sum;
    out[i] = o;
    acc2 = fmaf(o, o, acc2);
  }
  if (slot >= 0) grid_reduce_publish<0>(acc2, slot, st, red_part, tickets);
}

__global__ void k_smv_AT(const GbState *st, int pf, const int *__restrict__ rows, const float *__restrict__ vals,
                         int n, int d, const float *__restrict__ r, float *__restrict__ g) {
  if (!gb_pred(st, pf)) return;
  for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
    float sum = 0.0f;
    const size_t base = (size_t)j * d;
    for (int t = 0; t < d; ++t) sum = __fadd_rn(sum, __fmul_rn(vals[base + t], r[rows[base + t]]));
    g[j] = sum;
  }
}

// ------------------------------------------------------------------ enqueue
static int fft_smem(int logL) { return (FFT_ELEMS + (1 << logL) / 2) * (int)sizeof(float2); }

template <int INV, int LOAD, int STORE>
static void launch_fft(GbWork &w, cudaStream_t s, int pf, int pass, const float *vin, const float2 *cin,
                       float2 *cout, float *rout) {
  const GbOp &op = w.op;
  const int logL = pass == 1 ? op.log1 : op.log2;
  const int L = 1 << logL;
  const int nseq = pass == 1 ? (1 << op.log2) : (1 << op.log1);
  const int B = FFT_ELEMS / L;
  int blocks = (nseq + B - 1) / B;
  if (blocks > w.num_sms * 4) blocks = w.num_sms * 4;
  const int smem = fft_smem(logL);
  k_fft_pass<INV, LOAD, STORE><<<blocks, FFT_THREADS, smem, s>>>(w.st, pf, pass, logL, op.log1, op.log2, vin,
                                                                  cin, cout, rout);
}

void enq_A(GbWork &w, cudaStream_t s, const float *v, float *out, const float *y, int slot, int pf) {
  const GbOp &op = w.op;
  if (op.kind == GB_OP_DENSE) {
    int blocks = w.num_sms * 8;
    if (op.vec4)
      k_dense_gather<4><<<blocks, DG_THREADS, 0, s>>>(w.st, pf, op.A, op.lda, op.m, w.S, v, w.part);
    else
      k_dense_gather<1><<<blocks, DG_THREADS, 0, s>>>(w.st, pf, op.A, op.lda, op.m, w.S, v, w.part);
    k_dense_finish<<<w.red_blocks, 256, 0, s>>>(w.st, pf, w.part, op.lda, op.m, y, out, slot, w.red_part,
                                                 w.tickets);
  } else if (op.kind == GB_OP_DCT) {
    launch_fft<0, LOAD_MAKHOUL, STORE_CPLX_T>(w, s, pf, 1, v, nullptr, op.cbuf0, nullptr);
    launch_fft<0, LOAD_CPLX, STORE_CPLX_NAT>(w, s, pf, 2, nullptr, op.cbuf0, op.cbuf1, nullptr);
    k_dct_select<<<w.red_blocks, 256, 0, s>>>(w.st, pf, op.cbuf1, op.rows, op.m, op.n, y, out, slot,
                                               w.red_part, w.tickets);
  } else {
    k_smv_A<<<w.red_blocks, 256, 0, s>>>(w.st, pf, op.csr_ptr, op.csr_col, op.csr_val, op.m, v, y, out, slot,
                                         w.red_part, w.tickets);
  }
}

void enq_AT(GbWork &w, cudaStream_t s, const float *r, float *g, int pf) {
  const GbOp &op = w.op;
  if (op.kind == GB_OP_DENSE) {
    int blocks = w.num_sms * 8;
    if (op.vec4)
      k_dense_at<4><<<blocks, 256, 0, s>>>(w.st, pf, op.A, op.lda, op.m, op.n, r, g);
    else
      k_dense_at<1><<<blocks, 256, 0, s>>>(w.st, pf, op.A, op.lda, op.m, op.n, r, g);
  } else if (op.kind == GB_OP_DCT) {
    int blocks = (op.m + 255) / 256;
    if (blocks > w.num_sms * 8) blocks = w.num_sms * 8;
    k_dct_scatter<<<blocks, 256, 0, s>>>(w.st, pf, op.rows, op.m, r, op.freq);
    launch_fft<1, LOAD_FREQ, STORE_CPLX_T>(w, s, pf, 1, op.freq, nullptr, op.cbuf0, nullptr);
    launch_fft<1, LOAD_CPLX, STORE_MAKHOUL_REAL>(w, s, pf, 2, nullptr, op.cbuf0, nullptr, g);
  } else {
    int blocks = (op.n + 255) / 256;
    if (blocks > w.num_sms * 16) blocks = w.num_sms * 16;
    k_smv_AT<<<blocks, 256, 0, s>>>(w.st, pf, op.smv_rows, op.smv_vals, op.n, op.d, r, g);
  }
}

// one-time attribute setup for the FFT kernels (dynamic shared memory above 48 KB)
gb_status gb_ops_init_attributes() {
  const int smem = fft_smem(12);
  GB_CUDA_TRY(cudaFuncSetAttribute(k_fft_pass<0, LOAD_MAKHOUL, STORE_CPLX_T>,
                                   cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
  GB_CUDA_TRY(cudaFuncSetAttribute(k_fft_pass<0, LOAD_CPLX, STORE_CPLX_NAT>,
                                   cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
  GB_CUDA_TRY(cudaFuncSetAttribute(k_fft_pass<1, LOAD_FREQ, STORE_CPLX_T>,
                                   cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
  GB_CUDA_TRY(cudaFuncSetAttribute(k_fft_pass<1, LOAD_CPLX, STORE_MAKHOUL_REAL>,
                                   cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
  return GB_OK;
}
