// gb_noalloc.cu -- dense operator apply that allocates no device memory.
//
// gb_cs_operator_apply allocates a workspace on every call.  Some callers cannot do
// that: code running inside a CUDA stream capture (cudaMalloc is not capturable),
// memory-budgeted services that own every allocation up front, and embedders whose
// allocator is not CUDA's.  gb_cs_dense_apply_noalloc computes the same product with
// its scratch (device state, support list, partial row tiles, arrival counters) placed
// in one file-scope device array of GB_NOALLOC_SCRATCH_BYTES, which every GPU that loads
// this library holds until the process exits.
//
// Rules of use:
//   - the first call on a device looks up the scratch array's device address for that
//     device (cudaGetSymbolAddress); make that first call outside any stream capture;
//   - all calls share the one scratch array, which keeps the previous call's contents:
//     calls whose work overlaps on the GPU (different streams or threads without
//     ordering) race on it and must be serialised by the caller;
//   - m <= GB_NOALLOC_MAX_M and n <= GB_NOALLOC_MAX_N, otherwise GB_BAD_ARG; every such
//     shape fits, since the A x split count is lowered until its partial tiles fit;
//   - transpose == 2 reuses the support list of the previous transpose == 0 call on the
//     device, which must have had the same A, lda, m and n, with no transpose == 1 call in
//     between (that call rebuilds the scratch state); otherwise GB_BAD_ARG.
#include <string.h>

#include <algorithm>
#include <mutex>

#include "gb_internal.cuh"

#define GB_NOALLOC_SCRATCH_BYTES (1 << 20)
#define GB_NOALLOC_MAX_M 65536
#define GB_NOALLOC_MAX_N 65536

static __device__ __align__(256) unsigned char g_noalloc_scratch[GB_NOALLOC_SCRATCH_BYTES];

__global__ void k_init_state(GbState *st, GbState init);

namespace {

const int kMaxDevices = 64;
unsigned char *g_scratch_ptr[kMaxDevices] = {nullptr};
// the operator of the support list the last transpose == 0 call built (cleared by a
// transpose == 1 call, which reinitialises the scratch state)
struct SupportKey {
  const float *A;
  int lda, m, n;
};
SupportKey g_support[kMaxDevices] = {};
std::mutex g_scratch_mu;

// device address of the scratch array for the current device (looked up once)
gb_status scratch_for_current_device(unsigned char **out) {
  int dev = 0;
  GB_CUDA_TRY(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) {
    gb_set_error_message("device ordinal out of range for the no-alloc scratch table", __FILE__, __LINE__);
    return GB_UNSUPPORTED;
  }
  std::lock_guard<std::mutex> lock(g_scratch_mu);
  if (!g_scratch_ptr[dev]) {
    void *p = nullptr;
    GB_CUDA_TRY(cudaGetSymbolAddress(&p, g_noalloc_scratch));
    g_scratch_ptr[dev] = (unsigned char *)p;
  }
  *out = g_scratch_ptr[dev];
  return GB_OK;
}

size_t align256(size_t b) { return (b + 255) & ~(size_t)255; }

}  // namespace

extern "C" gb_status gb_cs_dense_apply_noalloc(const float *d_A, int lda, int m, int n, int transpose,
                                               const float *d_in, float *d_out, void *stream) {
  if (!d_A || !d_in || !d_out || m < 1 || n < 1 || transpose < 0 || transpose > 2) {
    gb_set_error_message("gb_cs_dense_apply_noalloc: null buffer or empty size", __FILE__, __LINE__);
    return GB_BAD_ARG;
  }
  if (m > GB_NOALLOC_MAX_M || n > GB_NOALLOC_MAX_N) {
    gb_set_error_message("gb_cs_dense_apply_noalloc: m and n must be <= 65536 (fixed scratch size)", __FILE__,
                         __LINE__);
    return GB_BAD_ARG;
  }
  if (lda <= 0) lda = m;
  if (lda < m) {
    gb_set_error_message("gb_cs_dense_apply_noalloc: lda < m", __FILE__, __LINE__);
    return GB_BAD_ARG;
  }
  unsigned char *base = nullptr;
  GB_TRY(scratch_for_current_device(&base));
  cudaStream_t s = (cudaStream_t)stream;
  GbWork w;
  memset(&w, 0, sizeof(w));
  int dev = 0;
  GB_CUDA_TRY(cudaGetDevice(&dev));
  GB_CUDA_TRY(cudaDeviceGetAttribute(&w.num_sms, cudaDevAttrMultiProcessorCount, dev));
  w.red_blocks = std::min(GB_MAXRB, w.num_sms * 2);
  w.wide_blocks = w.num_sms * 8;
  GbOp &op = w.op;
  op.kind = GB_OP_DENSE;
  op.m = m;
  op.n = n;
  op.lda = lda;
  op.A = d_A;
  // float4 streams of A, and for A^T r of the input too (A x reads its input per entry)
  op.vec4 = (lda % 4 == 0) && (((uintptr_t)d_A & 15) == 0) && (transpose != 1 || (((uintptr_t)d_in & 15) == 0));
  gb_dense_av_shape(m, w.num_sms, false, &w.av_ntile, &w.av_nsplit, &w.av_rows);
  // carve the scratch: state | support list | tile counts | arrival counters | partial tiles
  size_t off = 0;
  w.st = (GbState *)(base + off);
  off += align256(sizeof(GbState));
  w.S = (int *)(base + off);
  off += align256((size_t)GB_NOALLOC_MAX_N * 4);
  w.tile_cnt = (int *)(base + off);
  off += align256((size_t)((GB_NOALLOC_MAX_N + GB_TILE - 1) / GB_TILE) * 4);
  w.av_tickets = (unsigned int *)(base + off);
  const size_t tickets_bytes = align256((size_t)w.av_ntile * 4);
  off += tickets_bytes;
  w.part = (float *)(base + off);
  // fewer support splits until the partial tiles fit (one split, which writes no
  // partials, fits every m <= GB_NOALLOC_MAX_M)
  while (w.av_nsplit > 1 &&
         off + align256(gb_dense_part_floats_av(w.av_ntile, w.av_nsplit, w.av_rows) * 4) > GB_NOALLOC_SCRATCH_BYTES)
    --w.av_nsplit;
  w.part_cap = gb_dense_part_floats_av(w.av_ntile, w.av_nsplit, w.av_rows);
  off += align256(w.part_cap * 4);
  if (off > GB_NOALLOC_SCRATCH_BYTES) {
    gb_set_error_message("gb_cs_dense_apply_noalloc: scratch too small for this shape", __FILE__, __LINE__);
    return GB_BAD_ARG;
  }
  // state of a single operator application; the arrival counters must start at zero
  GbState init;
  memset(&init, 0, sizeof(init));
  init.m = m;
  init.n = n;
  init.lda = lda;
  init.active = 1;
  init.flags[F_ALWAYS] = 1;
  if (transpose == 2) {
    // A x on the support list of the previous transpose == 0 call: the state and the
    // list are still in the scratch array when that call was for the same operator
    {
      std::lock_guard<std::mutex> lock(g_scratch_mu);
      const SupportKey &k = g_support[dev];
      if (k.A != d_A || k.lda != lda || k.m != m || k.n != n) {
        gb_set_error_message("gb_cs_dense_apply_noalloc: transpose == 2 needs a previous transpose == 0 call "
                             "with the same A, lda, m and n on this device (and no transpose == 1 call since)",
                             __FILE__, __LINE__);
        return GB_BAD_ARG;
      }
    }
    GB_CUDA_TRY(cudaMemsetAsync(w.av_tickets, 0, tickets_bytes, s));
    enq_A(w, s, d_in, d_out, nullptr, -1, F_ALWAYS);
    GB_CUDA_TRY(cudaGetLastError());
    return GB_OK;
  }
  GB_CUDA_TRY(cudaMemsetAsync(w.av_tickets, 0, tickets_bytes, s));
  k_init_state<<<1, 1, 0, s>>>(w.st, init);
  if (transpose) {
    {
      std::lock_guard<std::mutex> lock(g_scratch_mu);
      g_support[dev] = SupportKey{};
    }
    enq_AT(w, s, d_in, d_out, F_ALWAYS);
  } else {
    enq_support_of_nonzeros(w, s, d_in, n);
    enq_A(w, s, d_in, d_out, nullptr, -1, F_ALWAYS);
    std::lock_guard<std::mutex> lock(g_scratch_mu);
    g_support[dev] = SupportKey{d_A, lda, m, n};
  }
  GB_CUDA_TRY(cudaGetLastError());
  return GB_OK;
}
