// gb_philox.cuh -- problem generation shared by every form of the library.
//
// Philox-4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as easy as 1, 2,
// 3", SC'11) keyed by (key, KEY_HI) with counter (block, block >> 32, stream, trial).  The
// reference draws problems with cuRAND's default generator, which cannot be reproduced
// outside that library; every implementation here (and the CPU oracle) uses this stream
// instead, with the reference's distributions.
#pragma once
#include <stdint.h>

namespace gbgen {

const uint32_t KEY_HI = 0x6A09E667u;
enum { ST_MATRIX = 1, ST_VALUES = 2, ST_SUPPORT = 3, ST_ROWS = 4, ST_SMV = 5, ST_SIGNS = 6, ST_NOISE = 7 };

__host__ __device__ inline void philox(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3, uint32_t k0, uint32_t k1,
                                       uint32_t out[4]) {
  for (int r = 0; r < 10; ++r) {
    const uint64_t p0 = (uint64_t)0xD2511F53u * c0;
    const uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
    const uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
    const uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
    const uint32_t n0 = hi1 ^ c1 ^ k0, n2 = hi0 ^ c3 ^ k1;
    c0 = n0; c1 = lo1; c2 = n2; c3 = lo0;
    k0 += 0x9E3779B9u; k1 += 0xBB67AE85u;
  }
  out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

// uniform on (0,1): 24 random bits centred in their cell (exact in float)
__host__ __device__ inline float u01(uint32_t x) { return ((float)(x >> 8) + 0.5f) * (1.0f / 16777216.0f); }

// Column j of a dense Gaussian matrix (createMeasurements_gen, N(0,1)/sqrt(m)), column-major:
// element e = j*m + i is lane e%4 of Philox block e/4 (two Box-Muller pairs per block).
// `lane`/`nlanes` split the column's blocks over cooperating threads; emit(i, a) also sees
// every entry a written to col[i] (for copies made from registers as the column is drawn).
template <class Emit>
__device__ inline void gen_dense_column_emit(float *col, int j, int m, uint32_t key, uint32_t trial, int ens, int lane,
                                             int nlanes, Emit &&emit) {
  const float scale = 1.0f / sqrtf((float)m);
  const uint64_t e0 = (uint64_t)j * (uint64_t)m, e1 = e0 + (uint64_t)m;
  for (uint64_t g = (e0 >> 2) + lane; g < ((e1 + 3) >> 2); g += nlanes) {
    uint32_t o[4];
    philox((uint32_t)g, (uint32_t)(g >> 32), ST_MATRIX, trial, key, KEY_HI, o);
    float v[4];
    if (ens == 2) {
      for (int t = 0; t < 4; ++t) v[t] = signbit(u01(o[t]) - 0.5f) ? -1.0f : 1.0f;
    } else {
      for (int t = 0; t < 2; ++t) {
        const float r = sqrtf(-2.0f * logf(u01(o[2 * t])));
        float sn, cs;
        sincospif(2.0f * u01(o[2 * t + 1]), &sn, &cs);
        v[2 * t] = r * cs;
        v[2 * t + 1] = r * sn;
      }
    }
    for (int t = 0; t < 4; ++t) {
      const uint64_t e = g * 4 + t;
      if (e >= e0 && e < e1) {
        const float a = v[t] * scale;
        col[e - e0] = a;
        emit((int)(e - e0), a);
      }
    }
  }
}

__device__ inline void gen_dense_column(float *col, int j, int m, uint32_t key, uint32_t trial, int ens, int lane,
                                        int nlanes) {
  gen_dense_column_emit(col, j, m, key, trial, ens, lane, nlanes, [](int, float) {});
}

// element e of a uniform stream
__host__ __device__ inline float uniform_at(uint32_t key, uint32_t trial, uint32_t stream, uint64_t e) {
  uint32_t o[4];
  philox((uint32_t)(e >> 2), (uint32_t)(e >> 34), stream, trial, key, KEY_HI, o);
  return u01(o[e & 3]);
}

}  // namespace gbgen
