/*
 * cuda_host_shim.h -- lets g++ compile a few of the reference's own CUDA source
 * files (unmodified, where they lie) so their SIMT kernels and host routines can be
 * executed on the CPU to produce golden vectors.  TEST INFRASTRUCTURE ONLY.
 *
 * Emulation model: a kernel "launch" is a loop over (block, thread) pairs on one
 * host thread.  That is a valid schedule for kernels whose threads do not
 * communicate through shared memory or __syncthreads barriers, which holds for
 * every kernel driven from ref_driver.cpp.  atomicAdd is a plain read-add-write.
 */
#pragma once
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <algorithm>
using std::abs;
using std::max;
using std::min;

#define __global__
#define __device__
#define __host__
#define __forceinline__ inline
#define __constant__ static
#define __shared__ static

struct gb_dim3 { unsigned int x, y, z; };
typedef gb_dim3 uint3;
extern gb_dim3 threadIdx, blockIdx, blockDim, gridDim;

inline int atomicAdd(int *p, int v) { int o = *p; *p = o + v; return o; }
inline unsigned int atomicAdd(unsigned int *p, unsigned int v) { unsigned int o = *p; *p = o + v; return o; }
inline float atomicAdd(float *p, float v) { float o = *p; *p = o + v; return o; }
inline int atomicSub(int *p, int v) { int o = *p; *p = o - v; return o; }
inline void __syncthreads() {}
inline float max(float a, int b) { return std::max(a, (float)b); }
inline float max(int a, float b) { return std::max((float)a, b); }

/* timing calls used by the reference's host routines become no-ops */
typedef int cudaEvent_t;
inline int cudaEventCreate(cudaEvent_t *) { return 0; }
inline int cudaEventRecord(cudaEvent_t, int) { return 0; }
inline int cudaEventSynchronize(cudaEvent_t) { return 0; }
inline int cudaEventElapsedTime(float *t, cudaEvent_t, cudaEvent_t) { *t = 0.0f; return 0; }
inline int cudaEventDestroy(cudaEvent_t) { return 0; }
inline int cudaThreadSynchronize() { return 0; }
inline int cudaDeviceSynchronize() { return 0; }
