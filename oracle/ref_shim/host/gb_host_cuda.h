/*
 * gb_host_cuda.h -- host (CPU) emulation of the CUDA C++ runtime, enough for g++ to
 * compile the reference's unmodified MEX gateways (GAGA/gaga/gaga_{gen,dct,smv}.cu and
 * everything they include) and run them on the CPU.  TEST INFRASTRUCTURE ONLY: it exists
 * to produce the reference's own outputs as golden fixtures.
 *
 * Execution model.  A kernel launch `k<<<grid, block>>>(args)` is rewritten by the build
 * recipe (oracle/build.py) into `GB_LAUNCH(k, grid, block)(args)`.  Blocks run one after
 * another in (z, y, x) order; inside a block every thread runs as a fiber on its own stack,
 * thread 0 first.  __syncthreads() suspends the calling fiber; when every live thread of
 * the block is suspended (or finished), all of them resume, in thread order.  That is the
 * barrier semantics CUDA gives a block (threads that have exited count as arrived).
 * __shared__ variables become function-scope statics, so the threads of a block share
 * them.  Atomics are plain read-modify-write (fibers only switch at barriers).  Device
 * memory is host memory: cudaMalloc is calloc, cudaMemcpy is memmove.
 *
 * Floating point: kernels run in FP32 as written (the build disables FP contraction);
 * __cosf/__sinf are cosf/sinf.  The closed libraries the reference calls (cuBLAS v1,
 * cuFFT, cuRAND, Thrust) are restated in gb_host_libs.h.
 */
#pragma once
#include <setjmp.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <sys/types.h>

#include <algorithm>
#include <cmath>
#include <functional>

#define __global__
#define __device__
#define __host__
#define __forceinline__ inline
#define __noinline__
#define __constant__ static
#define __shared__ static
#define __launch_bounds__(...)
#define __restrict__ __restrict

using std::abs;
using std::ceil;
using std::floor;
using std::sqrt;

struct uint3 {
  unsigned int x, y, z;
};
struct dim3 {
  unsigned int x, y, z;
  dim3(unsigned int a = 1, unsigned int b = 1, unsigned int c = 1) : x(a), y(b), z(c) {}
};
struct float2 {
  float x, y;
};
struct float4 {
  float x, y, z, w;
};
struct int2 {
  int x, y;
};
inline float2 make_float2(float a, float b) { return float2{a, b}; }

extern uint3 threadIdx, blockIdx;
extern dim3 blockDim, gridDim;

namespace gbh {
// runs `thread` for every thread of every block of the grid (gb_host_runtime.cpp)
void run_launch(dim3 grid, dim3 block, const void *kernel, const std::function<void()> &thread);
void syncthreads();
void *dynamic_shared();

template <class F>
struct Launch {
  F *f;
  dim3 g, b;
  template <class... A>
  void operator()(A... a) const {
    run_launch(g, b, reinterpret_cast<const void *>(f), [&]() { f(a...); });
  }
};
template <class F>
Launch<F> launch(F *f, dim3 g, dim3 b, size_t = 0, int = 0) {
  return Launch<F>{f, g, b};
}
}  // namespace gbh

#define GB_LAUNCH(fn, ...) ::gbh::launch(fn, __VA_ARGS__)

inline void __syncthreads() { gbh::syncthreads(); }

/* atomics: fibers switch only at barriers, so a plain read-modify-write is atomic */
inline int atomicAdd(int *p, int v) { int o = *p; *p = o + v; return o; }
inline unsigned int atomicAdd(unsigned int *p, unsigned int v) { unsigned int o = *p; *p = o + v; return o; }
inline float atomicAdd(float *p, float v) { float o = *p; *p = o + v; return o; }
inline int atomicSub(int *p, int v) { int o = *p; *p = o - v; return o; }
inline unsigned int atomicSub(unsigned int *p, unsigned int v) { unsigned int o = *p; *p = o - v; return o; }
inline int atomicExch(int *p, int v) { int o = *p; *p = v; return o; }
inline int atomicMax(int *p, int v) { int o = *p; if (v > o) *p = v; return o; }
inline int atomicMin(int *p, int v) { int o = *p; if (v < o) *p = v; return o; }
inline int atomicCAS(int *p, int c, int v) { int o = *p; if (o == c) *p = v; return o; }

/* device intrinsics used by the reference (round-to-nearest forms are the plain ops) */
inline int __mul24(int a, int b) { return a * b; }
inline float __fmul_rn(float a, float b) { return a * b; }
inline float __fadd_rn(float a, float b) { return a + b; }
inline float __fsub_rn(float a, float b) { return a - b; }
inline float __fdividef(float a, float b) { return a / b; }
inline float __cosf(float a) { return cosf(a); }
inline float __sinf(float a) { return sinf(a); }
inline float __expf(float a) { return expf(a); }
inline float __logf(float a) { return logf(a); }
inline float rsqrtf(float a) { return 1.0f / sqrtf(a); }

/* CUDA's host/device min and max overloads, including the mixed signed/unsigned ones */
inline int min(int a, int b) { return a < b ? a : b; }
inline int max(int a, int b) { return a > b ? a : b; }
inline unsigned int min(unsigned int a, unsigned int b) { return a < b ? a : b; }
inline unsigned int max(unsigned int a, unsigned int b) { return a > b ? a : b; }
inline unsigned int min(int a, unsigned int b) { return min((unsigned int)a, b); }
inline unsigned int min(unsigned int a, int b) { return min(a, (unsigned int)b); }
inline unsigned int max(int a, unsigned int b) { return max((unsigned int)a, b); }
inline unsigned int max(unsigned int a, int b) { return max(a, (unsigned int)b); }
inline long long min(long long a, long long b) { return a < b ? a : b; }
inline long long max(long long a, long long b) { return a > b ? a : b; }
inline float min(float a, float b) { return fminf(a, b); }
inline float max(float a, float b) { return fmaxf(a, b); }
inline float min(float a, int b) { return fminf(a, (float)b); }
inline float max(float a, int b) { return fmaxf(a, (float)b); }
inline float min(int a, float b) { return fminf((float)a, b); }
inline float max(int a, float b) { return fmaxf((float)a, b); }
inline double min(double a, double b) { return fmin(a, b); }
inline double max(double a, double b) { return fmax(a, b); }
inline double min(double a, float b) { return fmin(a, (double)b); }
inline double max(double a, float b) { return fmax(a, (double)b); }
inline double min(float a, double b) { return fmin((double)a, b); }
inline double max(float a, double b) { return fmax((double)a, b); }
inline double min(double a, int b) { return fmin(a, (double)b); }
inline double max(double a, int b) { return fmax(a, (double)b); }
inline double min(int a, double b) { return fmin((double)a, b); }
inline double max(int a, double b) { return fmax((double)a, b); }

/* runtime API */
typedef int cudaError_t;
typedef int cudaError;
enum { cudaSuccess = 0, cudaErrorMemoryAllocation = 2 };
enum cudaMemcpyKind {
  cudaMemcpyHostToHost = 0,
  cudaMemcpyHostToDevice = 1,
  cudaMemcpyDeviceToHost = 2,
  cudaMemcpyDeviceToDevice = 3,
  cudaMemcpyDefault = 4
};
typedef int cudaStream_t;
typedef int cudaEvent_t;
struct cudaDeviceProp {
  char name[256];
  size_t totalGlobalMem;
  int maxThreadsPerBlock;
  int multiProcessorCount;
  int warpSize;
};

inline cudaError_t cudaMalloc(void **p, size_t bytes) {
  *p = calloc(bytes ? bytes : 1, 1);
  return *p ? cudaSuccess : cudaErrorMemoryAllocation;
}
inline cudaError_t cudaFree(void *p) { free(p); return cudaSuccess; }
inline cudaError_t cudaMemcpy(void *d, const void *s, size_t bytes, int) { memmove(d, s, bytes); return cudaSuccess; }
inline cudaError_t cudaMemset(void *d, int v, size_t bytes) { memset(d, v, bytes); return cudaSuccess; }
template <class T>
cudaError_t cudaMemcpyToSymbol(const T &sym, const void *src, size_t bytes, size_t offset = 0, int = 1) {
  memcpy((char *)&sym + offset, src, bytes);
  return cudaSuccess;
}
inline cudaError_t cudaGetLastError() { return cudaSuccess; }
inline const char *cudaGetErrorString(cudaError_t) { return "no error (host emulation)"; }
inline cudaError_t cudaThreadSynchronize() { return cudaSuccess; }
inline cudaError_t cudaDeviceSynchronize() { return cudaSuccess; }
inline cudaError_t cudaSetDevice(int) { return cudaSuccess; }
inline cudaError_t cudaGetDeviceCount(int *c) { *c = 1; return cudaSuccess; }
inline cudaError_t cudaGetDeviceProperties(cudaDeviceProp *p, int) {
  memset(p, 0, sizeof(*p));
  strcpy(p->name, "host emulation");
  p->totalGlobalMem = (size_t)1 << 38;
  p->maxThreadsPerBlock = 1024;
  p->multiProcessorCount = 152;
  p->warpSize = 32;
  return cudaSuccess;
}
inline cudaError_t cudaEventCreate(cudaEvent_t *e) { *e = 0; return cudaSuccess; }
inline cudaError_t cudaEventRecord(cudaEvent_t, int = 0) { return cudaSuccess; }
inline cudaError_t cudaEventSynchronize(cudaEvent_t) { return cudaSuccess; }
inline cudaError_t cudaEventElapsedTime(float *t, cudaEvent_t, cudaEvent_t) { *t = 0.0f; return cudaSuccess; }
inline cudaError_t cudaEventDestroy(cudaEvent_t) { return cudaSuccess; }

/* math_constants.h */
#define CUDART_PI_F 3.141592654f
#define CUDART_PI 3.1415926535897931e+0
#define CUDART_PIO2 1.5707963267948966e+0
#define CUDART_PIO2_F 1.570796327f
#define CUDART_SQRT_HALF 7.0710678118654757e-1
#define CUDART_SQRT_HALF_F 0.707106781f
#define CUDART_INF_F (__builtin_huge_valf())
#define CUDART_NAN_F (__builtin_nanf(""))
