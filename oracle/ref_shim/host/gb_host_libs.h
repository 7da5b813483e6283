/*
 * gb_host_libs.h -- CPU restatements of the closed NVIDIA libraries the reference calls,
 * for the host emulation in gb_host_cuda.h.  TEST INFRASTRUCTURE ONLY.
 *
 *  cuBLAS v1 (legacy cublas.h, as the reference uses it): Scopy, Saxpy (fused
 *    multiply-add per element, as a GPU computes alpha*x+y), Sscal, Sdot / Snrm2 / Sasum
 *    (accumulated in double and rounded once: cuBLAS fixes no summation order, so the
 *    stand-in uses the most accurate cheap one), Isamax (1-based index of the first
 *    largest |x|, the BLAS definition).
 *  cuFFT: unnormalised complex-to-complex transforms of `batch` contiguous sequences,
 *    forward sign -1, computed in double and rounded to float once per output
 *    (radix-2 for power-of-two lengths, a direct DFT otherwise).
 *  cuRAND: a seeded counter-based generator (splitmix64 -> uniform (0,1], Box-Muller) with
 *    cuRAND's call signatures; the streams differ from cuRAND's (which are closed), so
 *    only the given-data usages of the gateways are used for fixtures.
 *  Thrust: device_ptr over host memory; sort, sort_by_key, reduce, max_element, count.
 */
#pragma once
#include <complex>
#include <map>
#include <vector>

#include "gb_host_cuda.h"

/* ------------------------------------------------------------------ cuBLAS v1 */
/* GBH_TRACE=1 in the environment prints every reduction's result (a debugging aid) */
namespace gbh {
inline bool trace_on() {
  static const int on = getenv("GBH_TRACE") ? atoi(getenv("GBH_TRACE")) : 0;
  return on != 0;
}
}  // namespace gbh
typedef int cublasStatus;
#define CUBLAS_STATUS_SUCCESS 0
inline cublasStatus cublasInit() { return CUBLAS_STATUS_SUCCESS; }
inline cublasStatus cublasShutdown() { return CUBLAS_STATUS_SUCCESS; }
inline cublasStatus cublasGetError() { return CUBLAS_STATUS_SUCCESS; }
inline void cublasScopy(int n, const float *x, int incx, float *y, int incy) {
  for (int i = 0; i < n; ++i) y[(size_t)i * incy] = x[(size_t)i * incx];
}
inline void cublasSaxpy(int n, float alpha, const float *x, int incx, float *y, int incy) {
  for (int i = 0; i < n; ++i) y[(size_t)i * incy] = fmaf(alpha, x[(size_t)i * incx], y[(size_t)i * incy]);
}
inline void cublasSscal(int n, float alpha, float *x, int incx) {
  for (int i = 0; i < n; ++i) x[(size_t)i * incx] *= alpha;
}
inline float cublasSdot(int n, const float *x, int incx, const float *y, int incy) {
  double s = 0.0;
  for (int i = 0; i < n; ++i) s += (double)x[(size_t)i * incx] * (double)y[(size_t)i * incy];
  if (gbh::trace_on()) fprintf(stderr, "Sdot n=%d %.9g\n", n, (float)s);
  return (float)s;
}
inline float cublasSnrm2(int n, const float *x, int incx) {
  double s = 0.0;
  for (int i = 0; i < n; ++i) s += (double)x[(size_t)i * incx] * (double)x[(size_t)i * incx];
  if (gbh::trace_on()) fprintf(stderr, "Snrm2 n=%d %.9g\n", n, (float)std::sqrt(s));
  return (float)std::sqrt(s);
}
inline float cublasSasum(int n, const float *x, int incx) {
  double s = 0.0;
  for (int i = 0; i < n; ++i) s += std::fabs((double)x[(size_t)i * incx]);
  return (float)s;
}
inline int cublasIsamax(int n, const float *x, int incx) {
  if (n < 1 || incx < 1) return 0;
  int best = 0;
  float bv = std::fabs(x[0]);
  for (int i = 1; i < n; ++i) {
    const float v = std::fabs(x[(size_t)i * incx]);
    if (v > bv) { bv = v; best = i; }
  }
  if (gbh::trace_on()) fprintf(stderr, "Isamax n=%d %d (%.9g)\n", n, best + 1, bv);
  return best + 1;
}

/* ------------------------------------------------------------------ cuFFT */
typedef int cufftHandle;
typedef float2 cufftComplex;
typedef int cufftResult;
typedef int cufftType;
#define CUFFT_SUCCESS 0
#define CUFFT_C2C 0x29
#define CUFFT_FORWARD -1
#define CUFFT_INVERSE 1
namespace gbh {
struct FftPlan { int nx, batch; };
std::map<int, FftPlan> &fft_plans();
void fft_c2c(const float2 *in, float2 *out, int n, int sign);
}  // namespace gbh
inline cufftResult cufftPlan1d(cufftHandle *plan, int nx, cufftType, int batch) {
  static int next = 1;
  *plan = next++;
  gbh::fft_plans()[*plan] = gbh::FftPlan{nx, batch};
  return CUFFT_SUCCESS;
}
inline cufftResult cufftExecC2C(cufftHandle plan, cufftComplex *in, cufftComplex *out, int dir) {
  const gbh::FftPlan p = gbh::fft_plans().at(plan);
  for (int b = 0; b < p.batch; ++b) gbh::fft_c2c(in + (size_t)b * p.nx, out + (size_t)b * p.nx, p.nx, dir);
  return CUFFT_SUCCESS;
}
inline cufftResult cufftDestroy(cufftHandle plan) {
  gbh::fft_plans().erase(plan);
  return CUFFT_SUCCESS;
}

/* ------------------------------------------------------------------ cuRAND */
typedef int curandStatus_t;
typedef int curandRngType_t;
struct gbh_curand_gen { unsigned long long seed, counter; };
typedef gbh_curand_gen *curandGenerator_t;
#define CURAND_STATUS_SUCCESS 0
#define CURAND_RNG_PSEUDO_DEFAULT 100
namespace gbh {
inline unsigned long long splitmix64(unsigned long long z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
inline double uniform01(curandGenerator_t g) {  // (0, 1]
  const unsigned long long r = splitmix64(g->seed * 0x100000001B3ull + g->counter++);
  return ((double)(r >> 11) + 1.0) * (1.0 / 9007199254740992.0);
}
}  // namespace gbh
inline curandStatus_t curandCreateGenerator(curandGenerator_t *g, curandRngType_t) {
  *g = new gbh_curand_gen{0, 0};
  return CURAND_STATUS_SUCCESS;
}
inline curandStatus_t curandDestroyGenerator(curandGenerator_t g) { delete g; return CURAND_STATUS_SUCCESS; }
inline curandStatus_t curandSetPseudoRandomGeneratorSeed(curandGenerator_t g, unsigned long long seed) {
  g->seed = seed;
  g->counter = 0;
  return CURAND_STATUS_SUCCESS;
}
inline curandStatus_t curandGenerateUniform(curandGenerator_t g, float *out, size_t n) {
  for (size_t i = 0; i < n; ++i) out[i] = (float)gbh::uniform01(g);
  return CURAND_STATUS_SUCCESS;
}
inline curandStatus_t curandGenerateNormal(curandGenerator_t g, float *out, size_t n, float mean, float sd) {
  for (size_t i = 0; i < n; i += 2) {
    const double u1 = gbh::uniform01(g), u2 = gbh::uniform01(g);
    const double r = std::sqrt(-2.0 * std::log(u1)), t = 6.283185307179586 * u2;
    out[i] = (float)(mean + sd * r * std::cos(t));
    if (i + 1 < n) out[i + 1] = (float)(mean + sd * r * std::sin(t));
  }
  return CURAND_STATUS_SUCCESS;
}

/* ------------------------------------------------------------------ Thrust */
namespace thrust {
template <class T>
struct device_ptr {
  T *p;
  device_ptr() : p(nullptr) {}
  explicit device_ptr(T *q) : p(q) {}
  T &operator*() const { return *p; }
  T &operator[](ptrdiff_t i) const { return p[i]; }
  device_ptr operator+(ptrdiff_t i) const { return device_ptr(p + i); }
  device_ptr operator-(ptrdiff_t i) const { return device_ptr(p - i); }
  ptrdiff_t operator-(const device_ptr &o) const { return p - o.p; }
  T *get() const { return p; }
};
template <class T>
struct plus {
  T operator()(const T &a, const T &b) const { return a + b; }
};
template <class T>
struct greater {
  bool operator()(const T &a, const T &b) const { return a > b; }
};
template <class T>
void sort(device_ptr<T> a, device_ptr<T> b) { std::sort(a.p, b.p); }
template <class T, class C>
void sort(device_ptr<T> a, device_ptr<T> b, C c) { std::sort(a.p, b.p, c); }
template <class K, class V>
void sort_by_key(device_ptr<K> a, device_ptr<K> b, device_ptr<V> v) {
  const ptrdiff_t n = b.p - a.p;
  std::vector<std::pair<K, V>> kv((size_t)n);
  for (ptrdiff_t i = 0; i < n; ++i) kv[i] = {a.p[i], v.p[i]};
  std::stable_sort(kv.begin(), kv.end(), [](const std::pair<K, V> &x, const std::pair<K, V> &y) { return x.first < y.first; });
  for (ptrdiff_t i = 0; i < n; ++i) { a.p[i] = kv[i].first; v.p[i] = kv[i].second; }
}
template <class T, class I, class Op>
I reduce(device_ptr<T> a, device_ptr<T> b, I init, Op op) {
  for (T *q = a.p; q != b.p; ++q) init = op(init, *q);
  return init;
}
template <class T>
device_ptr<T> max_element(device_ptr<T> a, device_ptr<T> b) { return device_ptr<T>(std::max_element(a.p, b.p)); }
template <class T, class V>
ptrdiff_t count(device_ptr<T> a, device_ptr<T> b, const V &v) { return std::count(a.p, b.p, (T)v); }
template <class T>
T *raw_pointer_cast(device_ptr<T> d) { return d.p; }
template <class T>
device_ptr<T> device_pointer_cast(T *p) { return device_ptr<T>(p); }
}  // namespace thrust
