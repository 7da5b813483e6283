/*
 * gb_host_runtime.cpp -- the out-of-line parts of the host emulation: the fiber block
 * scheduler behind GB_LAUNCH / __syncthreads, the cuFFT stand-in's transform, and the
 * mx API stand-in.  Compiled into each reference gateway library.  TEST INFRASTRUCTURE
 * ONLY.
 *
 * Fibers: each emulated thread of a block runs on its own stack, created once with
 * makecontext and reused for later blocks; switches use _setjmp/_longjmp (no signal-mask
 * system call), which needs _FORTIFY_SOURCE off (the recipe builds with -U_FORTIFY_SOURCE).
 * A kernel whose first launch met no barrier runs its later launches as plain calls per
 * thread; if such a kernel ever reaches __syncthreads the process aborts with a message
 * (a barrier reached outside a fiber would otherwise be silently wrong).
 */
#include <setjmp.h>
#include <stdarg.h>
#include <ucontext.h>

#include <complex>
#include <map>
#include <set>
#include <string>
#include <vector>

#include "gb_host_libs.h"
#include "mex.h"

uint3 threadIdx = {0, 0, 0}, blockIdx = {0, 0, 0};
dim3 blockDim(1, 1, 1), gridDim(1, 1, 1);

namespace gbh {
namespace {

enum { F_IDLE = 0, F_RUN = 1, F_BARRIER = 2, F_DONE = 3 };
const size_t kStack = 256 * 1024;

struct Fiber {
  ucontext_t uc;
  jmp_buf jb;
  char *stack;
  int state;
};

std::vector<Fiber *> g_fibers;
jmp_buf g_sched;
ucontext_t g_main;
int g_cur = -1;           // fiber running now (-1: none)
int g_creating = -1;
bool g_direct = false;    // running a barrier-free kernel without fibers
bool g_barrier_hit = false;
const std::function<void()> *g_body = nullptr;
std::set<const void *> g_barrier_free;  // kernels whose first launch met no barrier
std::set<const void *> g_seen;
std::vector<char> g_dyn_smem(1 << 20);

void fiber_entry() {
  const int me = g_creating;
  Fiber *f = g_fibers[me];
  if (!_setjmp(f->jb)) swapcontext(&f->uc, &g_main);  // parked until the first task
  for (;;) {
    (*g_body)();
    f->state = F_DONE;
    if (!_setjmp(f->jb)) _longjmp(g_sched, 1);
  }
}

void ensure_fibers(int nt) {
  while ((int)g_fibers.size() < nt) {
    Fiber *f = new Fiber();
    f->stack = (char *)malloc(kStack);
    getcontext(&f->uc);
    f->uc.uc_stack.ss_sp = f->stack;
    f->uc.uc_stack.ss_size = kStack;
    f->uc.uc_link = nullptr;
    makecontext(&f->uc, (void (*)())fiber_entry, 0);
    g_creating = (int)g_fibers.size();
    g_fibers.push_back(f);
    swapcontext(&g_main, &f->uc);
  }
}

void set_thread(int t, const dim3 &b) {
  threadIdx.x = t % b.x;
  threadIdx.y = (t / b.x) % b.y;
  threadIdx.z = t / (b.x * b.y);
}

}  // namespace

void *dynamic_shared() { return g_dyn_smem.data(); }

void syncthreads() {
  if (g_direct || g_cur < 0) {
    fprintf(stderr, "host emulation: __syncthreads outside a fiber (a kernel believed barrier-free)\n");
    abort();
  }
  g_barrier_hit = true;
  Fiber *f = g_fibers[g_cur];
  f->state = F_BARRIER;
  if (!_setjmp(f->jb)) _longjmp(g_sched, 1);
}

void run_launch(dim3 g, dim3 b, const void *kernel, const std::function<void()> &thread) {
  const int nt = (int)(b.x * b.y * b.z);
  if (nt <= 0 || g.x * g.y * g.z == 0) return;
  const std::function<void()> *saved_body = g_body;
  gridDim = g;
  blockDim = b;
  g_body = &thread;
  const bool direct = g_barrier_free.count(kernel) != 0;
  const bool first = g_seen.insert(kernel).second;
  g_barrier_hit = false;
  if (!direct) ensure_fibers(nt);
  // the scheduler's locals live in memory (volatile): _setjmp / _longjmp restore registers
  for (volatile unsigned bz = 0; bz < g.z; ++bz)
    for (volatile unsigned by = 0; by < g.y; ++by)
      for (volatile unsigned bx = 0; bx < g.x; ++bx) {
        blockIdx.x = bx;
        blockIdx.y = by;
        blockIdx.z = bz;
        if (direct) {
          g_direct = true;
          for (int t = 0; t < nt; ++t) {
            set_thread(t, b);
            thread();
          }
          g_direct = false;
          continue;
        }
        for (int t = 0; t < nt; ++t) g_fibers[t]->state = F_RUN;
        volatile int live = nt;
        while (live > 0) {
          for (volatile int t = 0; t < nt; ++t) {
            Fiber *volatile f = g_fibers[t];
            if (f->state == F_DONE) continue;
            f->state = F_RUN;
            set_thread(t, b);
            g_cur = t;
            if (!_setjmp(g_sched)) _longjmp(f->jb, 1);
            g_cur = -1;
            if (f->state == F_DONE) --live;
          }
        }
      }
  if (first && !direct && !g_barrier_hit) g_barrier_free.insert(kernel);
  g_body = saved_body;
}

std::map<int, FftPlan> &fft_plans() {
  static std::map<int, FftPlan> plans;
  return plans;
}

void fft_c2c(const float2 *in, float2 *out, int n, int sign) {
  typedef std::complex<double> cd;
  std::vector<cd> a((size_t)n);
  for (int i = 0; i < n; ++i) a[i] = cd(in[i].x, in[i].y);
  if (n > 0 && (n & (n - 1)) == 0) {
    for (int i = 1, j = 0; i < n; ++i) {  // bit reversal
      int bit = n >> 1;
      for (; j & bit; bit >>= 1) j ^= bit;
      j ^= bit;
      if (i < j) std::swap(a[i], a[j]);
    }
    for (int len = 2; len <= n; len <<= 1) {
      const double ang = sign * 2.0 * M_PI / len;
      for (int i = 0; i < n; i += len)
        for (int k = 0; k < len / 2; ++k) {
          const cd w(std::cos(ang * k), std::sin(ang * k));
          const cd u = a[i + k], v = a[i + k + len / 2] * w;
          a[i + k] = u + v;
          a[i + k + len / 2] = u - v;
        }
    }
  } else {
    std::vector<cd> b((size_t)n);
    for (int k = 0; k < n; ++k) {
      cd s(0.0, 0.0);
      for (int j = 0; j < n; ++j) {
        const double ang = sign * 2.0 * M_PI * (double)(((long long)j * k) % n) / n;
        s += a[j] * cd(std::cos(ang), std::sin(ang));
      }
      b[k] = s;
    }
    a.swap(b);
  }
  for (int i = 0; i < n; ++i) out[i] = float2{(float)a[i].real(), (float)a[i].imag()};
}

}  // namespace gbh

/* ------------------------------------------------------------------ mx API */
struct gbmx_array {
  int cls;
  size_t m, n;
  std::vector<unsigned char> data;
  std::vector<mxArray *> cells;
};

static size_t gbmx_elem_size(int cls) {
  switch (cls) {
    case mxDOUBLE_CLASS: case mxINT64_CLASS: case mxUINT64_CLASS: return 8;
    case mxSINGLE_CLASS: case mxINT32_CLASS: case mxUINT32_CLASS: return 4;
    case mxINT16_CLASS: case mxUINT16_CLASS: case mxCHAR_CLASS: return 2;
    default: return 1;
  }
}

extern "C" {
mxArray *mxCreateNumericMatrix(size_t m, size_t n, mxClassID cls, mxComplexity) {
  mxArray *a = new gbmx_array();
  a->cls = cls;
  a->m = m;
  a->n = n;
  a->data.assign(m * n * gbmx_elem_size(cls) + 8, 0);
  return a;
}
void *mxGetData(const mxArray *a) { return (void *)a->data.data(); }
size_t mxGetM(const mxArray *a) { return a->m; }
size_t mxGetN(const mxArray *a) { return a->n; }
double mxGetScalar(const mxArray *a) {
  const void *p = a->data.data();
  switch (a->cls) {
    case mxDOUBLE_CLASS: return *(const double *)p;
    case mxSINGLE_CLASS: return *(const float *)p;
    case mxINT32_CLASS: return *(const int *)p;
    case mxUINT32_CLASS: return *(const unsigned int *)p;
    case mxINT64_CLASS: return (double)*(const long long *)p;
    default: return 0.0;
  }
}
int mxGetString(const mxArray *a, char *buf, size_t buflen) {
  if (a->cls != mxCHAR_CLASS || buflen == 0) return 1;
  const size_t len = a->m * a->n;
  const unsigned short *c = (const unsigned short *)a->data.data();
  size_t i = 0;
  for (; i < len && i + 1 < buflen; ++i) buf[i] = (char)c[i];
  buf[i] = 0;
  return i < len ? 1 : 0;
}
int mxIsCell(const mxArray *a) { return a && a->cls == mxCELL_CLASS; }
mxArray *mxGetCell(const mxArray *a, size_t index) { return index < a->cells.size() ? a->cells[index] : nullptr; }
size_t mxCalcSingleSubscript(const mxArray *a, size_t nsubs, const int *subs) {
  size_t idx = 0, stride = 1;
  for (size_t d = 0; d < nsubs; ++d) {
    idx += (size_t)subs[d] * stride;
    stride *= d == 0 ? a->m : a->n;
  }
  return idx;
}
int mexPrintf(const char *fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  const int r = vprintf(fmt, ap);
  va_end(ap);
  return r;
}

static char g_mex_error[1024];
void mexErrMsgIdAndTxt(const char *id, const char *fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  int off = snprintf(g_mex_error, sizeof g_mex_error, "%s: ", id);
  if (off < 0) off = 0;
  vsnprintf(g_mex_error + off, sizeof g_mex_error - off, fmt, ap);
  va_end(ap);
}
const char *gbmx_last_error(void) { return g_mex_error; }
void gbmx_clear_error(void) { g_mex_error[0] = 0; }

mxArray *gbmx_numeric(int cls, int m, int n, const void *data) {
  mxArray *a = mxCreateNumericMatrix(m, n, (mxClassID)cls, mxREAL);
  if (data) memcpy(a->data.data(), data, (size_t)m * n * gbmx_elem_size(cls));
  return a;
}
mxArray *gbmx_string(const char *s) {
  const size_t len = strlen(s);
  mxArray *a = mxCreateNumericMatrix(1, len, mxCHAR_CLASS, mxREAL);
  unsigned short *c = (unsigned short *)a->data.data();
  for (size_t i = 0; i < len; ++i) c[i] = (unsigned char)s[i];
  return a;
}
mxArray *gbmx_cell(int m, int n) {
  mxArray *a = new gbmx_array();
  a->cls = mxCELL_CLASS;
  a->m = m;
  a->n = n;
  a->cells.assign((size_t)m * n, nullptr);
  return a;
}
void gbmx_cell_set(mxArray *cell, int index, mxArray *elem) { cell->cells.at(index) = elem; }
int gbmx_class(const mxArray *a) { return a->cls; }
void gbmx_free(mxArray *a) {
  if (!a) return;
  for (mxArray *c : a->cells) gbmx_free(c);
  delete a;
}
}
