/*
 * ref_driver.cpp -- runs reference kernels and host routines on the CPU through
 * cuda_host_shim.h.  The reference sources are #included from the reference tree,
 * unmodified (include path set by oracle/build.py).  TEST INFRASTRUCTURE ONLY:
 * used to write tests/golden fixtures and to pin the oracle.
 *
 * Every launch uses blockDim = 1 and gridDim = number of work items, so that each
 * emulated thread index is in range (LinearBinning reads vec[xIndex] before its
 * bounds check, GAGA/gaga/kernels.cu:138).
 */
#include "cuda_host_shim.h"

gb_dim3 threadIdx = {0, 0, 0}, blockIdx = {0, 0, 0}, blockDim = {1, 1, 1}, gridDim = {1, 1, 1};

#include "kernels.cu"            /* GAGA/gaga/kernels.cu */
#include "expander/kernels.cu"   /* GAGA/gaga/expander/kernels.cu */
#include "expander/serial_l0.cu" /* GAGA/gaga/expander/serial_l0.cu */

template <class F> static void launch1d(int items, F f) {
  blockDim = {1, 1, 1};
  gridDim = {(unsigned)items, 1, 1};
  threadIdx = {0, 0, 0};
  for (int b = 0; b < items; ++b) {
    blockIdx = {(unsigned)b, 0, 0};
    f();
  }
}

extern "C" {

void ref_linear_binning(float *vec, int *bin, int *counters, int num_bins, int max_bin, int n,
                        float slope, float intercept) {
  launch1d(n, [&] { LinearBinning(vec, bin, counters, num_bins, max_bin, n, slope, intercept); });
}

void ref_threshold(float *vec, int *bin, int k_bin, int n) {
  launch1d(n, [&] { threshold(vec, bin, k_bin, n); });
}

void ref_threshold_one(float *vec, float *vec_thres, int *bin, int k_bin, int n) {
  launch1d(n, [&] { threshold_one(vec, vec_thres, bin, k_bin, n); });
}

int ref_check_support_evolution(int *bin, int *bin_prev, int k_bin, int k_bin_prev, int n) {
  int flag = 0;
  launch1d(n, [&] { checkSupportEvolution(bin, bin_prev, k_bin, k_bin_prev, &flag, n); });
  return flag;
}

int ref_l0_scores(float *scores, float *res, float *vec, float *updates, int *rows, int n, int d,
                  int thresh, int shift) {
  int found = 0;
  launch1d(n, [&] { cuda_compute_scores_l0(scores, res, vec, updates, rows, &found, n, d, thresh, shift); });
  return found;
}

void ref_update_residual(float *res, int *rows, float *updates, int n, int d) {
  launch1d(n, [&] { cuda_update_residual(res, rows, updates, n, d); });
}

int ref_serial_l0(float *vec, float *y, float *res, int *rows, int *cols, int n, int m, int k, int d,
                  int alpha, float tol, int maxiter, float *res_record, float *time_record) {
  int iter = 0;
  /* serial_l0 reads timeRecord[-1] on its first pass (serial_l0.cu:148); give it a
   * slot in front of the caller's array */
  serial_l0(vec, y, res, rows, cols, n, m, k, d, alpha, tol, maxiter, &iter, res_record, time_record + 1);
  return iter;
}
}
