// gb_resident.h -- the cluster-resident NIHT / HTP / CGIHT kernel (gb_resident.cu): the batched
// form's small trials and the single-trial drop-in's small dense solves.
#pragma once
#include <cuda_runtime.h>

#include <mutex>

#include "gb_internal.cuh"

// trials with n <= this go to the resident kernel unless the caller says otherwise
#define GB_RESIDENT_N_DEFAULT 8192

// One launch solving `count` NIHT, HTP or CGIHT trials, trial order[q] for q < count (indices into the
// batch tables n, m, k, tid and the result arrays, all device pointers), each by one
// cluster of CTAs.  n_cap / m_cap bound the trials' n and m; cluster = CTAs per cluster
// (0: four, or the smallest power of two above that the sizes fit).
struct GbResidentArgs {
  int count;
  const int *order;  // host array of count trial indices, largest first
  const int *n, *m, *k;
  const unsigned int *tid;
  unsigned int seed;
  float tol_rel;
  int maxiter;
  int *iters;
  float *err;
  int *ok;
  double *bytes;
  int n_cap, m_cap, cluster;
  int alg;  // GB_ALG_NIHT, GB_ALG_HTP or GB_ALG_CGIHT
  const float *ml_params;  // CGIHT from the learned warm start (device MLP parameters) or null
  int *fb;                 // with it: per trial, 1 when the warm start was abandoned
  int gfmt = 0;            // the A^T r operand (GB_GRAD_*); the buffers' format (A24 covers both)
  const unsigned char *gfmts = nullptr;  // per trial (device), or null: gfmt for all
  int rec_every = 0;       // CGIHT residual recurrence (GbState::rec_every)
};

gb_status gb_resident_enqueue(const GbResidentArgs &a, cudaStream_t s);
// CTAs per cluster the resident form uses for these sizes (0: the sizes do not fit)
int gb_resident_pick_cluster(int n_cap, int m_cap, int requested, int gb_alg, int learned = 0);
// shared memory per CTA, and the most a CTA can have
size_t gb_resident_smem(int n_cap, int m_cap, int C, int gb_alg, int learned = 0);
int gb_resident_max_smem();
// cluster size of the last resident launch on this device (0: none)
int gb_resident_last_cluster();
// held for the whole of gb_cs_solve_batch (gb_batch.cu): the engines are shared per device
std::recursive_mutex &gb_batch_mutex();
// The single-trial drop-in's dense NIHT, HTP or CGIHT (the learned warm start when w.ml_params;
// state initialised in w.st, y in w.y) on one cluster; x to w.x and the final state to w.st.  *used = 0: not eligible, nothing
// launched.
gb_status gb_resident_solve_single(GbWork &w, int gb_alg, int num_bins, cudaStream_t s, int *used);
// after a synchronisation: GB_CUDA_ERROR if a resident launch found its shared memory smaller
// than its layout (it then did nothing)
gb_status gb_resident_check();

