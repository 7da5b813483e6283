// gb_batch.cu -- batched multi-trial form (see gb_cs_solve_batch in include/gb_cs.h).
#include "gb_internal.cuh"

extern "C" gb_status gb_cs_solve_batch(const gb_batch *b, int *iters_out, float *rel_err_out, int *success_out,
                                       int *num_success) {
  (void)b; (void)iters_out; (void)rel_err_out; (void)success_out; (void)num_success;
  gb_set_error_message("batched form not built", __FILE__, __LINE__);
  return GB_UNSUPPORTED;
}
