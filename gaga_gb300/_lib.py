"""ctypes binding of libgb_cs.so (declarations mirror include/gb_cs.h).

The library is the only compute path: importing this module fails loudly when the
CUDA extension has not been built (run ``__graft_entry__.build()`` or
``python gaga_gb300/build.py``).
"""
import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "lib", "libgb_cs.so")

GB_OK, GB_BAD_ARG, GB_OOM, GB_WATCHDOG, GB_CUDA_ERROR, GB_UNSUPPORTED, GB_NO_DEVICE = range(7)
STATUS_NAMES = {0: "GB_OK", 1: "GB_BAD_ARG", 2: "GB_OOM", 3: "GB_WATCHDOG", 4: "GB_CUDA_ERROR",
                5: "GB_UNSUPPORTED", 6: "GB_NO_DEVICE"}
GB_OP_DENSE, GB_OP_DCT, GB_OP_SMV = 0, 1, 2
GB_HOST, GB_DEVICE = 0, 1
GB_ALG_NIHT, GB_ALG_HTP, GB_ALG_IHT, GB_ALG_HT_SD, GB_ALG_HT_CG, GB_ALG_CSMPSP, GB_ALG_CGIHT = 0, 1, 2, 3, 4, 5, 6
GB_ALG_FIHT, GB_ALG_ALPS, GB_ALG_CGIHT_PROJ, GB_ALG_PARALLEL_L0 = 7, 8, 9, 14

# every symbol include/gb_cs.h declares
EXPORTS = ["gb_cs_version", "gb_cs_last_error", "gb_cs_default_options", "gb_cs_alg_id", "gb_cs_solve",
           "gb_cs_generate_and_solve", "gb_cs_linear_binning", "gb_cs_find_support_set", "gb_cs_find_support_set_sort",
           "gb_cs_operator_apply", "gb_cs_operator_time", "gb_cs_l0_step", "gb_cs_solve_batch", "gb_cs_batch_last_stats",
           "gb_cs_batch_last_cluster",
           "gb_cs_dense_apply_noalloc", "gb_cs_solve_shared_batch", "gb_cs_shared_last_stats",
           "gb_cs_shared_last_fallbacks",
           "gb_cs_gemm_bf16_tn", "gb_cs_mlp_num_params", "gb_cs_mlp_features", "gb_cs_mlp_forward",
           "gb_cs_mlp_grad", "gb_cs_mlp_train", "gb_cs_write_result"]


class Options(C.Structure):
    _fields_ = [("tol", C.c_float), ("tol_is_relative", C.c_int), ("maxiter", C.c_int), ("num_bins", C.c_int),
                ("restart_flag", C.c_int), ("l0_thresh", C.c_int), ("vec_distribution", C.c_int),
                ("matrix_ensemble", C.c_int), ("k_fixed", C.c_int), ("seed", C.c_uint), ("noise", C.c_float),
                ("gpu_number", C.c_int), ("conv_rate_num", C.c_int), ("alpha", C.c_float),
                ("support_flag", C.c_int), ("timing", C.c_int), ("learned_params", C.c_void_p),
                ("results_dir", C.c_char_p), ("proj_frac_tol", C.c_float), ("watchdog_passes", C.c_int)]


class Problem(C.Structure):
    _fields_ = [("kind", C.c_int), ("m", C.c_int), ("n", C.c_int), ("k", C.c_int), ("y", C.c_void_p),
                ("A", C.c_void_p), ("lda", C.c_int), ("rows", C.c_void_p), ("cols", C.c_void_p),
                ("vals", C.c_void_p), ("d", C.c_int), ("index_base", C.c_int), ("location", C.c_int),
                ("stream", C.c_void_p)]


class Result(C.Structure):
    _fields_ = [("iter", C.c_int), ("conv_rate", C.c_float), ("norms", C.c_float * 3), ("times", C.c_float * 3),
                ("support", C.c_int * 4), ("k_used", C.c_int), ("resid_prev", C.c_float * 16),
                ("stop_reason", C.c_int), ("res_record", C.c_void_p), ("warm_start", C.c_int),
                ("time_per_iteration", C.c_void_p), ("time_supp_set", C.c_void_p),
                ("cg_per_iteration", C.c_void_p), ("time_for_cg", C.c_void_p), ("time_record", C.c_void_p)]


class BinState(C.Structure):
    _fields_ = [("num_bins", C.c_int), ("max_bin", C.c_int), ("k_bin", C.c_int), ("sum", C.c_int),
                ("alpha", C.c_float), ("min_val", C.c_float)]


class Batch(C.Structure):
    _fields_ = [("ntrials", C.c_int), ("n", C.c_void_p), ("m", C.c_void_p), ("k", C.c_void_p),
                ("trial_id", C.c_void_p), ("seed", C.c_uint), ("alg", C.c_int), ("tol_rel", C.c_float),
                ("maxiter", C.c_int), ("use_learned", C.c_int), ("learned_params", C.c_void_p),
                ("slots", C.c_int), ("sm_share", C.c_int), ("stream", C.c_void_p), ("resident_n", C.c_int),
                ("cluster", C.c_int), ("grad_format", C.c_int), ("grad_formats", C.c_void_p),
                ("av_rows", C.c_int), ("residual_refresh", C.c_int)]


class SharedBatch(C.Structure):
    _fields_ = [("ntrials", C.c_int), ("m", C.c_int), ("n", C.c_int), ("k", C.c_void_p), ("seed", C.c_uint),
                ("first_trial", C.c_uint),
                ("tol_rel", C.c_float), ("maxiter", C.c_int), ("precision", C.c_int), ("d_A_out", C.c_void_p), ("d_Y_out", C.c_void_p),
                ("d_X0_out", C.c_void_p), ("stream", C.c_void_p), ("alg", C.c_int), ("learned_params", C.c_void_p),
                ("d_X_out", C.c_void_p)]


_lib = None


def load():
    """Load libgb_cs.so; raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError("libgb_cs.so is not built (%s); run `python gaga_gb300/build.py`" % LIB_PATH)
    L = C.CDLL(LIB_PATH)
    vp, i, f = C.c_void_p, C.c_int, C.c_float
    L.gb_cs_version.restype = C.c_char_p
    L.gb_cs_last_error.restype = C.c_char_p
    L.gb_cs_default_options.argtypes = [C.POINTER(Options), C.c_char_p, i]
    L.gb_cs_alg_id.argtypes = [C.c_char_p]
    L.gb_cs_alg_id.restype = i
    L.gb_cs_solve.argtypes = [C.c_char_p, C.POINTER(Problem), C.POINTER(Options), vp, C.POINTER(Result)]
    L.gb_cs_solve.restype = i
    L.gb_cs_generate_and_solve.argtypes = [C.c_char_p, i, i, i, i, i, C.POINTER(Options), vp, vp,
                                           C.POINTER(Result)]
    L.gb_cs_generate_and_solve.restype = i
    L.gb_cs_linear_binning.argtypes = [vp, i, i, i, f, f, vp, vp, vp]
    L.gb_cs_linear_binning.restype = i
    L.gb_cs_find_support_set.argtypes = [vp, i, i, f, f, f, C.POINTER(BinState), vp, vp, i, vp]
    L.gb_cs_find_support_set.restype = i
    L.gb_cs_find_support_set_sort.argtypes = [vp, vp, i, i, f, f, C.POINTER(C.c_float), vp]
    L.gb_cs_find_support_set_sort.restype = i
    L.gb_cs_operator_apply.argtypes = [C.POINTER(Problem), i, vp, vp]
    L.gb_cs_operator_apply.restype = i
    L.gb_cs_operator_time.argtypes = [C.POINTER(Problem), i, vp, vp, i, i, vp, C.c_size_t, C.POINTER(C.c_float)]
    L.gb_cs_operator_time.restype = i
    L.gb_cs_l0_step.argtypes = [vp, vp, vp, vp, i, i, i, i, i, C.POINTER(C.c_int), vp]
    L.gb_cs_l0_step.restype = i
    L.gb_cs_solve_batch.argtypes = [C.POINTER(Batch), vp, vp, vp, C.POINTER(C.c_int)]
    L.gb_cs_solve_batch.restype = i
    L.gb_cs_batch_last_stats.argtypes = [C.POINTER(C.c_double), C.POINTER(C.c_float)]
    L.gb_cs_batch_last_stats.restype = None
    L.gb_cs_batch_last_cluster.argtypes = []
    L.gb_cs_batch_last_cluster.restype = i
    L.gb_cs_dense_apply_noalloc.argtypes = [vp, i, i, i, i, vp, vp, vp]
    L.gb_cs_dense_apply_noalloc.restype = i
    L.gb_cs_solve_shared_batch.argtypes = [C.POINTER(SharedBatch), vp, vp, vp, C.POINTER(C.c_int)]
    L.gb_cs_solve_shared_batch.restype = i
    L.gb_cs_shared_last_stats.argtypes = [C.POINTER(C.c_double), C.POINTER(C.c_float)]
    L.gb_cs_shared_last_stats.restype = None
    L.gb_cs_shared_last_fallbacks.argtypes = []
    L.gb_cs_shared_last_fallbacks.restype = i
    L.gb_cs_gemm_bf16_tn.argtypes = [vp, vp, vp, i, i, i, vp, vp, vp]
    L.gb_cs_gemm_bf16_tn.restype = i
    L.gb_cs_mlp_num_params.argtypes = []
    L.gb_cs_mlp_num_params.restype = i
    L.gb_cs_mlp_features.argtypes = [vp, i, i, i, vp, vp]
    L.gb_cs_mlp_features.restype = i
    L.gb_cs_mlp_forward.argtypes = [vp, vp, i, vp, vp]
    L.gb_cs_mlp_forward.restype = i
    L.gb_cs_mlp_grad.argtypes = [vp, vp, vp, i, vp, vp, vp]
    L.gb_cs_mlp_grad.restype = i
    L.gb_cs_mlp_train.argtypes = [vp, vp, vp, i, i, i, f, C.c_uint, vp, vp]
    L.gb_cs_mlp_train.restype = i
    L.gb_cs_write_result.argtypes = [C.c_char_p, C.c_char_p, i, i, i, i, i, C.POINTER(Options), C.POINTER(Result),
                                     C.c_char_p, i]
    L.gb_cs_write_result.restype = i
    _lib = L
    return L


class GagaError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__("%s: %s" % (STATUS_NAMES.get(status, status), msg))
        self.status = status


def check(status):
    if status != GB_OK:
        raise GagaError(status, load().gb_cs_last_error().decode(errors="replace"))
