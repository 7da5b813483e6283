"""ctypes binding of the CPU oracle (oracle/gbo.c).  Test infrastructure only."""
import ctypes as C
import os

import numpy as np

from . import build as _build

NIHT, HTP, IHT, HT_SD, HT_CG, CSMPSP, CGIHT, FIHT, ALPS, CGIHT_PROJ, PARALLEL_L0, SERIAL_L0 = (0, 1, 2, 3, 4, 5, 6, 7, 8,
                                                                                        9, 14, 15)
PARALLEL_LDDSR, PARALLEL_L0_SWIPE, SMP = 13, 18, 10
OP_DENSE, OP_DCT, OP_SMV = 0, 1, 2
ALG_IDS = {"NIHT": NIHT, "HTP": HTP, "IHT": IHT, "ThresholdSD": HT_SD, "ThresholdCG": HT_CG, "CSMPSP": CSMPSP,
           "CGIHT": CGIHT, "FIHT": FIHT, "ALPS": ALPS, "CGIHTprojected": CGIHT_PROJ,
           "parallel_l0": PARALLEL_L0, "serial_l0": SERIAL_L0}

_lib = None


def lib():
    global _lib
    if _lib is None:
        path = _build.build_oracle()
        _lib = C.CDLL(path)
        _declare(_lib)
    return _lib


class GboOp(C.Structure):
    _fields_ = [("kind", C.c_int), ("m", C.c_int), ("n", C.c_int), ("A", C.c_void_p), ("lda", C.c_int),
                ("dct_rows", C.c_void_p), ("smv_rows", C.c_void_p), ("smv_vals", C.c_void_p), ("d", C.c_int)]


class GboOpts(C.Structure):
    _fields_ = [("alg", C.c_int), ("tol", C.c_float), ("maxiter", C.c_int), ("num_bins", C.c_int),
                ("restart", C.c_int), ("l0_thresh", C.c_int), ("threads", C.c_int), ("proj_frac_tol", C.c_float),
                ("timing", C.c_int), ("supp_flag", C.c_int), ("alpha", C.c_float)]


class GboInfo(C.Structure):
    _fields_ = [("iter", C.c_int), ("sum", C.c_int), ("conv_rate", C.c_float),
                ("resid_prev", C.c_float * 16), ("k_bin", C.c_int), ("ucg_steps", C.c_int), ("rcg_steps", C.c_int)]


class GboBinState(C.Structure):
    _fields_ = [("num_bins", C.c_int), ("max_bin", C.c_int), ("k_bin", C.c_int), ("sum", C.c_int),
                ("alpha", C.c_float), ("min_val", C.c_float)]


def _p(a):
    return C.c_void_p(a.ctypes.data) if a is not None else C.c_void_p(0)


def _declare(L):
    vp, i, f, u = C.c_void_p, C.c_int, C.c_float, C.c_uint32
    sig = {
        "gbo_philox4x32_10": (None, [vp, vp, vp]),
        "gbo_gen_dense": (None, [i, i, i, i, u, u, vp]),
        "gbo_gen_vector": (i, [i, i, i, u, u, vp]),
        "gbo_gen_dct_rows": (None, [i, i, u, u, vp]),
        "gbo_gen_smv": (None, [i, i, i, i, u, u, vp, vp]),
        "gbo_A": (None, [vp, vp, vp]),
        "gbo_AT": (None, [vp, vp, vp]),
        "gbo_dct2": (None, [i, vp, vp]),
        "gbo_dct3": (None, [i, vp, vp]),
        "gbo_linear_binning": (None, [vp, i, i, i, f, f, vp, vp]),
        "gbo_find_support_set": (i, [vp, vp, vp, f, f, f, vp, i, i]),
        "gbo_threshold": (None, [vp, vp, i, i]),
        "gbo_find_support_set_sort": (f, [vp, vp, f, f, vp, i, i]),
        "gbo_max_magnitude": (f, [vp, i]),
        "gbo_solve": (i, [vp, vp, i, vp, vp, vp]),
        "gbo_parallel_l0": (i, [vp, vp, vp, vp, vp, vp, vp]),
        "gbo_serial_l0": (i, [vp, vp, vp, vp, vp, vp, vp]),
        "gbo_smp": (i, [vp, vp, i, vp, vp, vp, vp, vp]),
        "gbo_seq_decode": (i, [vp, vp, i, vp, i, vp, vp, vp, vp]),
        "gbo_l0_scores": (None, [vp, vp, vp, vp, i, i, i, i, vp]),
        "gbo_l0_update_residual": (None, [vp, vp, vp, i, i]),
        "gbo_results": (None, [vp, vp, i, i, vp, vp]),
        "gbo_solve_dense_trials": (i, [i, vp, vp, vp, u, vp, i, f, i, i, vp, vp]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args


def f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


class Op:
    """Operator handle keeping its numpy buffers alive."""

    def __init__(self, kind, m, n, A=None, lda=None, dct_rows=None, smv_rows=None, smv_vals=None, d=0):
        self.kind, self.m, self.n, self.d = kind, m, n, d
        self.A = None if A is None else f32(A)
        self.lda = lda if lda is not None else m
        self.dct_rows = None if dct_rows is None else i32(dct_rows)
        self.smv_rows = None if smv_rows is None else i32(smv_rows)
        self.smv_vals = None if smv_vals is None else f32(smv_vals)
        self.c = GboOp(kind, m, n, _p(self.A), self.lda, _p(self.dct_rows), _p(self.smv_rows),
                       _p(self.smv_vals), d)

    @staticmethod
    def dense(A_colmajor, m, n, lda=None):
        return Op(OP_DENSE, m, n, A=A_colmajor, lda=lda)

    @staticmethod
    def dct(n, rows):
        return Op(OP_DCT, len(rows), n, dct_rows=rows)

    @staticmethod
    def smv(m, n, d, rows, vals):
        return Op(OP_SMV, m, n, smv_rows=rows, smv_vals=vals, d=d)


# ---------------- generation ----------------
def gen_dense(m, n, seed, trial=0, ens=1, lda=None):
    """Column-major dense matrix, returned as a flat float32 array of length lda*n."""
    lda = lda or m
    A = np.empty(lda * n, dtype=np.float32)
    lib().gbo_gen_dense(m, n, lda, ens, seed, trial, _p(A))
    return A


def gen_vector(n, k, vec_dist, seed, trial=0):
    x = np.zeros(n, dtype=np.float32)
    ks = lib().gbo_gen_vector(n, k, vec_dist, seed, trial, _p(x))
    return x, ks


def gen_dct_rows(n, m, seed, trial=0):
    rows = np.empty(m, dtype=np.int32)
    lib().gbo_gen_dct_rows(n, m, seed, trial, _p(rows))
    return rows


def gen_smv(m, n, d, ens, seed, trial=0):
    rows = np.empty(n * d, dtype=np.int32)
    vals = np.empty(n * d, dtype=np.float32)
    lib().gbo_gen_smv(m, n, d, ens, seed, trial, _p(rows), _p(vals))
    return rows, vals


# ---------------- operators ----------------
def A(op, x):
    x = f32(x)
    y = np.empty(op.m, dtype=np.float32)
    lib().gbo_A(C.byref(op.c), _p(x), _p(y))
    return y


def AT(op, r):
    r = f32(r)
    g = np.empty(op.n, dtype=np.float32)
    lib().gbo_AT(C.byref(op.c), _p(r), _p(g))
    return g


def dct2(x):
    x = f32(x)
    out = np.empty_like(x)
    lib().gbo_dct2(len(x), _p(x), _p(out))
    return out


def dct3(x):
    x = f32(x)
    out = np.empty_like(x)
    lib().gbo_dct3(len(x), _p(x), _p(out))
    return out


# ---------------- support selection ----------------
def linear_binning(v, num_bins, max_bin, slope, intercept):
    v = f32(v)
    bins = np.zeros(len(v), dtype=np.int32)
    cnt = np.zeros(num_bins, dtype=np.int32)
    lib().gbo_linear_binning(_p(v), len(v), num_bins, max_bin, slope, intercept, _p(bins), _p(cnt))
    return bins, cnt


def find_support_set(v, k, num_bins, slope, intercept, max_change, state=None, bins=None):
    """One FindSupportSet call.  ``state`` is a GboBinState (created on first use)."""
    v = f32(v)
    if state is None:
        alpha = np.float32(0.25)
        state = GboBinState(num_bins, int(np.float32(num_bins) * (np.float32(1.0) - alpha)), 0, 0,
                            float(alpha), 0.0)
    if bins is None:
        bins = np.zeros(len(v), dtype=np.int32)
    cnt = np.zeros(num_bins, dtype=np.int32)
    s = lib().gbo_find_support_set(_p(v), _p(bins), _p(cnt), slope, intercept, max_change,
                                   C.byref(state), len(v), k)
    return s, bins, cnt, state


def find_support_set_sort(v, bins, T, max_change, k):
    """One FindSupportSet_sort call on copies of v and bins: (v, bins, T)."""
    v = f32(v).copy()
    bins = np.ascontiguousarray(bins, dtype=np.int32).copy()
    buf = np.zeros(len(v), dtype=np.float32)
    T = lib().gbo_find_support_set_sort(_p(v), _p(bins), T, max_change, _p(buf), len(v), k)
    return v, bins, np.float32(T)


def max_magnitude(v):
    v = f32(v)
    return lib().gbo_max_magnitude(_p(v), len(v))


# ---------------- solvers ----------------
def default_num_bins(n):
    return max(n // 20, 1000)


def solve(alg, op, y, k, tol, maxiter=None, num_bins=None, restart=0, threads=0, proj_frac_tol=3.0, timing=0,
          supp_flag=0, alpha=0.25):
    alg_id = ALG_IDS[alg] if isinstance(alg, str) else alg
    if maxiter is None:
        maxiter = 300 if alg_id == HTP else 5000
    num_bins = num_bins or default_num_bins(op.n)
    y = f32(y)
    x = np.zeros(op.n, dtype=np.float32)
    o = GboOpts(alg_id, tol, maxiter, num_bins, restart, 1, threads, proj_frac_tol, timing, supp_flag, alpha)
    info = GboInfo()
    lib().gbo_solve(C.byref(op.c), _p(y), k, C.byref(o), _p(x), C.byref(info))
    return x, info


def smp(op, y, k, tol, maxiter, num_bins=None):
    """Sparse matching pursuit (smp) on an expander operator."""
    y = f32(y)
    x = np.zeros(op.n, dtype=np.float32)
    res = np.zeros(op.m, dtype=np.float32)
    rec = np.zeros(maxiter + 1, dtype=np.float32)
    o = GboOpts(SMP, tol, maxiter, num_bins or default_num_bins(op.n), 0, 1, 0)
    info = GboInfo()
    lib().gbo_smp(C.byref(op.c), _p(y), int(k), C.byref(o), _p(x), _p(res), _p(rec), C.byref(info))
    return x, res, rec, info


SEQ_VARIANTS = {"ssmp": 0, "er": 1, "ssmp_naive": 2, "er_naive": 3}


def seq_decode(alg, op, y, k, tol, maxiter, num_bins=None):
    """The sequential expander decoders ssmp, er, ssmp_naive, er_naive."""
    y = f32(y)
    x = np.zeros(op.n, dtype=np.float32)
    res = np.zeros(op.m, dtype=np.float32)
    rec = np.zeros(maxiter + 1, dtype=np.float32)
    o = GboOpts(0, tol, maxiter, num_bins or default_num_bins(op.n), 0, 1, 0)
    info = GboInfo()
    rc = lib().gbo_seq_decode(C.byref(op.c), _p(y), int(k), C.byref(o), SEQ_VARIANTS[alg], _p(x), _p(res), _p(rec),
                              C.byref(info))
    if rc != 0:
        raise ValueError("gbo_seq_decode: unsupported arguments")
    return x, res, rec, info


def parallel_l0(op, y, tol, maxiter, l0_thresh=1, variant="parallel_l0"):
    """parallel_l0, or its variants parallel_lddsr / parallel_l0_swipe."""
    y = f32(y)
    x = np.zeros(op.n, dtype=np.float32)
    res = np.zeros(op.m, dtype=np.float32)
    rec = np.zeros(maxiter + 1, dtype=np.float32)
    alg = {"parallel_l0": PARALLEL_L0, "parallel_lddsr": PARALLEL_LDDSR, "parallel_l0_swipe": PARALLEL_L0_SWIPE}[variant]
    o = GboOpts(alg, tol, maxiter, 1000, 0, l0_thresh, 0)
    info = GboInfo()
    lib().gbo_parallel_l0(C.byref(op.c), _p(y), C.byref(o), _p(x), _p(res), _p(rec), C.byref(info))
    return x, res, rec, info


def serial_l0(op, y, tol, maxiter, l0_thresh=1):
    y = f32(y)
    x = np.zeros(op.n, dtype=np.float32)
    res = y.copy()
    rec = np.zeros(maxiter + 1, dtype=np.float32)
    o = GboOpts(SERIAL_L0, tol, maxiter, 1000, 0, l0_thresh, 0)
    info = GboInfo()
    lib().gbo_serial_l0(C.byref(op.c), _p(y), C.byref(o), _p(x), _p(res), _p(rec), C.byref(info))
    return x, res, rec, info


def l0_scores(res, x, rows, n, d, thresh, shift):
    res, x, rows = f32(res), f32(x).copy(), i32(rows)
    upd = np.zeros(n, dtype=np.float32)
    found = C.c_int(0)
    lib().gbo_l0_scores(_p(res), _p(x), _p(upd), _p(rows), n, d, thresh, shift, C.byref(found))
    return x, upd, found.value


def l0_update_residual(res, rows, updates, n, d):
    res = f32(res).copy()
    lib().gbo_l0_update_residual(_p(res), _p(i32(rows)), _p(f32(updates)), n, d)
    return res


def results(x, x_true, k):
    norms = np.zeros(3, dtype=np.float32)
    supp = np.zeros(4, dtype=np.int32)
    lib().gbo_results(_p(f32(x)), _p(f32(x_true)), len(x), k, _p(norms), _p(supp))
    return norms, supp


def solve_dense_trials(n, m, k, seed, trial_ids, alg="NIHT", tol_rel=1e-4, maxiter=5000, threads=0):
    n, m, k = i32(n), i32(m), i32(k)
    tids = np.ascontiguousarray(trial_ids, dtype=np.uint32)
    iters = np.zeros(len(n), dtype=np.int32)
    err = np.zeros(len(n), dtype=np.float32)
    ok = lib().gbo_solve_dense_trials(len(n), _p(n), _p(m), _p(k), seed, _p(tids), ALG_IDS[alg], tol_rel,
                                      maxiter, threads, _p(iters), _p(err))
    return ok, iters, err


# ---------------- the reference's own code run on the CPU (oracle/_ref) ----------------
_ref = None


def ref_lib():
    """The reference's kernels compiled for the CPU; None where the reference tree is absent."""
    global _ref
    if _ref is None:
        path = _build.build_ref()
        if path is None:
            return None
        _ref = C.CDLL(path)
        vp, i, f = C.c_void_p, C.c_int, C.c_float
        _ref.ref_linear_binning.argtypes = [vp, vp, vp, i, i, i, f, f]
        _ref.ref_threshold.argtypes = [vp, vp, i, i]
        _ref.ref_threshold_one.argtypes = [vp, vp, vp, i, i]
        _ref.ref_check_support_evolution.argtypes = [vp, vp, i, i, i]
        _ref.ref_check_support_evolution.restype = i
        _ref.ref_l0_scores.argtypes = [vp, vp, vp, vp, vp, i, i, i, i]
        _ref.ref_l0_scores.restype = i
        _ref.ref_update_residual.argtypes = [vp, vp, vp, i, i]
        _ref.ref_serial_l0.argtypes = [vp, vp, vp, vp, vp, i, i, i, i, i, f, i, vp, vp]
        _ref.ref_serial_l0.restype = i
    return _ref
