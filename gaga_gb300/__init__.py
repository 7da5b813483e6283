"""GB300-native greedy sparse recovery (NIHT / HTP / CGIHT / expander l0).

Python mirror of GAGA's MATLAB front end (GAGA/gaga/gaga_cs.m, gagaOptions.m) over the
C ABI of libgb_cs.so (include/gb_cs.h).  Argument order, option names and outputs
follow the reference:

    norms, times, iters, support, conv, x = gaga_cs('NIHT', 'gen', k, m, n, opts)
    x, iters, conv = gaga_cs('CGIHT', 'gen', y, A, k, opts)
    x, iters, conv = gaga_cs('HTP', 'dct', y, rows, k, m, n, opts)
    x, iters, conv, res_record, time_record = gaga_cs('parallel_l0', 'smv', y, rows, cols, vals, k, opts)

Index arrays are 1-based by default, as MATLAB passes them to the reference gateways
(GAGA/gaga/gaga_dct.cu:543, gaga_smv.cu:684-685); pass ``index_base=0`` for 0-based data.
Inputs may be numpy arrays (host) or CUDA tensors exposing ``data_ptr()`` (device).
"""
import ctypes as C

import numpy as np

from . import _lib, autotune, learned, sweep
from ._lib import GagaError

__all__ = ["gaga_cs", "gaga_options", "GagaError", "solve_batch", "version"]

_OPTION_NAMES = {"tol", "maxiter", "vecDistribution", "matrixEnsemble", "seed", "numBins", "threadsPerBlockn",
                 "threadsPerBlockm", "threadsPerBlocknp", "threadsPerBlockBin", "convRateNum", "kFixed", "noise",
                 "gpuNumber", "timing", "alpha", "supportFlag", "restartFlag", "projFracTol", "l0_thresh",
                 "band_percentage", "debug_mode", "tol_is_relative", "learnedWarmStart", "resultsDir",
                 "watchdogPasses"}


def version():
    return _lib.load().gb_cs_version().decode()


def gaga_options(*pairs):
    """gagaOptions (GAGA/gaga/gagaOptions.m): name/value pairs -> option dict."""
    if len(pairs) % 2:
        raise ValueError("options come in name/value pairs")
    out = {}
    for name, value in zip(pairs[0::2], pairs[1::2]):
        if name not in _OPTION_NAMES:
            raise ValueError("The following option is not recognised: %s" % name)
        out[name] = value
    return out


def _options(alg, n, opts, ens):
    L = _lib.load()
    o = _lib.Options()
    L.gb_cs_default_options(C.byref(o), alg.encode(), int(n))
    if ens == "gen":
        o.matrix_ensemble = 1
    elif ens == "smv":
        o.matrix_ensemble = 3
    for name, v in (opts or {}).items():
        if name == "tol":
            o.tol = float(v)
        elif name == "tol_is_relative":
            o.tol_is_relative = int(bool(v))
        elif name == "maxiter":
            o.maxiter = int(v)
        elif name == "numBins":
            o.num_bins = int(v)
        elif name == "restartFlag":
            o.restart_flag = 1 if v in ("on", 1, True) else 0
        elif name == "l0_thresh":
            o.l0_thresh = int(v)
        elif name == "vecDistribution":
            o.vec_distribution = {"binary": 1, "uniform": 0, "gaussian": 2}[v]
        elif name == "matrixEnsemble":
            if ens == "gen":
                o.matrix_ensemble = {"gaussian": 1, "binary": 2}[v]
            else:
                o.matrix_ensemble = {"ones": 1, "binary": 2, "expander": 3}[v]
        elif name == "kFixed":
            o.k_fixed = 1 if v in ("on", 1, True) else 0
        elif name == "seed":
            o.seed = int(v) & 0xFFFFFFFF
        elif name == "noise":
            o.noise = float(v)
        elif name == "gpuNumber":
            o.gpu_number = int(v)
        elif name == "convRateNum":
            o.conv_rate_num = int(v)
        elif name == "alpha":
            o.alpha = float(v)
        elif name == "supportFlag":
            o.support_flag = int(v)
        elif name == "timing":
            o.timing = 1 if v in ("on", 1, True) else 0
        elif name == "projFracTol":
            o.proj_frac_tol = float(v)
        elif name == "watchdogPasses":
            # extension: bound on the device-side loop passes (0: maxiter + 4) -> GB_WATCHDOG
            o.watchdog_passes = int(v)
        elif name == "resultsDir":
            # extension: append the reference's result line to the dated file in this directory
            o._results_dir = None if v is None else str(v).encode()
            o.results_dir = o._results_dir
        elif name == "learnedWarmStart":
            # extension: a CUDA tensor of gb_cs_mlp_num_params() FP32 MLP parameters (CGIHT)
            o.learned_params = None if v is None else v.data_ptr()
        # threadsPerBlock*, band_percentage, debug_mode: accepted, no effect
    return o


_last_timings = None


def _attach_timing(alg, o, r):
    """Timing variants (timing 'on', NIHT / HTP): per-iteration buffers for the result."""
    global _last_timings
    _last_timings = None
    if not o.timing or o.maxiter <= 0 or alg not in ("NIHT", "HTP"):
        return None
    bufs = {name: np.zeros(o.maxiter, dtype=np.float32)
            for name in ("time_per_iteration", "time_supp_set", "cg_per_iteration", "time_for_cg")}
    for name, b in bufs.items():
        setattr(r, name, b.ctypes.data)
    return bufs


def _keep_timing(bufs, r):
    global _last_timings
    if bufs is not None and (r.time_per_iteration or 0):
        _last_timings = {name: b[: r.iter].copy() for name, b in bufs.items()}


def last_timings():
    """Per-iteration times (ms) of the last solve run with timing 'on' (NIHT or HTP):
    time_per_iteration, time_supp_set, cg_per_iteration, time_for_cg (the arrays the
    reference's timing variants record, GAGA/gaga/algorithms_timings.cu), or None."""
    return _last_timings


def _is_device(a):
    return hasattr(a, "data_ptr") and getattr(a, "is_cuda", False)


class _Buf:
    """Host (numpy) or device (CUDA tensor) buffer view with a raw pointer."""

    def __init__(self, a, dtype):
        if _is_device(a):
            self.device = True
            self.obj = a.contiguous() if hasattr(a, "contiguous") else a
            self.ptr = self.obj.data_ptr()
            self.size = self.obj.numel()
        else:
            self.device = False
            self.obj = np.ascontiguousarray(a, dtype=dtype)
            self.ptr = self.obj.ctypes.data
            self.size = self.obj.size


def _solve(alg, kind, y, k, m, n, opts, ens, A=None, lda=0, rows=None, cols=None, vals=None, d=0,
           index_base=1, want_record=False, stream=None):
    L = _lib.load()
    o = _options(alg, n, opts, ens)
    yb = _Buf(y, np.float32)
    device = yb.device
    p = _lib.Problem()
    p.kind, p.m, p.n, p.k = kind, int(m), int(n), int(k)
    p.y = yb.ptr
    keep = [yb]
    if A is not None:
        ab = _Buf(A, np.float32)
        keep.append(ab)
        p.A, p.lda = ab.ptr, int(lda)
    for name, arr, dt in (("rows", rows, np.int32), ("cols", cols, np.int32), ("vals", vals, np.float32)):
        if arr is not None:
            b = _Buf(arr, dt)
            keep.append(b)
            setattr(p, name, b.ptr)
    p.d = int(d)
    p.index_base = int(index_base)
    p.location = _lib.GB_DEVICE if device else _lib.GB_HOST
    p.stream = stream
    if device:
        import torch

        x = torch.zeros(n, dtype=torch.float32, device=y.device)
        xptr = x.data_ptr()
    else:
        x = np.zeros(n, dtype=np.float32)
        xptr = x.ctypes.data
    r = _lib.Result()
    rec = trec = None
    if want_record:
        rec = np.zeros(o.maxiter + 1, dtype=np.float32)
        trec = np.zeros(o.maxiter + 1, dtype=np.float32)
        r.res_record = rec.ctypes.data
        r.time_record = trec.ctypes.data
    tb = _attach_timing(alg, o, r)
    _lib.check(L.gb_cs_solve(alg.encode(), C.byref(p), C.byref(o), C.c_void_p(xptr), C.byref(r)))
    _keep_timing(tb, r)
    return x, r, (rec, trec)


def _size(a):
    return int(np.prod(np.shape(a))) if not _is_device(a) else a.numel()


def gaga_cs(alg, ens, *args, index_base=1, stream=None):
    """Mirror of gaga_cs.m (GAGA/gaga/gaga_cs.m:7-64)."""
    if ens == "gen":
        if len(args) in (3, 4) and _size(args[1]) > 1:
            y, A, k = args[:3]
            opts = args[3] if len(args) == 4 else None
            if _is_device(A):
                m, n = A.shape
                # a torch (row-major) m x n tensor is passed as its transpose in memory: the
                # column-major view of A is A.t() contiguous
                At = A.t().contiguous()
                x, r, _ = _solve(alg, _lib.GB_OP_DENSE, y, k, m, n, opts, ens, A=At, lda=m, stream=stream)
            else:
                A = np.asarray(A, dtype=np.float32)
                m, n = A.shape
                Acm = np.asfortranarray(A).ravel(order="F")
                x, r, _ = _solve(alg, _lib.GB_OP_DENSE, y, k, m, n, opts, ens, A=Acm, lda=m, stream=stream)
            return x, r.iter, r.conv_rate
        if len(args) in (3, 4):
            k, m, n = args[:3]
            return _generate(alg, _lib.GB_OP_DENSE, k, m, n, 0, args[3] if len(args) == 4 else None, ens)
        raise ValueError("Either five or six input arguments required.")
    if ens == "dct":
        if len(args) in (5, 6) and _size(args[1]) > 1:
            y, rows, k, m, n = args[:5]
            opts = args[5] if len(args) == 6 else None
            x, r, _ = _solve(alg, _lib.GB_OP_DCT, y, k, m, n, opts, ens, rows=rows, index_base=index_base,
                             stream=stream)
            return x, r.iter, r.conv_rate
        if len(args) in (3, 4):
            k, m, n = args[:3]
            return _generate(alg, _lib.GB_OP_DCT, k, m, n, 0, args[3] if len(args) == 4 else None, ens)
        raise ValueError("Either seven or eight input arguments required.")
    if ens == "smv":
        if len(args) in (5, 6) and _size(args[2]) > 1:
            y, rows, cols, vals, k = args[:5]
            opts = args[5] if len(args) == 6 else None
            c = np.asarray(cols.cpu() if _is_device(cols) else cols, dtype=np.int64)
            r_ = np.asarray(rows.cpu() if _is_device(rows) else rows, dtype=np.int64)
            # p = run length of equal column indices; m, n = largest indices (gaga_smv.cu:157-170)
            p_ = 1
            while p_ < len(c) and c[p_ - 1] == c[p_]:
                p_ += 1
            m = int(r_.max()) + 1 - index_base
            n = int(c.max()) + 1 - index_base
            x, r, (rec, trec) = _solve(alg, _lib.GB_OP_SMV, y, k, m, n, opts, ens, rows=rows, cols=cols, vals=vals,
                                       d=p_, index_base=index_base, want_record=True, stream=stream)
            return x, r.iter, r.conv_rate, rec, trec
        if len(args) in (4, 5):
            k, m, n, p_ = args[:4]
            return _generate(alg, _lib.GB_OP_SMV, k, m, n, p_, args[4] if len(args) == 5 else None, ens)
        raise ValueError("Either six or seven input arguments required.")
    raise ValueError("ens must be either dct, gen, or smv.")


def _generate(alg, kind, k, m, n, d, opts, ens):
    L = _lib.load()
    o = _options(alg, n, opts, ens)
    x = np.zeros(n, dtype=np.float32)
    xt = np.zeros(n, dtype=np.float32)
    r = _lib.Result()
    rec = np.zeros(o.maxiter + 1, dtype=np.float32) if kind == _lib.GB_OP_SMV else None
    trec = np.zeros(o.maxiter + 1, dtype=np.float32) if kind == _lib.GB_OP_SMV else None
    if rec is not None:
        r.res_record = rec.ctypes.data
        r.time_record = trec.ctypes.data
    tb = _attach_timing(alg, o, r)
    _lib.check(L.gb_cs_generate_and_solve(alg.encode(), kind, int(k), int(m), int(n), int(d), C.byref(o),
                                          C.c_void_p(x.ctypes.data), C.c_void_p(xt.ctypes.data), C.byref(r)))
    _keep_timing(tb, r)
    norms = np.array(r.norms, dtype=np.float32)
    times = np.array(r.times, dtype=np.float32)
    support = np.array(r.support, dtype=np.int32)
    out = (norms, times, np.int32(r.iter), support, np.float32(r.conv_rate), x)
    if kind == _lib.GB_OP_SMV:
        out = out + (rec, trec)
    return out


def generate_and_solve(alg, ens, k, m, n, d=0, opts=None):
    """Like gaga_cs's generate usage, also returning the generated signal and k used."""
    L = _lib.load()
    kind = {"gen": _lib.GB_OP_DENSE, "dct": _lib.GB_OP_DCT, "smv": _lib.GB_OP_SMV}[ens]
    o = _options(alg, n, opts, ens)
    x = np.zeros(n, dtype=np.float32)
    xt = np.zeros(n, dtype=np.float32)
    r = _lib.Result()
    tb = _attach_timing(alg, o, r)
    _lib.check(L.gb_cs_generate_and_solve(alg.encode(), kind, int(k), int(m), int(n), int(d), C.byref(o),
                                          C.c_void_p(x.ctypes.data), C.c_void_p(xt.ctypes.data), C.byref(r)))
    _keep_timing(tb, r)
    return x, xt, r


GRAD_FORMATS = {"fp32": 0, "a24": 1, "bf16": 2}


def solve_batch(n, m, k, seed, trial_ids=None, alg="NIHT", tol_rel=1e-4, maxiter=5000, stream=None,
                learned_params=None, slots=0, sm_share=0, resident_n=0, cluster=0, grad_format="fp32",
                residual_refresh=0, grad_formats=None, av_rows=0):
    """Batched multi-trial dense form (gb_cs_solve_batch); learned_params (a CUDA tensor of
    MLP parameters, CGIHT only) turns on the learned warm start; slots / sm_share set the
    schedule of the slot graphs (0: automatic; gaga_gb300.autotune picks them by
    measurement); trials with n <= resident_n (0: 8192, < 0: none) are solved by the
    cluster-resident kernel with `cluster` CTAs per trial (0: 4, or more when the sizes need
    it); grad_format ("fp32", "a24" or "bf16") is the operand of A^T r (24-bit or BF16
    copies of A stream 3 or 2 bytes per entry; A x, the residual and the stopping test keep
    FP32 A); grad_formats (one of "a24" / "bf16" per trial) picks it per trial instead;
    residual_refresh N > 0 (CGIHT) updates the residual of a restricted step on an unchanged
    support as r - alpha A p, recomputing y - A x every N-th iteration; av_rows (128 or 256,
    0: 128) is the row tile of the slot graphs' A x_S kernel."""
    L = _lib.load()
    n = np.ascontiguousarray(n, dtype=np.int32)
    m = np.ascontiguousarray(m, dtype=np.int32)
    k = np.ascontiguousarray(k, dtype=np.int32)
    tids = None if trial_ids is None else np.ascontiguousarray(trial_ids, dtype=np.uint32)
    fmts = None
    if grad_formats is not None:
        fmts = np.ascontiguousarray([GRAD_FORMATS[f] if isinstance(f, str) else int(f) for f in grad_formats],
                                    dtype=np.uint8)
    b = _lib.Batch(len(n), n.ctypes.data, m.ctypes.data, k.ctypes.data, None if tids is None else tids.ctypes.data,
                   int(seed) & 0xFFFFFFFF, {"NIHT": 0, "HTP": 1, "CGIHT": 6}[alg], float(tol_rel), int(maxiter),
                   0 if learned_params is None else 1,
                   None if learned_params is None else learned_params.data_ptr(), int(slots), int(sm_share), stream,
                   int(resident_n), int(cluster), GRAD_FORMATS[grad_format],
                   None if fmts is None else fmts.ctypes.data, int(av_rows), int(residual_refresh))
    iters = np.zeros(len(n), dtype=np.int32)
    err = np.zeros(len(n), dtype=np.float32)
    ok = np.zeros(len(n), dtype=np.int32)
    ns = C.c_int(0)
    _lib.check(L.gb_cs_solve_batch(C.byref(b), C.c_void_p(iters.ctypes.data), C.c_void_p(err.ctypes.data),
                                   C.c_void_p(ok.ctypes.data), C.byref(ns)))
    return ns.value, iters, err, ok


def batch_slot_count():
    """Slot streams (one graph launch each) the batched form uses per call."""
    import os

    return int(os.environ.get("GB_CS_BATCH_SLOTS", "16"))


def batch_last_stats():
    """(algorithmic matvec bytes, device ms) of the last solve_batch call."""
    L = _lib.load()
    b, t = C.c_double(0), C.c_float(0)
    L.gb_cs_batch_last_stats(C.byref(b), C.byref(t))
    return b.value, t.value


def solve_shared_batch(m, n, k, seed, tol_rel=1e-4, maxiter=5000, precision=3, outputs=False, first_trial=0,
                       stream=None, alg="NIHT", learned_params=None):
    """Shared-matrix batched form (gb_cs_solve_shared_batch): len(k) NIHT or CGIHT trials
    with one dense Gaussian A, operator work as BF16 tensor-core GEMMs, least-squares debias.
    precision: bit 0 splits A^T r, bit 1 splits A x_thres into BF16 high/low parts.
    learned_params: CGIHT's warm-start network (a CUDA tensor, gaga_gb300.learned), or None.

    Returns (num_success, iters, rel_err, ok) and, with outputs=True, also the generated
    A (m x n column-major, as an (n, m) CUDA tensor), Y (T x m) and X0 (T x n) on the device;
    with outputs="x" also the final X (T x n).
    """
    L = _lib.load()
    k = np.ascontiguousarray(k, dtype=np.int32)
    T = len(k)
    A = Y = X0 = X = None
    if outputs:
        import torch
        A = torch.empty((n, m), dtype=torch.float32, device="cuda")
        Y = torch.empty((T, m), dtype=torch.float32, device="cuda")
        X0 = torch.empty((T, n), dtype=torch.float32, device="cuda")
        if outputs == "x":
            X = torch.empty((T, n), dtype=torch.float32, device="cuda")
    b = _lib.SharedBatch(T, int(m), int(n), k.ctypes.data, int(seed) & 0xFFFFFFFF, int(first_trial) & 0xFFFFFFFF,
                         float(tol_rel), int(maxiter),
                         int(precision), None if A is None else A.data_ptr(), None if Y is None else Y.data_ptr(),
                         None if X0 is None else X0.data_ptr(), stream, {"NIHT": 0, "CGIHT": 6}[alg],
                         None if learned_params is None else learned_params.data_ptr(),
                         None if X is None else X.data_ptr())
    iters = np.zeros(T, dtype=np.int32)
    err = np.zeros(T, dtype=np.float32)
    ok = np.zeros(T, dtype=np.int32)
    ns = C.c_int(0)
    _lib.check(L.gb_cs_solve_shared_batch(C.byref(b), C.c_void_p(iters.ctypes.data), C.c_void_p(err.ctypes.data),
                                          C.c_void_p(ok.ctypes.data), C.byref(ns)))
    if outputs == "x":
        return ns.value, iters, err, ok, A, Y, X0, X
    if outputs:
        return ns.value, iters, err, ok, A, Y, X0
    return ns.value, iters, err, ok


def shared_last_fallbacks():
    """Trials of the last solve_shared_batch call whose learned warm start was abandoned."""
    return int(_lib.load().gb_cs_shared_last_fallbacks())


def shared_last_stats():
    """(GEMM FLOPs, device ms) of the last solve_shared_batch call."""
    L = _lib.load()
    fl, t = C.c_double(0), C.c_float(0)
    L.gb_cs_shared_last_stats(C.byref(fl), C.byref(t))
    return fl.value, t.value


def gemm_bf16_tn(A, B, Y=None, want_bf16=False):
    """Ct = [Y -] (A B^T)^T for BF16 CUDA tensors A (M x K), B (N x K); returns (Ct, Cb)."""
    import torch
    L = _lib.load()
    M, K = A.shape
    N = B.shape[0]
    Ct = torch.empty((N, M), dtype=torch.float32, device=A.device)
    Cb = torch.empty((N, M), dtype=torch.bfloat16, device=A.device) if want_bf16 else None
    _lib.check(L.gb_cs_gemm_bf16_tn(A.data_ptr(), B.data_ptr(), Ct.data_ptr(), M, N, K,
                                    None if Y is None else Y.data_ptr(), None if Cb is None else Cb.data_ptr(),
                                    torch.cuda.current_stream().cuda_stream))
    return Ct, Cb
