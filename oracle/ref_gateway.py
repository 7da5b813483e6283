"""Calls into the reference's own MEX gateways (gaga_gen / gaga_dct / gaga_smv, compiled for
the CPU by oracle/build.py:build_ref_gateways) with MATLAB-style arguments.

Test infrastructure only: it produces the reference's outputs on given data (the
"solve given data" usage of each gateway, GAGA/gaga/gaga_gen.cu:115-134,
gaga_dct.cu:112-127, gaga_smv.cu:159-195) for the golden fixtures under tests/golden.
The gateways need the reference tree, so only tests/golden/make_ref_loops.py calls them;
bind() / call() and the argument builders also drive this library's own MEX shim
(gaga_gb300/mex/gb_gaga_mex.cpp) in the tests.
"""
import ctypes as C

import numpy as np

from . import build as _build

# class ids of oracle/ref_shim/host/mex.h
mxCHAR, mxDOUBLE, mxSINGLE, mxINT32, mxUINT32, mxCELL = 4, 6, 7, 12, 13, 1
_INT_OPTS = {"maxiter", "numBins", "supportFlag", "convRateNum", "gpuNumber", "threadsPerBlockn", "threadsPerBlockm",
             "threadsPerBlocknp", "threadsPerBlockBin", "l0_thresh", "debug_mode", "num_band_levels"}
_libs = {}


def bind(path):
    """Loads a MEX-style library (a gateway over the stand-in mx API of
    oracle/ref_shim/host/mex.h) and declares its mx calls."""
    L = C.CDLL(path)
    vp, i = C.c_void_p, C.c_int
    L.gbmx_numeric.restype = vp
    L.gbmx_numeric.argtypes = [i, i, i, vp]
    L.gbmx_string.restype = vp
    L.gbmx_string.argtypes = [C.c_char_p]
    L.gbmx_cell.restype = vp
    L.gbmx_cell.argtypes = [i, i]
    L.gbmx_cell_set.argtypes = [vp, i, vp]
    L.gbmx_free.argtypes = [vp]
    L.mexFunction.argtypes = [i, vp, i, vp]
    L.mxGetData.restype = vp
    L.mxGetData.argtypes = [vp]
    L.mxGetM.restype = C.c_size_t
    L.mxGetM.argtypes = [vp]
    L.mxGetN.restype = C.c_size_t
    L.mxGetN.argtypes = [vp]
    L.gbmx_class.argtypes = [vp]
    L.gbmx_last_error.restype = C.c_char_p
    return L


def lib(gateway):
    if gateway not in _libs:
        paths = _build.build_ref_gateways()
        if paths is None:
            raise RuntimeError("the reference tree is not available (GAGA_REFERENCE_ROOT)")
        _libs[gateway] = bind(_build.lib_gateway(gateway))
    return _libs[gateway]


_NP = {mxSINGLE: np.float32, mxINT32: np.int32, mxUINT32: np.uint32, mxDOUBLE: np.float64}


def _num(L, a, cls):
    a = np.asarray(a, dtype=_NP[cls])
    if a.ndim == 0:
        m, n = 1, 1
    elif a.ndim == 1:
        m, n = a.shape[0], 1
    else:
        m, n = a.shape
    buf = np.asfortranarray(a).reshape(-1, order="F")
    return L.gbmx_numeric(cls, m, n, buf.ctypes.data)


def _options(L, opts):
    """gagaOptions (GAGA/gaga/gagaOptions.m): an l x 2 cell of names and typed values."""
    cell = L.gbmx_cell(len(opts), 2)
    for i, (name, val) in enumerate(opts):
        L.gbmx_cell_set(cell, i, L.gbmx_string(name.encode()))
        if isinstance(val, str):
            v = L.gbmx_string(val.encode())
        elif name in _INT_OPTS:
            v = _num(L, val, mxINT32)
        elif name == "seed":
            v = _num(L, val, mxUINT32)
        else:
            v = _num(L, val, mxSINGLE)
        L.gbmx_cell_set(cell, len(opts) + i, v)
    return cell


def _out(L, p):
    cls = L.gbmx_class(p)
    m, n = L.mxGetM(p), L.mxGetN(p)
    dt = _NP[cls]
    a = np.ctypeslib.as_array(C.cast(L.mxGetData(p), C.POINTER(np.ctypeslib.as_ctypes_type(dt))), shape=(m * n,))
    return a.copy()


def call(L, nlhs, args):
    """mexFunction(nlhs, plhs, nrhs, prhs) of library L; returns the outputs as numpy arrays
    (None where the gateway left an output unset) and frees every array."""
    prhs = (C.c_void_p * len(args))(*args)
    plhs = (C.c_void_p * nlhs)()
    L.mexFunction(nlhs, plhs, len(args), prhs)
    outs = [_out(L, plhs[i]) if plhs[i] else None for i in range(nlhs)]
    for a in list(args) + [plhs[i] for i in range(nlhs)]:
        if a:
            L.gbmx_free(a)
    return outs


def out_classes(L, nlhs, args):
    """Like call(), but returns the mx class ids of the outputs."""
    prhs = (C.c_void_p * len(args))(*args)
    plhs = (C.c_void_p * nlhs)()
    L.mexFunction(nlhs, plhs, len(args), prhs)
    cls = [L.gbmx_class(plhs[i]) if plhs[i] else None for i in range(nlhs)]
    for a in list(args) + [plhs[i] for i in range(nlhs)]:
        if a:
            L.gbmx_free(a)
    return cls


def gen_args(L, alg, y, A, k, opts=()):
    args = [L.gbmx_string(alg.encode()), _num(L, y, mxSINGLE), _num(L, A, mxSINGLE), _num(L, float(k), mxDOUBLE)]
    return args + ([_options(L, opts)] if opts else [])


def dct_args(L, alg, y, rows_1based, k, m, n, opts=()):
    args = [L.gbmx_string(alg.encode()), _num(L, y, mxSINGLE), _num(L, rows_1based, mxINT32),
            _num(L, float(k), mxDOUBLE), _num(L, float(m), mxDOUBLE), _num(L, float(n), mxDOUBLE)]
    return args + ([_options(L, opts)] if opts else [])


def smv_args(L, alg, y, rows_1based, cols_1based, vals, k, opts=()):
    args = [L.gbmx_string(alg.encode()), _num(L, y, mxSINGLE), _num(L, rows_1based, mxINT32),
            _num(L, cols_1based, mxINT32), _num(L, vals, mxSINGLE), _num(L, float(k), mxDOUBLE)]
    return args + ([_options(L, opts)] if opts else [])


def gaga_gen(alg, y, A, k, opts=(), L=None):
    """[x iters convRate] = gaga_gen(alg, y, A, k, opts); A is m x n (numpy, any order)."""
    L = L or lib("gen")
    x, it, conv = call(L, 3, gen_args(L, alg, y, A, k, opts))
    return x, int(it[0]), float(conv[0])


def gaga_dct(alg, y, rows_1based, k, m, n, opts=(), L=None):
    """[x iters convRate] = gaga_dct(alg, y, rows, k, m, n, opts); rows are 1-based."""
    L = L or lib("dct")
    x, it, conv = call(L, 3, dct_args(L, alg, y, rows_1based, k, m, n, opts))
    return x, int(it[0]), float(conv[0])


def gaga_smv(alg, y, rows_1based, cols_1based, vals, k, opts=(), L=None):
    """[x iters convRate resRecord timeRecord] = gaga_smv(alg, y, rows, cols, vals, k, opts)."""
    L = L or lib("smv")
    x, it, conv, rec, trec = call(L, 5, smv_args(L, alg, y, rows_1based, cols_1based, vals, k, opts))
    return x, int(it[0]), float(conv[0]), rec
