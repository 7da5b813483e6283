"""Host-side logic on the CPU: the C ABI library loads and exports every declared
symbol, option defaults mirror the reference, argument validation happens before any
device work, and the oracle recovers the first workload."""
import ctypes as C
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    text = open(os.path.join(ROOT, "include", "gb_cs.h")).read()
    return sorted(set(re.findall(r"\b(gb_cs_\w+)\s*\(", text)))


def test_library_exports_every_declared_symbol(gb):
    L = gb._lib.load()
    syms = declared_symbols()
    assert len(syms) >= 10
    missing = [s for s in syms if not hasattr(L, s)]
    assert not missing, missing
    assert sorted(gb._lib.EXPORTS) == syms


def test_library_links_every_translation_unit(gb):
    """Every symbol the library needs is defined in it or versioned in the C/C++ runtime (a
    translation unit left out of the build shows up as an unversioned undefined symbol)."""
    import shutil
    import subprocess

    nm = shutil.which("nm")
    if nm is None:
        pytest.skip("nm not available")
    out = subprocess.run([nm, "-D", "--undefined-only", gb._lib.LIB_PATH], capture_output=True, text=True).stdout
    missing = [ln.split()[-1] for ln in out.splitlines() if ln.split() and ln.split()[0] == "U" and "@" not in ln]
    assert not missing, missing


def test_default_options_mirror_reference(gb):
    L = gb._lib.load()
    o = gb._lib.Options()
    L.gb_cs_default_options(C.byref(o), b"NIHT", 4096)
    assert o.tol == -10.0  # float tol = 10^(-4) is C XOR (GAGA/gaga/gaga_gen.cu:183)
    assert o.maxiter == 5000 and o.num_bins == 1000 and o.conv_rate_num == 16
    L.gb_cs_default_options(C.byref(o), b"HTP", 2 ** 20)
    assert o.maxiter == 300 and o.num_bins == 52428
    assert o.vec_distribution == 1 and abs(o.alpha - 0.25) < 1e-7


def test_alg_ids(gb):
    L = gb._lib.load()
    names = (b"NIHT", b"HTP", b"IHT", b"ThresholdSD", b"ThresholdCG", b"CGIHT", b"parallel_l0", b"CSMPSP")
    assert [L.gb_cs_alg_id(a) for a in names] == [0, 1, 2, 3, 4, 6, 14, -1]


def test_bad_arguments_rejected_before_device_work(gb):
    L = gb._lib.load()
    p = gb._lib.Problem()
    p.kind, p.m, p.n, p.k = 0, 10, 20, 2
    x = np.zeros(20, np.float32)
    r = gb._lib.Result()
    assert L.gb_cs_solve(b"FOO", C.byref(p), None, C.c_void_p(x.ctypes.data), C.byref(r)) == gb._lib.GB_BAD_ARG
    assert b"algorithm" in L.gb_cs_last_error()
    assert L.gb_cs_solve(b"parallel_l0", C.byref(p), None, C.c_void_p(x.ctypes.data),
                         C.byref(r)) == gb._lib.GB_BAD_ARG
    o = gb._lib.Options()
    L.gb_cs_default_options(C.byref(o), b"NIHT", 20)
    o.maxiter = -1
    assert L.gb_cs_solve(b"NIHT", C.byref(p), C.byref(o), C.c_void_p(x.ctypes.data), C.byref(r)) == gb._lib.GB_BAD_ARG


def test_gaga_options(gb):
    o = gb.gaga_options("tol", 1e-4, "maxiter", 400, "restartFlag", "on")
    assert o == {"tol": 1e-4, "maxiter": 400, "restartFlag": "on"}
    with pytest.raises(ValueError):
        gb.gaga_options("tolerance", 1)
    with pytest.raises(ValueError):
        gb.gaga_options("tol")


def test_gaga_cs_argument_count(gb):
    with pytest.raises(ValueError):
        gb.gaga_cs("NIHT", "gen", 1, 2)
    with pytest.raises(ValueError):
        gb.gaga_cs("NIHT", "xyz", 1, 2, 3)


@pytest.mark.parametrize("alg", ["NIHT", "HTP", "CGIHT"])
def test_oracle_recovers_first_workload(gbo, alg):
    """Dense Gaussian n=4096, m=1024, k=102, +-1 signal, tol 1e-4*||y||."""
    n, m, k = 4096, 1024, 102
    A = gbo.gen_dense(m, n, seed=1234)
    x0, ks = gbo.gen_vector(n, k, 1, seed=1234)
    op = gbo.Op.dense(A, m, n)
    y = gbo.A(op, x0)
    x, info = gbo.solve(alg, op, y, ks, 1e-4 * float(np.linalg.norm(y)))
    norms, supp = gbo.results(x, x0, ks)
    assert norms[1] < 1e-3
    assert supp[0] == ks and supp[1] == 0


def test_oracle_parallel_l0_exact(gbo):
    n, m, d = 4096, 1024, 7
    rows, vals = gbo.gen_smv(m, n, d, 3, seed=2)
    x0, ks = gbo.gen_vector(n, m // 20, 1, seed=2)
    op = gbo.Op.smv(m, n, d, rows, vals)
    y = gbo.A(op, x0)
    x, res, rec, info = gbo.parallel_l0(op, y, tol=1e-6, maxiter=200)
    assert np.array_equal(x, x0)
    assert not np.any(res)


def test_generators_are_deterministic(gbo):
    a = gbo.gen_dense(64, 100, seed=3)
    b = gbo.gen_dense(64, 100, seed=3)
    assert np.array_equal(a, b)
    assert not np.array_equal(a, gbo.gen_dense(64, 100, seed=4))
    rows = gbo.gen_dct_rows(1024, 256, seed=1)
    assert len(set(rows.tolist())) == 256 and rows.min() >= 0 and rows.max() < 1024
    r, v = gbo.gen_smv(128, 500, 7, 3, seed=1)
    cols = r.reshape(500, 7)
    assert all(len(set(c.tolist())) == 7 for c in cols)
