"""The NIHT / HTP timing variants (GAGA/gaga/algorithms_timings.cu) on the GPU.

With timing on, NIHT and HTP run the timing variants' loops: alpha from the options, no
cycle test, the rate test's 1/16-th root, and the support step chosen by supportFlag
(0 adaptive binning, 1 binning every iteration, 2 / 3 the sort-based FindSupportSet_sort,
GAGA/gaga/functions.cu:446-465).  They also record per-iteration times.

  - FindSupportSet_sort itself (gb_cs_find_support_set_sort: radix select of the k-th
    largest |v|, threshold, bins) equals the oracle bit for bit, ties and both branches
    included;
  - every variant solves as the oracle's restatement does: same verdict (relative l2 to the
    planted signal <= 1e-3), and when recovered x within 1e-4 of the oracle's and the
    iteration count within 3;
  - the per-iteration records are complete and consistent, and generate-and-solve writes
    the reference's timing file.
"""
import ctypes as C
import os
import re

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _sort_gpu(gb, v, bins, T, max_change, k):
    import torch

    L = gb._lib.load()
    dv = torch.from_numpy(np.ascontiguousarray(v, dtype=np.float32)).cuda()
    db = torch.from_numpy(np.ascontiguousarray(bins, dtype=np.int32)).cuda()
    Tout = C.c_float(0)
    gb._lib.check(L.gb_cs_find_support_set_sort(C.c_void_p(dv.data_ptr()), C.c_void_p(db.data_ptr()), len(v), k,
                                                float(T), float(max_change), C.byref(Tout), None))
    torch.cuda.synchronize()
    return dv.cpu().numpy(), db.cpu().numpy(), np.float32(Tout.value)


@pytest.mark.parametrize("n,k,kind", [(1000, 1, "gauss"), (1000, 1000, "gauss"), (4097, 300, "ties"),
                                      (2 ** 20, 26214, "gauss"), (2 ** 20 + 5, 5000, "ties"),
                                      (70000, 700, "tiny")])
def test_find_support_set_sort_bit_exact(gb, gbo, n, k, kind):
    rng = np.random.default_rng(n + k)
    if kind == "gauss":
        v = rng.standard_normal(n).astype(np.float32)
    elif kind == "ties":
        v = (np.round(rng.standard_normal(n) * 4) / 4).astype(np.float32)
    else:  # subnormal and zero magnitudes: the low radix digits decide
        v = (rng.integers(-50, 50, n) * np.float32(1e-40)).astype(np.float32)
    bins = rng.integers(0, 5, n).astype(np.int32)
    # a new T (T <= max_change), then a lowered T on the result
    xg, bg, Tg = _sort_gpu(gb, v, bins, 0.0, 1.0, k)
    xo, bo, To = gbo.find_support_set_sort(v, bins, 0.0, 1.0, k)
    assert Tg == To == np.sort(np.abs(v))[n - k]
    assert np.array_equal(xg, xo) and np.array_equal(bg, bo)
    mc = np.float32(To / 3)
    xg2, bg2, Tg2 = _sort_gpu(gb, xg, bg, To, mc, k)
    xo2, bo2, To2 = gbo.find_support_set_sort(xo, bo, To, mc, k)
    assert Tg2 == To2
    assert np.array_equal(xg2, xo2) and np.array_equal(bg2, bo2)


def test_find_support_set_sort_rejects_bad_k(gb):
    with pytest.raises(gb.GagaError):
        _sort_gpu(gb, np.ones(10, np.float32), np.zeros(10, np.int32), 0.0, 1.0, 11)


def _dense(gbo, k, seed):
    n, m = 4096, 1024
    A = gbo.gen_dense(m, n, seed)
    x0, ks = gbo.gen_vector(n, k, 1, seed)
    return gbo.Op.dense(A, m, n), x0, ks, ("gen", (A.reshape(n, m).T.copy(),))


def _dct(gbo, k, seed):
    n = 2 ** 14
    m = n // 4
    rows = gbo.gen_dct_rows(n, m, seed=seed)
    x0, ks = gbo.gen_vector(n, k, 2, seed=seed)
    return gbo.Op.dct(n, rows), x0, ks, ("dct", (rows,))


def _smv(gbo, k, seed):
    n, m, d = 2 ** 14, 2 ** 12, 7
    rows, vals = gbo.gen_smv(m, n, d, 1, seed=seed)
    x0, ks = gbo.gen_vector(n, k, 1, seed=seed)
    return gbo.Op.smv(m, n, d, rows, vals), x0, ks, ("smv", (rows, vals, d))


def _solve_gpu(gb, alg, op, y, ks, opts, spec):
    kind, extra = spec
    if kind == "gen":
        x, it, conv = gb.gaga_cs(alg, "gen", y, extra[0], ks, opts)
    elif kind == "dct":
        x, it, conv = gb.gaga_cs(alg, "dct", y, extra[0], ks, op.m, op.n, opts, index_base=0)
    else:
        rows, vals, d = extra
        cols = np.repeat(np.arange(op.n, dtype=np.int32), d)
        x, it, conv, rec, trec = gb.gaga_cs(alg, "smv", y, rows, cols, vals, ks, opts, index_base=0)
    return np.asarray(x), it


CASES = [("dense", _dense, 20), ("dense", _dense, 102), ("dense", _dense, 230), ("dct", _dct, 100),
         ("smv", _smv, 60)]


@pytest.mark.parametrize("alg", ["NIHT", "HTP"])
@pytest.mark.parametrize("supp_flag", [0, 1, 2, 3])
@pytest.mark.parametrize("name,make,k", CASES)
def test_timing_variant_matches_oracle(gb, gbo, alg, supp_flag, name, make, k):
    op, x0, ks, spec = make(gbo, k, seed=60 + k)
    y = gbo.A(op, x0)
    tol = 1e-5 * float(np.linalg.norm(y))
    alpha = 0.25 if supp_flag != 1 else 0.5
    opts = gb.gaga_options("tol", tol, "timing", "on", "supportFlag", supp_flag, "alpha", alpha)
    x, it = _solve_gpu(gb, alg, op, y, ks, opts, spec)
    xo, info = gbo.solve(alg, op, y, ks, tol, timing=1, supp_flag=supp_flag, alpha=alpha)
    ok_gpu = np.linalg.norm(x - x0) / np.linalg.norm(x0) <= 1e-3
    ok_ora = np.linalg.norm(xo - x0) / np.linalg.norm(x0) <= 1e-3
    assert ok_gpu == ok_ora, (alg, supp_flag, name, k, it, info.iter)
    if ok_ora:
        assert np.linalg.norm(x - xo) / np.linalg.norm(xo) < 1e-4
        assert abs(it - info.iter) <= 3, (it, info.iter)
    t = gb.last_timings()
    assert t is not None and len(t["time_per_iteration"]) == it


@pytest.mark.parametrize("alg", ["NIHT", "HTP"])
def test_timing_records_and_file(gb, tmp_path, alg):
    """generate-and-solve with timing on: per-iteration records (positive iteration times,
    the support step inside them, HTP's CG steps in 1..15) whose mean is timeIter, and the
    gpu_timings[_HTP]_data_gen file with one line per iteration."""
    opts = gb.gaga_options("tol", 1e-5, "tol_is_relative", 1, "seed", 11, "timing", "on", "supportFlag", 3,
                           "resultsDir", str(tmp_path))
    norms, times, iters, supp, conv, x = gb.gaga_cs(alg, "gen", 40, 1024, 4096, opts)
    assert norms[1] < 1e-3 and iters > 0
    t = gb.last_timings()
    tpi, tss = t["time_per_iteration"], t["time_supp_set"]
    assert len(tpi) == iters and np.all(tpi > 0) and np.all(tss > 0) and np.all(tss <= tpi)
    assert abs(times[1] - tpi.mean()) <= 1e-6 * max(1.0, float(tpi.mean()))
    assert float(tpi.sum()) <= float(times[0]) * 1.01
    if alg == "HTP":
        cg = t["cg_per_iteration"]
        assert np.all((cg >= 0) & (cg <= 15)) and cg.sum() > 0
        assert np.all(t["time_for_cg"] <= tpi)
    files = [f for f in os.listdir(tmp_path) if f.startswith("gpu_timings")]
    assert len(files) == 1
    assert re.match(r"gpu_timings_%sdata_gen\d{8}\.txt$" % ("HTP_" if alg == "HTP" else ""), files[0])
    lines = open(os.path.join(tmp_path, files[0])).read().splitlines()
    assert lines[0].startswith("%s_S_gen output: k 40, m 1024, n 4096" % alg)
    assert "supp_flag 3 matrixEnsemble 1" in lines[0]
    assert len(lines) == 1 + iters and lines[-1].startswith("iteration %d time_iteration" % (iters - 1))


def test_timing_ignored_by_other_algorithms(gb):
    """Other algorithms run their plain loops with timing on (gaga_gen.cu:331-334)."""
    base = gb.gaga_options("tol", 1e-5, "tol_is_relative", 1, "seed", 12)
    on = gb.gaga_options("tol", 1e-5, "tol_is_relative", 1, "seed", 12, "timing", "on", "supportFlag", 2)
    a = gb.gaga_cs("CGIHT", "gen", 40, 1024, 4096, base)
    b = gb.gaga_cs("CGIHT", "gen", 40, 1024, 4096, on)
    assert a[2] == b[2] and np.array_equal(a[5], b[5])
    assert gb.last_timings() is None


def test_timing_rejects_bad_support_flag(gb):
    with pytest.raises(gb.GagaError):
        gb.gaga_cs("NIHT", "gen", 10, 256, 1024, gb.gaga_options("timing", "on", "supportFlag", 4, "seed", 1))
