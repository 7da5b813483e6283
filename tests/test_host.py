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
    names = (b"NIHT", b"HTP", b"IHT", b"ThresholdSD", b"ThresholdCG", b"CSMPSP", b"CGIHT", b"FIHT", b"ALPS",
             b"CGIHTprojected", b"smp", b"ssmp", b"er", b"parallel_lddsr", b"parallel_l0", b"er_naive",
             b"ssmp_naive", b"parallel_l0_swipe", b"ALPS2")
    assert [L.gb_cs_alg_id(a) for a in names] == [0, 1, 2, 3, 4, 5, 6, 7, 8, 9, 10, 11, 12, 13, 14, 16, 17, 18, -1]


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


def test_result_file_lines_match_reference_format(gb, tmp_path):
    """gb_cs_write_result appends File_output_gen / File_output / File_output_smv lines
    (GAGA/gaga/functions.cu:34-80) to the dated gpu_data_* files."""
    L = gb._lib.load()
    o = gb._lib.Options()
    L.gb_cs_default_options(C.byref(o), b"NIHT", 4096)
    o.seed = 17
    r = gb._lib.Result()
    r.norms[0], r.norms[1], r.norms[2] = 1.5e-5, 2.25e-5, 3.0e-5
    r.times[0], r.times[1], r.times[2] = 12.5, 0.5, 40.0
    r.iter, r.conv_rate = 25, 0.75
    for j, v in enumerate((102, 0, 3994, 0)):
        r.support[j] = v
    buf = C.create_string_buffer(512)
    assert L.gb_cs_write_result(str(tmp_path).encode(), b"NIHT", 0, 102, 1024, 4096, 0, C.byref(o), C.byref(r), buf,
                                512) == 0
    path = buf.value.decode()
    assert re.search(r"gpu_data_gen\d{8}\.txt$", path)
    tail = ("errorl1 %0.7e errorl2 %0.7e errorlinf %0.7e timeALG %0.7e timeIter %0.7e timeTotal %0.7e "
            "iterations %d converge_rate %0.7e TruePos %d FalsePos %d TrueNeg %d FalseNeg %d " % (
                np.float32(1.5e-5), np.float32(2.25e-5), np.float32(3.0e-5), 12.5, 0.5, 40.0, 25, 0.75, 102, 0,
                3994, 0))
    want = "NIHT_S_gen output: k 102, m 1024, n 4096, vecDistribution 1 matrixEnsemble 1 " + tail + "seed 17 \n"
    assert open(path).read() == want
    # DCT and expander lines, and the noise file name
    o.noise = 0.01
    assert L.gb_cs_write_result(str(tmp_path).encode(), b"CGIHT", 2, 10, 100, 400, 7, C.byref(o), C.byref(r), buf,
                                512) == 0
    path = buf.value.decode()
    assert path.endswith("_noise0.010.txt") and "gpu_data_smv" in path
    line = open(path).read()
    assert line.startswith("CGIHT_S_smv output: k 10, m 100, n 400, vecDistribution 1 nonzeros_per_column 7 "
                           "matrixEnsemble 3 errorl1")
    assert line.endswith("seed 17 band_percentage 0.00 noise_level 0.0100 \n")
    o.noise = 0.0
    assert L.gb_cs_write_result(str(tmp_path).encode(), b"HTP", 1, 10, 100, 512, 0, C.byref(o), C.byref(r), buf,
                                512) == 0
    assert open(buf.value.decode()).read().startswith("HTP_S_dct output: k 10, m 100, n 512, vecDistribution 1 error")


def test_timing_result_file_lines_match_reference_format(gb, tmp_path):
    """With timing on, NIHT and HTP results go to gpu_timings[_HTP]_data_* files: the
    File_output_timings* summary line, then one line per iteration
    (GAGA/gaga/functions.cu:82-208, results.cu:1206,1375,1545,1716,1890,2061)."""
    L = gb._lib.load()
    o = gb._lib.Options()
    L.gb_cs_default_options(C.byref(o), b"NIHT", 4096)
    o.seed, o.timing, o.support_flag, o.alpha = 5, 1, 2, 0.125
    r = gb._lib.Result()
    r.norms[0], r.norms[1], r.norms[2] = 1e-6, 2e-6, 3e-6
    r.times[0], r.times[1], r.times[2] = 4.0, 2.0, 9.0
    r.iter, r.conv_rate = 2, 0.5
    for j, v in enumerate((20, 0, 4076, 0)):
        r.support[j] = v
    tpi = np.array([1.5, 2.5], dtype=np.float32)
    tss = np.array([0.25, 0.5], dtype=np.float32)
    cgi = np.array([3, 15], dtype=np.float32)
    tcg = np.array([0.75, 1.25], dtype=np.float32)
    r.time_per_iteration, r.time_supp_set = tpi.ctypes.data, tss.ctypes.data
    r.cg_per_iteration, r.time_for_cg = cgi.ctypes.data, tcg.ctypes.data
    buf = C.create_string_buffer(512)
    d = str(tmp_path).encode()
    assert L.gb_cs_write_result(d, b"NIHT", 0, 20, 1024, 4096, 0, C.byref(o), C.byref(r), buf, 512) == 0
    path = buf.value.decode()
    assert re.search(r"gpu_timings_data_gen\d{8}\.txt$", path)
    head = ("NIHT_S_gen output: k 20, m 1024, n 4096, vecDistribution 1 errorl1 %0.7e errorl2 %0.7e "
            "errorlinf %0.7e timeALG %0.7e timeIter %0.7e timeTotal %0.7e iterations 2 converge_rate %0.7e "
            "TruePos 20 FalsePos 0 TrueNeg 4076 FalseNeg 0 seed 5 alpha %0.7e supp_flag 2 matrixEnsemble 1 \n" % (
                np.float32(1e-6), np.float32(2e-6), np.float32(3e-6), 4.0, 2.0, 9.0, 0.5, 0.125))
    body = "".join("iteration %d time_iteration %0.7e time_supp_set %0.7e\n" % (j, tpi[j], tss[j]) for j in range(2))
    assert open(path).read() == head + body
    # HTP on the DCT: its own file, the CG columns, no matrixEnsemble
    assert L.gb_cs_write_result(d, b"HTP", 1, 20, 1024, 4096, 0, C.byref(o), C.byref(r), buf, 512) == 0
    path = buf.value.decode()
    assert re.search(r"gpu_timings_HTP_data_dct\d{8}\.txt$", path)
    lines = open(path).read().splitlines(keepends=True)
    assert lines[0].startswith("HTP_S_dct output: k 20,") and lines[0].endswith("alpha 1.2500000e-01 supp_flag 2 \n")
    assert lines[2] == "iteration 1 time_iteration %0.7e time_supp_set %0.7e cg_per_iteration 15 time_for_cg %0.7e\n" % (
        2.5, 0.5, 1.25)
    # expander: NonzerosPerCol and matrixEnsemble close the summary line
    assert L.gb_cs_write_result(d, b"NIHT", 2, 20, 1024, 4096, 7, C.byref(o), C.byref(r), buf, 512) == 0
    assert open(buf.value.decode()).readline().endswith("supp_flag 2 NonzerosPerCol 7 matrixEnsemble 3 \n")
    # without the per-iteration arrays the timing file cannot be written
    r.time_per_iteration = None
    assert L.gb_cs_write_result(d, b"NIHT", 0, 20, 1024, 4096, 0, C.byref(o), C.byref(r), buf, 512) != 0


def test_mex_shim_builds_and_rejects_bad_calls(gb):
    """The MEX gateways (gaga_gb300/mex/gb_gaga_mex.cpp) compile against a MATLAB API
    (the stand-in mex.h) with -Wall -Wextra -Werror and link to libgb_cs.so.  Calls that
    the reference rejects (unknown algorithm, wrong output count, GAGA/gaga/gaga_gen.cu:49-50,
    85-87) raise the gateway error and leave every output unset; none reaches the GPU."""
    import numpy as np

    import mex_shim
    from oracle import ref_gateway as rg

    for g in ("gen", "dct", "smv"):
        L = mex_shim.load(g)
        y = np.ones(8, np.float32)
        if g == "gen":
            args = rg.gen_args(L, "NOT_AN_ALG", y, np.ones((8, 16), np.float32), 2)
        elif g == "dct":
            args = rg.dct_args(L, "NOT_AN_ALG", y, np.arange(1, 9, dtype=np.int32), 2, 8, 16)
        else:
            cols = np.repeat(np.arange(1, 17, dtype=np.int32), 2)
            args = rg.smv_args(L, "NOT_AN_ALG", y, np.ones(32, np.int32), cols, np.ones(32, np.float32), 2)
        L.gbmx_clear_error()
        outs = rg.call(L, 5 if g == "smv" else 3, args)
        assert all(o is None for o in outs) and b"unknown algorithm" in L.gbmx_last_error()
        L.gbmx_clear_error()
        outs = rg.call(L, 2, rg.gen_args(L, "NIHT", y, np.ones((8, 16), np.float32), 2))
        assert all(o is None for o in outs) and b"usage" in L.gbmx_last_error()


def test_transition_operand_policy():
    """24-bit operand within the band around rho*(delta), BF16 elsewhere; rho* from verdicts
    is the smallest 0.02-grid rho where fewer than half recover."""
    import numpy as np

    from gaga_gb300 import transition

    n = np.full(5, 1000)
    m = np.full(5, 500)  # delta 0.5: rho* = 0.32
    k = np.array([50, 120, 160, 200, 240])  # rho 0.10, 0.24, 0.32, 0.40, 0.48
    assert list(transition.operand_formats(n, m, k, band0=0.08, exp=0.0)) == ["bf16", "a24", "a24", "a24", "bf16"]
    # the band narrows with n: 0.08 at n = 1024, 0.08 / 2 at n = 1024 * 2^(1 / 0.3)
    assert abs(float(transition.band(1024)) - 0.08) < 1e-12
    assert abs(float(transition.band(1024 * 2 ** (1 / 0.3))) - 0.04) < 1e-9
    nn = np.full(3, 16384)
    mm = np.full(3, 8192)  # rho* = 0.32, band 0.035
    assert list(transition.operand_formats(nn, mm, np.array([2130, 2621, 2950]))) == ["bf16", "a24", "bf16"]
    rho = np.round(np.arange(0.02, 0.52, 0.02), 2)
    nn = np.full(len(rho), 1000)
    mm = np.full(len(rho), 500)
    kk = np.round(rho * 500).astype(int)
    ok = (rho < 0.3).astype(int)
    assert transition.rho_star_from_verdicts(nn, mm, kk, ok) == {0.5: 0.3}


def test_sweep_partial_round_spreads_over_the_grid():
    """3072 independent trials = 2 rounds of the 1125-point grid + 822 points of a third,
    which the strided order spreads over every n (not the grid's first, small-n points)."""
    import collections

    import numpy as np

    from gaga_gb300 import sweep

    n, m, k, tid = sweep.sweep_trials(3072)
    per_n = collections.Counter(n.tolist())
    assert set(per_n) == set(sweep.N_VALUES)
    assert max(per_n.values()) - min(per_n.values()) <= 25
    pts = collections.Counter(zip(n.tolist(), m.tolist(), k.tolist()))
    assert len(pts) == len(sweep.grid()) and set(pts.values()) <= {2, 3}
    assert len(set(tid.tolist())) == 3072
