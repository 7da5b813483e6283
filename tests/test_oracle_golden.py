"""The oracle pinned against the golden fixtures (tests/golden, written by
tests/golden/make_golden.py from the reference's own source run on the CPU, and from
scipy's orthonormal DCT).  CPU only."""
import os

import numpy as np
import pytest

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load(name):
    return np.load(os.path.join(GOLD, name))


def test_linear_binning_matches_reference(gbo):
    z = load("linear_binning.npz")
    assert len(z["names"]) >= 5
    for name in z["names"]:
        bins, cnt = gbo.linear_binning(z[f"{name}__v"], int(z[f"{name}__num_bins"]), int(z[f"{name}__max_bin"]),
                                       float(z[f"{name}__slope"]), float(z[f"{name}__intercept"]))
        assert np.array_equal(bins, z[f"{name}__bins"]), name
        assert np.array_equal(cnt, z[f"{name}__counters"]), name


def test_threshold_matches_reference(gbo):
    z = load("threshold.npz")
    v, bins = z["v"], z["bins"]
    for kb in z["k_bins"]:
        a = v.copy()
        gbo.lib().gbo_threshold(a.ctypes.data, bins.ctypes.data, int(kb), len(a))
        assert np.array_equal(a, z[f"threshold_{kb}"])
        b = np.where(bins <= kb, v, np.float32(0))
        assert np.array_equal(b, z[f"threshold_one_{kb}"])


def test_support_evolution_matches_reference(gbo):
    z = load("support_evolution.npz")
    for i in range(int(z["count"])):
        cur, prev = z[f"c{i}__cur"], z[f"c{i}__prev"]
        kc, kp = int(z[f"c{i}__kcur"]), int(z[f"c{i}__kprev"])
        changed = int(np.any((prev <= kp) & (cur > kc)))
        assert changed == int(z[f"c{i}__flag"] > 0)


def test_l0_step_matches_reference(gbo):
    z = load("l0_step.npz")
    for i in range(int(z["count"])):
        g = lambda key: z[f"c{i}__{key}"]
        n, d, shift = int(g("n")), int(g("d")), int(g("shift"))
        x, upd, found = gbo.l0_scores(g("res"), np.zeros(n, np.float32), g("rows"), n, d, 1, shift)
        assert found == int(g("found"))
        assert np.array_equal(x, g("x_after"))
        assert np.array_equal(upd, g("updates"))
        res2 = gbo.l0_update_residual(g("res"), g("rows"), upd, n, d)
        assert np.array_equal(res2, g("res_after"))


def test_serial_l0_matches_reference(gbo):
    z = load("serial_l0.npz")
    for i in range(int(z["count"])):
        g = lambda key: z[f"c{i}__{key}"]
        m, n, d = int(g("m")), int(g("n")), int(g("d"))
        op = gbo.Op.smv(m, n, d, g("rows"), np.ones(n * d, np.float32))
        x, res, rec, info = gbo.serial_l0(op, g("y"), tol=1e-6, maxiter=int(g("maxiter")))
        it = int(g("iter"))
        assert info.iter == it
        assert np.array_equal(x, g("x"))
        assert np.array_equal(res, g("res"))
        assert np.array_equal(rec[:it], g("rec")[:it])


def test_dct_matches_scipy(gbo):
    z = load("dct_scipy.npz")
    for N in z["sizes"]:
        x = z[f"N{N}__x"]
        d2, d3 = gbo.dct2(x), gbo.dct3(x)
        np.testing.assert_allclose(d2, z[f"N{N}__dct2"], rtol=0, atol=1e-5 * np.abs(z[f"N{N}__dct2"]).max())
        np.testing.assert_allclose(d3, z[f"N{N}__dct3"], rtol=0, atol=1e-5 * np.abs(z[f"N{N}__dct3"]).max())


def test_ref_library_matches_fixtures_when_present(gbo):
    """Where the reference tree is present, its CPU build still reproduces the fixtures."""
    R = gbo.ref_lib()
    if R is None:
        pytest.skip("reference tree not present")
    import ctypes as C

    z = load("linear_binning.npz")
    name = z["names"][0]
    v = z[f"{name}__v"].copy()
    nb, mb = int(z[f"{name}__num_bins"]), int(z[f"{name}__max_bin"])
    bins = np.zeros(len(v), np.int32)
    cnt = np.zeros(nb, np.int32)
    R.ref_linear_binning(v.ctypes.data, bins.ctypes.data, cnt.ctypes.data, nb, mb, len(v),
                         C.c_float(float(z[f"{name}__slope"])), C.c_float(float(z[f"{name}__intercept"])))
    assert np.array_equal(bins, z[f"{name}__bins"])


@pytest.mark.parametrize("alg", ["IHT", "ThresholdSD", "ThresholdCG", "CSMPSP", "FIHT", "ALPS", "CGIHTprojected"])
def test_oracle_remaining_algorithms_recover_easy_problem(gbo, alg):
    """IHT, ThresholdSD and ThresholdCG restated from the reference recover a problem well
    inside their recovery region (one-step thresholding needs a small rho)."""
    n, m, k = 4096, 1024, 20
    A = gbo.gen_dense(m, n, 12)
    x0, ks = gbo.gen_vector(n, k, 1, 12)
    op = gbo.Op.dense(A, m, n)
    y = gbo.A(op, x0)
    x, info = gbo.solve(alg, op, y, ks, 1e-5 * float(np.linalg.norm(y)))
    assert np.linalg.norm(x - x0) / np.linalg.norm(x0) < 1e-3, (alg, info.iter)


@pytest.mark.parametrize("variant", ["parallel_l0", "parallel_lddsr", "parallel_l0_swipe"])
def test_oracle_l0_variants_decode(gbo, variant):
    """The expander decoders recover a +-1 signal well inside their recovery region."""
    n, m, d = 4096, 1024, 7
    rows, vals = gbo.gen_smv(m, n, d, 3, seed=23)
    x0, ks = gbo.gen_vector(n, 20, 1, seed=23)
    op = gbo.Op.smv(m, n, d, rows, vals)
    y = gbo.A(op, x0)
    x, res, rec, info = gbo.parallel_l0(op, y, tol=1e-6, maxiter=300, variant=variant)
    assert np.array_equal(x, x0), (variant, info.iter)


def test_oracle_sort_support(gbo):
    """FindSupportSet_sort restated: T is element n-k of |v| sorted ascending and the new
    bins are 1 / 2 around it; a lowered T thresholds without touching surviving bins
    (GAGA/gaga/functions.cu:446-465, kernels.cu:85-95)."""
    rng = np.random.default_rng(3)
    v = np.round(rng.standard_normal(5000) * 8).astype(np.float32) / 8  # many ties
    k = 300
    x, b, T = gbo.find_support_set_sort(v, np.full(5000, 7, np.int32), 0.0, 1.0, k)
    assert T == np.sort(np.abs(v))[5000 - k]
    keep = np.abs(v) >= T
    assert np.array_equal(x, np.where(keep, v, 0)) and np.array_equal(b, np.where(keep, 1, 2))
    b[:10] = 9
    x2, b2, T2 = gbo.find_support_set_sort(x, b, T, np.float32(0.25), k)
    assert T2 == np.float32(T - np.float32(0.25))
    assert np.array_equal(b2[:10], np.where(np.abs(x[:10]) < T2, 2, 9))


@pytest.mark.parametrize("alg", ["NIHT", "HTP"])
@pytest.mark.parametrize("supp_flag", [0, 1, 2, 3])
def test_oracle_timing_variants_recover(gbo, alg, supp_flag):
    """The timing variants (algorithms_timings.cu) recover an easy dense problem with every
    supportFlag, as the plain loops do."""
    n, m, k = 2048, 512, 25
    A = gbo.gen_dense(m, n, 8)
    x0, ks = gbo.gen_vector(n, k, 1, 8)
    op = gbo.Op.dense(A, m, n)
    y = gbo.A(op, x0)
    x, info = gbo.solve(alg, op, y, ks, 1e-5 * float(np.linalg.norm(y)), timing=1, supp_flag=supp_flag)
    assert np.linalg.norm(x - x0) / np.linalg.norm(x0) < 1e-3 and info.iter > 0


@pytest.mark.parametrize("alg", ["ssmp", "er", "ssmp_naive", "er_naive"])
def test_oracle_sequential_decoders(gbo, alg):
    """ssmp / er and their naive forms decode a +-1 signal on the unit expander exactly; the
    naive forms (every score recomputed) follow the same path as the incremental ones."""
    n, m, d, k = 2 ** 12, 2 ** 10, 7, 40
    rows, vals = gbo.gen_smv(m, n, d, 3, seed=5)
    x0, ks = gbo.gen_vector(n, k, 1, seed=5)
    op = gbo.Op.smv(m, n, d, rows, vals)
    y = gbo.A(op, x0)
    x, res, rec, info = gbo.seq_decode(alg, op, y, ks, 1e-6, 2000)
    assert np.array_equal(x, x0)
    base = alg.replace("_naive", "")
    xb, resb, recb, infob = gbo.seq_decode(base, op, y, ks, 1e-6, 2000)
    assert info.iter == infob.iter and np.array_equal(rec, recb)


def test_oracle_counts_cgiht_steps(gbo):
    """The oracle's CGIHT reports how many of its iterations were unrestricted and restricted
    CG steps: they add up to the iterations, the first step (restartFlag off) is unrestricted,
    and with restartFlag on every step is restricted."""
    import numpy as np

    rng = np.random.default_rng(11)
    m, n, k = 128, 256, 20
    A = (rng.standard_normal((m, n)) / np.sqrt(m)).astype(np.float32)
    x0 = np.zeros(n, np.float32)
    x0[rng.choice(n, k, replace=False)] = rng.choice([-1.0, 1.0], k)
    y = (A @ x0).astype(np.float32)
    op = gbo.Op.dense(np.asfortranarray(A).ravel(order="F"), m, n)
    tol = 1e-4 * float(np.linalg.norm(y))
    x, info = gbo.solve("CGIHT", op, y, k, tol, maxiter=500)
    assert info.iter > 1 and info.ucg_steps + info.rcg_steps == info.iter
    assert info.ucg_steps >= 1
    x, info = gbo.solve("CGIHT", op, y, k, tol, maxiter=500, restart=1)
    assert info.ucg_steps == 0 and info.rcg_steps == info.iter
