"""The generate-and-solve usage (gaga_cs(alg, ens, k, m, n[, p], opts), GAGA/gaga/gaga_gen.cu:90-114,
gaga_dct.cu, gaga_smv.cu:110-130) under each problem-generation option: the signal's value
distribution (vecDistribution uniform / binary / gaussian, GAGA/gaga/createVector.cu), the dense
ensemble (matrixEnsemble gaussian / binary, createMeasurements_gen.cu:81-100), the expander's
values (ones / binary / expander, createMeasurements_smv.cu:178-197), kFixed and noise.

The library draws its problems with the same Philox streams as the oracle's generators, so the
drawn signal is compared with the oracle's draw, and the verdict and solution with the oracle's
solve of the regenerated problem.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

VEC = {"uniform": 0, "binary": 1, "gaussian": 2}


def _rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.mark.parametrize("vec", ["uniform", "binary", "gaussian"])
@pytest.mark.parametrize("ens", ["gaussian", "binary"])
def test_dense_generation_options(gb, gbo, vec, ens):
    n, m, k, seed = 2048, 768, 40, 101
    opts = gb.gaga_options("tol", 1e-5, "tol_is_relative", 1, "seed", seed, "vecDistribution", vec,
                           "matrixEnsemble", ens)
    x, xt, r = gb.generate_and_solve("NIHT", "gen", k, m, n, 0, opts)
    xo_t, ks = gbo.gen_vector(n, k, VEC[vec], seed)
    np.testing.assert_allclose(xt, xo_t, rtol=1e-6, atol=0)
    assert r.k_used == ks
    A = gbo.gen_dense(m, n, seed, 0, 1 if ens == "gaussian" else 2)
    op = gbo.Op.dense(A, m, n)
    y = gbo.A(op, xo_t)
    xo, info = gbo.solve("NIHT", op, y, ks, 1e-5 * float(np.linalg.norm(y)))
    ok_o = _rel(xo, xo_t) <= 1e-3
    assert (r.norms[1] <= 1e-3) == ok_o
    if ok_o:
        assert _rel(x, xo) < 1e-4
        assert abs(r.iter - info.iter) <= 3


@pytest.mark.parametrize("ens", ["ones", "binary", "expander"])
def test_expander_generation_options(gb, gbo, ens):
    n, m, d, k, seed = 4096, 1024, 7, 50, 103
    opts = gb.gaga_options("tol", 1e-5, "tol_is_relative", 1, "seed", seed, "matrixEnsemble", ens)
    x, xt, r = gb.generate_and_solve("NIHT", "smv", k, m, n, d, opts)
    xo_t, ks = gbo.gen_vector(n, k, 1, seed)
    assert np.array_equal(xt, xo_t)
    rows, vals = gbo.gen_smv(m, n, d, {"ones": 1, "binary": 2, "expander": 3}[ens], seed)
    op = gbo.Op.smv(m, n, d, rows, vals)
    y = gbo.A(op, xo_t)
    xo, info = gbo.solve("NIHT", op, y, ks, 1e-5 * float(np.linalg.norm(y)))
    ok_o = _rel(xo, xo_t) <= 1e-3
    assert (r.norms[1] <= 1e-3) == ok_o
    if ok_o:
        assert _rel(x, xo) < 1e-4


def test_dct_generation(gb, gbo):
    n, k, seed = 2 ** 14, 200, 105
    m = n // 4
    opts = gb.gaga_options("tol", 1e-5, "tol_is_relative", 1, "seed", seed, "vecDistribution", "gaussian")
    x, xt, r = gb.generate_and_solve("CGIHT", "dct", k, m, n, 0, opts)
    xo_t, ks = gbo.gen_vector(n, k, 2, seed)
    np.testing.assert_allclose(xt, xo_t, rtol=1e-6, atol=0)
    rows = gbo.gen_dct_rows(n, m, seed)
    op = gbo.Op.dct(n, rows)
    y = gbo.A(op, xo_t)
    xo, info = gbo.solve("CGIHT", op, y, ks, 1e-5 * float(np.linalg.norm(y)))
    ok_o = _rel(xo, xo_t) <= 1e-3
    assert (r.norms[1] <= 1e-3) == ok_o
    if ok_o:
        assert _rel(x, xo) < 1e-3


def test_kfixed_redraws_until_exact_k(gb, gbo):
    """kFixed: the support scheme can draw more than k entries; the generator redraws with
    seed + 1, + 2, ... until exactly k (gaga_gen.cu kFixed option)."""
    n, m, k, seed = 1024, 400, 60, 7
    opts = gb.gaga_options("tol", 1e-5, "tol_is_relative", 1, "seed", seed, "kFixed", "on")
    x, xt, r = gb.generate_and_solve("NIHT", "gen", k, m, n, 0, opts)
    assert r.k_used == k and np.count_nonzero(xt) == k
    s = seed
    while True:
        xo_t, ks = gbo.gen_vector(n, k, 1, s)
        if ks == k:
            break
        s += 1
    assert np.array_equal(xt, xo_t)


def test_dense_noise(gb):
    """noise: y = A x + e with ||e|| = noise ||A x|| (createProblem_gen.cu:244-254): the
    solution's error sits at the noise level, neither exact nor lost."""
    opts = gb.gaga_options("tol", 1e-5, "tol_is_relative", 1, "seed", 11, "noise", 0.01)
    x, xt, r = gb.generate_and_solve("CGIHT", "gen", 30, 1024, 4096, 0, opts)
    assert 1e-4 < r.norms[1] < 0.05
