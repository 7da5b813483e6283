"""Cluster-resident NIHT (gb_resident.cu): the batched form's small trials, one thread-block
cluster per trial, against the single-trial drop-in, the slot graphs and the CPU oracle.

Both forms solve bit-identical problems (seed + trial id); the resident kernel sums in a
different order (per-CTA partials combined in rank order), so success verdicts must agree
on almost every trial and recovered signals must meet the 1e-3 verdict in both.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SEED = 777


def pick(ns, count, seed_total=4096):
    from gaga_gb300 import sweep

    n, m, k, tid = sweep.sweep_trials(seed_total)
    idx = np.flatnonzero(np.isin(n, ns))
    idx = idx[np.linspace(0, len(idx) - 1, count).astype(int)]
    return n[idx], m[idx], k[idx], tid[idx]


def plain(gb, n, m, k, tid, maxiter):
    opts = gb.gaga_options("tol", 1e-4, "tol_is_relative", 1, "maxiter", maxiter, "seed", int(SEED + tid))
    x, xt, r = gb.generate_and_solve("NIHT", "gen", int(k), int(m), int(n), 0, opts)
    return r


@pytest.mark.parametrize("cluster", [1, 2, 4])
def test_resident_matches_plain(gb, cluster):
    n, m, k, tid = pick([1024, 2048], 24)
    ns, iters, err, ok = gb.solve_batch(n, m, k, SEED, tid, alg="NIHT", maxiter=1000, resident_n=4096,
                                        cluster=cluster)
    agree = 0
    for i in range(len(n)):
        r = plain(gb, n[i], m[i], k[i], tid[i], 1000)
        v_plain = r.norms[1] <= 1e-3
        agree += int(v_plain == bool(ok[i]))
        if v_plain and ok[i]:
            assert err[i] < 1e-3
            assert abs(int(iters[i]) - int(r.iter)) <= max(3, r.iter // 10), (i, iters[i], r.iter)
    assert agree >= len(n) - 1, (agree, len(n))
    assert ns == int(ok.sum()) and 0 < ns < len(n)


def test_resident_matches_slots_and_is_deterministic(gb):
    """n = 1024 ... 4096 through the resident kernel (automatic cluster size) and through the
    slot graphs alone; the resident result repeats bit for bit."""
    n, m, k, tid = pick([1024, 2048, 4096], 48)
    res = gb.solve_batch(n, m, k, SEED, tid, alg="NIHT", maxiter=1000, resident_n=4096)
    again = gb.solve_batch(n, m, k, SEED, tid, alg="NIHT", maxiter=1000, resident_n=4096)
    slots = gb.solve_batch(n, m, k, SEED, tid, alg="NIHT", maxiter=1000, resident_n=-1)
    assert np.array_equal(res[1], again[1]) and np.array_equal(res[2], again[2])
    assert np.sum(res[3] == slots[3]) >= len(n) - 1
    both = (res[3] == 1) & (slots[3] == 1)
    assert np.all(res[2][both] < 1e-3)
    b, ms = gb.batch_last_stats()
    assert b > 0 and ms > 0


def test_resident_with_large_trials_alongside(gb):
    """Small trials in the resident kernel while n = 8192 / 16384 trials run in the slot
    graphs at the same time; every verdict as in the slots-only solve."""
    n, m, k, tid = pick([1024, 2048, 4096, 8192, 16384], 20)
    res = gb.solve_batch(n, m, k, SEED, tid, alg="NIHT", maxiter=600, resident_n=4096)
    slots = gb.solve_batch(n, m, k, SEED, tid, alg="NIHT", maxiter=600, resident_n=-1)
    assert np.sum(res[3] == slots[3]) >= len(n) - 1
    assert res[0] == int(res[3].sum())


def test_resident_n8192(gb):
    """n = 8192 trials (four CTAs per cluster by default) against the slot graphs."""
    n, m, k, tid = pick([8192], 8)
    res = gb.solve_batch(n, m, k, SEED, tid, alg="NIHT", maxiter=600, resident_n=8192)
    slots = gb.solve_batch(n, m, k, SEED, tid, alg="NIHT", maxiter=600, resident_n=-1)
    assert np.sum(res[3] == slots[3]) >= len(n) - 1


def test_resident_matches_oracle(gb, gbo):
    n, m, k, tid = pick([1024, 2048], 8)
    ns, iters, err, ok = gb.solve_batch(n, m, k, SEED, tid, alg="NIHT", maxiter=1000, resident_n=4096)
    ok_o, it_o, err_o = gbo.solve_dense_trials(n, m, k, SEED, tid, alg="NIHT", tol_rel=1e-4, maxiter=1000)
    assert np.sum((err_o <= 1e-3) == ok.astype(bool)) >= len(n) - 1


def test_resident_zero_iterations(gb):
    """maxiter = 0: the trial is drawn, H_k(A^T y) is its answer."""
    n, m, k, tid = pick([1024], 4)
    res = gb.solve_batch(n, m, k, SEED, tid, alg="NIHT", maxiter=0, resident_n=4096)
    assert np.all(res[1] == 0) and np.all(np.isfinite(res[2]))


def test_resident_rejects_oversized_cluster(gb):
    n, m, k, tid = pick([1024], 2)
    with pytest.raises(gb.GagaError):
        gb.solve_batch(n, m, k, SEED, tid, alg="NIHT", resident_n=4096, cluster=32)


@pytest.mark.parametrize("cluster", [1, 3, 4, 8])
def test_resident_ragged_sizes(gb, cluster):
    """n and m that are not multiples of 4, 32 or the cluster size, tiny and one-row
    problems: the column and row shares and the zero-padded rows must cover every entry
    exactly once, so verdicts match the slot graphs."""
    n = np.array([16, 17, 33, 100, 257, 1000, 1001, 2047, 3001, 5000, 777, 64], dtype=np.int32)
    m = np.array([1, 9, 20, 37, 130, 333, 500, 999, 1500, 2501, 388, 63], dtype=np.int32)
    k = np.maximum(1, (m // 8)).astype(np.int32)
    tid = np.arange(len(n), dtype=np.uint32) + 40000
    res = gb.solve_batch(n, m, k, SEED, tid, alg="NIHT", maxiter=500, resident_n=8192, cluster=cluster)
    slots = gb.solve_batch(n, m, k, SEED, tid, alg="NIHT", maxiter=500, resident_n=-1)
    assert np.all(np.isfinite(res[2]))
    assert np.sum(res[3] == slots[3]) >= len(n) - 1, (res[3], slots[3])
    both = (res[3] == 1) & (slots[3] == 1)
    assert np.all(res[2][both] < 1e-3)


def test_resident_largest_rows(gb):
    """m up to 8192 rows (four row quads per thread in A x_S) at n = 8192."""
    n = np.array([8192, 8192, 8192], dtype=np.int32)
    m = np.array([8192, 7373, 4096], dtype=np.int32)
    k = np.array([400, 1500, 800], dtype=np.int32)
    tid = np.arange(3, dtype=np.uint32) + 50000
    res = gb.solve_batch(n, m, k, SEED, tid, alg="NIHT", maxiter=400, resident_n=8192, cluster=8)
    slots = gb.solve_batch(n, m, k, SEED, tid, alg="NIHT", maxiter=400, resident_n=-1)
    assert np.array_equal(res[3], slots[3])
    assert np.all(res[2][res[3] == 1] < 1e-3)


def _dense(gbo, n, m, k, seed):
    A = gbo.gen_dense(m, n, seed, 0, 1)
    x0, ks = gbo.gen_vector(n, k, 1, seed)
    op = gbo.Op.dense(A, m, n)
    return A, x0, ks, op, gbo.A(op, x0)


@pytest.mark.parametrize("alg,restart", [("NIHT", "off"), ("HTP", "off"), ("CGIHT", "off"), ("CGIHT", "on")])
@pytest.mark.parametrize("n,m,k", [(1024, 400, 40), (2048, 1024, 200), (4096, 1024, 102), (3000, 1200, 330)])
def test_single_trial_on_one_cluster_matches_oracle(gb, gbo, alg, restart, n, m, k):
    """The drop-in's dense NIHT / HTP / CGIHT (restartFlag off and on), which runs on one cluster at
    these sizes: same verdict as the oracle's solve of the same problem; when recovered, x
    within 1e-4, the same support and iterations within 3."""
    A, x0, ks, op, y = _dense(gbo, n, m, k, seed=n + m + k)
    tol = 1e-4 * float(np.linalg.norm(y))
    opts = gb.gaga_options("tol", tol, "restartFlag", restart)
    x, iters, conv = gb.gaga_cs(alg, "gen", y, A.reshape(n, m).T, ks, opts)
    xo, info = gbo.solve(alg, op, y, ks, tol, restart=1 if restart == "on" else 0)
    ok, ok_o = (np.linalg.norm(v - x0) / np.linalg.norm(x0) <= 1e-3 for v in (x, xo))
    assert ok == ok_o
    if ok:
        assert np.linalg.norm(x - xo) / np.linalg.norm(xo) < 1e-4
        assert np.array_equal(np.flatnonzero(x), np.flatnonzero(xo))
        assert abs(int(iters) - int(info.iter)) <= 3


@pytest.mark.parametrize("alg", ["CGIHT", "HTP"])
def test_batched_resident_matches_slots(gb, alg):
    """Batched CGIHT and HTP: the resident kernel against the slot graphs on the same trials
    (n = 1024 ... 8192), verdicts agreeing on all but at most one, repeat runs bit-identical."""
    n, m, k, tid = pick([1024, 2048, 4096, 8192], 40)
    res = gb.solve_batch(n, m, k, SEED, tid, alg=alg, maxiter=800, resident_n=8192)
    again = gb.solve_batch(n, m, k, SEED, tid, alg=alg, maxiter=800, resident_n=8192)
    slots = gb.solve_batch(n, m, k, SEED, tid, alg=alg, maxiter=800, resident_n=-1)
    assert np.array_equal(res[1], again[1]) and np.array_equal(res[2], again[2])
    assert np.sum(res[3] == slots[3]) >= len(n) - 1, (res[3], slots[3])
    both = (res[3] == 1) & (slots[3] == 1)
    assert np.all(res[2][both] < 1e-3)
    assert 0 < res[0] < len(n)


@pytest.mark.parametrize("alg", ["CGIHT", "HTP"])
@pytest.mark.parametrize("cluster", [1, 4])
def test_batched_resident_matches_oracle(gb, gbo, alg, cluster):
    n, m, k, tid = pick([1024, 2048], 8)
    ns, iters, err, ok = gb.solve_batch(n, m, k, SEED, tid, alg=alg, maxiter=1000, resident_n=4096,
                                        cluster=cluster)
    ok_o, it_o, err_o = gbo.solve_dense_trials(n, m, k, SEED, tid, alg=alg, tol_rel=1e-4, maxiter=1000)
    assert np.sum((err_o <= 1e-3) == ok.astype(bool)) >= len(n) - 1
