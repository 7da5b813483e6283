"""Batched form (gb_cs_solve_batch) against the single-trial drop-in and the CPU oracle.

Every batched trial is the problem gb_cs_generate_and_solve draws with seed + trial id,
so both forms solve bit-identical inputs; their FP32 trajectories differ only in
reduction order, so success verdicts (relative l2 error <= 1e-3) must agree on almost
every trial and recovered signals must agree to 1e-4.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SEED = 777


def pick(ns, count):
    from gaga_gb300 import sweep

    n, m, k, tid = sweep.sweep_trials(4096)
    idx = np.flatnonzero(np.isin(n, ns))
    idx = idx[np.linspace(0, len(idx) - 1, count).astype(int)]
    return n[idx], m[idx], k[idx], tid[idx]


def plain(gb, n, m, k, tid, maxiter):
    opts = gb.gaga_options("tol", 1e-4, "tol_is_relative", 1, "maxiter", maxiter, "seed", int(SEED + tid))
    x, xt, r = gb.generate_and_solve("NIHT", "gen", int(k), int(m), int(n), 0, opts)
    return x, xt, r


def test_batch_matches_plain_small(gb):
    n, m, k, tid = pick([1024, 2048, 4096], 48)
    ns, iters, err, ok = gb.solve_batch(n, m, k, SEED, tid, alg="NIHT", tol_rel=1e-4, maxiter=1000)
    agree = 0
    for i in range(len(n)):
        x, xt, r = plain(gb, n[i], m[i], k[i], tid[i], 1000)
        v_plain = r.norms[1] <= 1e-3
        agree += int(v_plain == bool(ok[i]))
        if v_plain and ok[i]:
            assert err[i] < 1e-3 and r.norms[1] < 1e-3
    assert agree >= len(n) - 1, (agree, len(n))
    assert ns == int(ok.sum())
    assert 0 < ns < len(n)  # the sample straddles the phase transition


def test_batch_large_trials(gb):
    """n = 8192 and 16384 trials next to each other in one batch."""
    n, m, k, tid = pick([8192, 16384], 6)
    ns, iters, err, ok = gb.solve_batch(n, m, k, SEED, tid, alg="NIHT", tol_rel=1e-4, maxiter=800)
    for i in range(len(n)):
        x, xt, r = plain(gb, n[i], m[i], k[i], tid[i], 800)
        assert (r.norms[1] <= 1e-3) == bool(ok[i]), (i, n[i], m[i], k[i], r.norms[1], err[i])
    bytes_, ms = gb.batch_last_stats()
    assert bytes_ > 0 and ms > 0


def test_batch_matches_oracle(gb, gbo):
    n, m, k, tid = pick([1024, 2048], 8)
    ns, iters, err, ok = gb.solve_batch(n, m, k, SEED, tid, alg="NIHT", tol_rel=1e-4, maxiter=1000)
    ok_o, it_o, err_o = gbo.solve_dense_trials(n, m, k, SEED, tid, alg="NIHT", tol_rel=1e-4, maxiter=1000)
    assert np.sum((err_o <= 1e-3) == ok.astype(bool)) >= len(n) - 1


def test_batch_rejects_bad_sizes(gb):
    with pytest.raises(gb.GagaError):
        gb.solve_batch([100], [200], [5], SEED)
    with pytest.raises(gb.GagaError):
        gb.solve_batch([8], [4], [1], SEED)


def test_batch_schedule_and_autotune(gb, tmp_path, monkeypatch):
    """Explicit schedules give the same verdicts on problems away from the phase transition,
    and the autotuner returns one of its measured candidates."""
    from gaga_gb300 import autotune

    monkeypatch.setenv("GB_CS_TUNE_CACHE", str(tmp_path / "tune.json"))
    n = np.array([1024, 2048, 4096] * 8, dtype=np.int32)
    m = (n // 2).astype(np.int32)
    k = (m // 20).astype(np.int32)  # rho = 0.05: deep inside the recovery region
    tid = np.arange(len(n), dtype=np.uint32)
    ref = gb.solve_batch(n, m, k, SEED, tid, alg="NIHT", maxiter=1000)
    for slots, share, rows in ((4, 38, 0), (12, 152, 0), (8, 38, 256)):
        got = gb.solve_batch(n, m, k, SEED, tid, alg="NIHT", maxiter=1000, slots=slots, sm_share=share,
                             resident_n=-1, av_rows=rows)
        assert got[0] == ref[0] == len(n)
    res = autotune.tune_batch(n, m, k, SEED, tid, alg="NIHT", maxiter=1000, stride=2, slots=(4, 8),
                              fractions=(0.5, 1.0), clusters=(4,))
    assert (res["slots"], res["sm_share"]) in {(c["slots"], c["sm_share"]) for c in res["candidates"]}
    # 2 slot counts x 2 shares x 1 cluster size, then the 256-row A x_S tile at the best
    assert len(res["candidates"]) == 5 and not res["cached"] and res["av_rows"] in (128, 256)
    again = autotune.tune_batch(n, m, k, SEED, tid, alg="NIHT", maxiter=1000, stride=2, slots=(4, 8),
                                fractions=(0.5, 1.0), clusters=(4,))
    assert again["cached"] and again["slots"] == res["slots"]
    # CGIHT with the BF16 A^T r operand tunes the resident cluster size too, under its own key
    cg = autotune.tune_batch(n, m, k, SEED, tid, alg="CGIHT", maxiter=1000, stride=2, slots=(4,), fractions=(0.5,),
                             clusters=(4, 8), grad_format="bf16", av_rows_candidates=())
    assert {c["cluster"] for c in cg["candidates"]} == {4, 8} and cg["cluster"] in (4, 8)
    assert cg["key"] != res["key"] and not cg["cached"]


def test_batch_calls_from_two_threads(gb):
    """Two host threads calling the batched form at once (ctypes releases the GIL): the
    calls are serialised on the shared engines and each returns the single-call result."""
    import threading

    n, m, k, tid = pick([1024, 2048, 8192, 16384], 12)
    ref = gb.solve_batch(n, m, k, SEED, tid, alg="NIHT", tol_rel=1e-4, maxiter=600)
    out = [None, None]

    def work(i):
        out[i] = gb.solve_batch(n, m, k, SEED, tid, alg="NIHT", tol_rel=1e-4, maxiter=600)

    th = [threading.Thread(target=work, args=(i,)) for i in range(2)]
    for t in th:
        t.start()
    for t in th:
        t.join()
    for o in out:
        assert o is not None
        assert np.array_equal(o[1], ref[1]) and np.array_equal(o[2], ref[2]) and np.array_equal(o[3], ref[3])


@pytest.mark.parametrize("fmt", ["a24", "bf16"])
@pytest.mark.parametrize("resident_n", [0, -1])
def test_batch_compact_gradient_operand(gb, fmt, resident_n):
    """CGIHT with the A^T r operand rounded to 24 bits or to BF16 (A x, the residual and the
    stopping test on FP32 A), in the cluster-resident kernel (resident_n 0) and in the slot
    graphs (-1): recovered trials meet the same 1e-3 error bar, verdicts agree with the FP32
    operand on all but a few trials at the phase transition (24 bits: rounding at 2^-16
    leaves every verdict of this sample unchanged), and the operator bytes shrink by the
    format's share of A^T r."""
    n, m, k, tid = pick([1024, 2048, 4096], 48)
    ns0, it0, err0, ok0 = gb.solve_batch(n, m, k, SEED, tid, alg="CGIHT", tol_rel=1e-4, maxiter=1000,
                                         resident_n=resident_n)
    b0, _ = gb.batch_last_stats()
    ns1, it1, err1, ok1 = gb.solve_batch(n, m, k, SEED, tid, alg="CGIHT", tol_rel=1e-4, maxiter=1000,
                                         resident_n=resident_n, grad_format=fmt)
    b1, _ = gb.batch_last_stats()
    assert np.all(err1[ok1 == 1] <= 1e-3)
    agree = int((ok0 == ok1).sum())
    assert agree >= (len(n) if fmt == "a24" else len(n) - 3), (agree, len(n))
    assert 0 < ns1 < len(n)
    # bytes per iteration: A^T r streams 3 (2) of the FP32 operand's 4 bytes per entry
    per0, per1 = b0 / max(1, it0.sum()), b1 / max(1, it1.sum())
    assert per1 < per0 * (0.95 if fmt == "a24" else 0.85), (per0, per1)


def test_batch_compact_gradient_operand_rejected_for_htp(gb):
    from gaga_gb300 import _lib

    n, m, k, tid = pick([1024], 2)
    with pytest.raises(_lib.GagaError):
        gb.solve_batch(n, m, k, SEED, tid, alg="HTP", tol_rel=1e-4, maxiter=100, grad_format="a24")


@pytest.mark.parametrize("resident_n", [0, -1])
def test_batch_cgiht_residual_recurrence(gb, resident_n):
    """CGIHT with residual_refresh = 8: a restricted step on an unchanged support updates the
    residual as r - alpha A p.  The residual and the stopping test still converge to the
    FP32 ones (y - A x is recomputed every 8th iteration and whenever the support changes):
    recovered trials meet the 1e-3 bar, verdicts agree with the exact residual on all but
    a few transition trials, and the operator bytes per iteration drop by the skipped A x_S
    passes."""
    n, m, k, tid = pick([1024, 2048, 4096], 48)
    ns0, it0, err0, ok0 = gb.solve_batch(n, m, k, SEED, tid, alg="CGIHT", tol_rel=1e-4, maxiter=1000,
                                         resident_n=resident_n)
    b0, _ = gb.batch_last_stats()
    ns1, it1, err1, ok1 = gb.solve_batch(n, m, k, SEED, tid, alg="CGIHT", tol_rel=1e-4, maxiter=1000,
                                         resident_n=resident_n, residual_refresh=8)
    b1, _ = gb.batch_last_stats()
    assert np.all(err1[ok1 == 1] <= 1e-3)
    assert int((ok0 == ok1).sum()) >= len(n) - 2
    assert 0 < ns1 < len(n)
    assert b1 / max(1, it1.sum()) < 0.97 * b0 / max(1, it0.sum())


@pytest.mark.parametrize("resident_n", [0, -1])
def test_batch_per_trial_operand_formats(gb, resident_n):
    """Per-trial A^T r operands (grad_formats): every trial's iterations and error equal its
    result in the run where all trials use its format (trials never share reductions)."""
    n, m, k, tid = pick([1024, 2048, 4096], 24)
    fmts = np.where(np.arange(len(n)) % 3 == 0, "a24", "bf16")
    res = {}
    for f in ("a24", "bf16"):
        res[f] = gb.solve_batch(n, m, k, SEED, tid, alg="CGIHT", tol_rel=1e-4, maxiter=1000, resident_n=resident_n,
                                grad_format=f)
    ns, it, err, ok = gb.solve_batch(n, m, k, SEED, tid, alg="CGIHT", tol_rel=1e-4, maxiter=1000,
                                     resident_n=resident_n, grad_format="a24", grad_formats=fmts)
    for i, f in enumerate(fmts):
        assert it[i] == res[f][1][i] and err[i] == res[f][2][i], (i, f)


def test_batch_per_trial_operand_formats_rejected(gb):
    from gaga_gb300 import _lib

    n, m, k, tid = pick([1024], 2)
    with pytest.raises(_lib.GagaError):
        gb.solve_batch(n, m, k, SEED, tid, alg="CGIHT", tol_rel=1e-4, maxiter=100, grad_formats=["a24", "fp32"])
