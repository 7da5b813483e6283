"""Shared-matrix batched form (gb_cs_solve_shared_batch) and its BF16 GEMM.

The GEMM is checked against an FP64 product of the same BF16-rounded operands.  The
shared-matrix solve draws its A and signals on the device; the test reads them back and
checks them against the oracle's generators, then solves every trial again with the
single-trial FP32 drop-in (gb_cs_solve on the same A and y) and compares verdicts
(relative l2 error <= 1e-3).  The BF16 operator changes the iterates, not the problem,
so verdicts agree except at the edge of the phase transition.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SEED = 4242


def _bf16_round(a):
    """Round-to-nearest-even FP32 -> BF16 -> FP32 in numpy."""
    u = np.ascontiguousarray(a, dtype=np.float32).view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) >> 16 << 16
    return u.astype(np.uint32).view(np.float32)


@pytest.mark.parametrize("M,N,K", [(128, 128, 32), (256, 384, 160), (512, 128, 1024)])
def test_gemm_bf16_tn(gb, M, N, K):
    import torch

    rng = np.random.default_rng(M + N + K)
    A = _bf16_round(rng.standard_normal((M, K)).astype(np.float32))
    B = _bf16_round(rng.standard_normal((N, K)).astype(np.float32))
    Y = rng.standard_normal((N, M)).astype(np.float32)
    dA = torch.from_numpy(A).to(torch.bfloat16).cuda()
    dB = torch.from_numpy(B).to(torch.bfloat16).cuda()
    assert np.array_equal(dA.float().cpu().numpy(), A)
    ref = (A.astype(np.float64) @ B.astype(np.float64).T).T  # (N, M)
    Ct, _ = gb.gemm_bf16_tn(dA, dB)
    torch.cuda.synchronize()
    got = Ct.cpu().numpy()
    # FP32 accumulation of K products: |error| <= ~K * eps32 * sum|a b|
    bound = K * 2.0 ** -23 * (np.abs(A).astype(np.float64) @ np.abs(B).astype(np.float64).T).T
    assert np.all(np.abs(got - ref) <= bound + 1e-6)
    Ct2, Cb = gb.gemm_bf16_tn(dA, dB, Y=torch.from_numpy(Y).cuda(), want_bf16=True)
    torch.cuda.synchronize()
    got2 = Ct2.cpu().numpy()
    assert np.all(np.abs(got2 - (Y - ref)) <= bound + 1e-5)
    assert np.array_equal(Cb.float().cpu().numpy(), _bf16_round(got2))


@pytest.mark.parametrize("M,N,K", [(128, 256, 64), (384, 512, 1024), (1024, 256, 24576), (256, 256, 64),
                                   (512, 768, 448), (768, 512, 960), (2048, 1024, 4096)])
def test_gemm_tcgen05(gb, M, N, K):
    """N % 256 == 0 and K % 64 == 0 run the tcgen05 + TMA kernel (the CTA-pair instance when
    M % 256 == 0; fewer, exactly as many and more k-blocks than ring stages): check it against an
    FP64 product of the same BF16 operands, against the single-CTA instance (GB_CS_GEMM_PAIR=0)
    and against the mma.sync kernel (GB_CS_GEMM=mma)."""
    import os

    import torch

    rng = np.random.default_rng(M * 7 + N + K)
    A = _bf16_round(rng.standard_normal((M, K)).astype(np.float32))
    B = _bf16_round(rng.standard_normal((N, K)).astype(np.float32))
    Y = rng.standard_normal((N, M)).astype(np.float32)
    dA = torch.from_numpy(A).to(torch.bfloat16).cuda()
    dB = torch.from_numpy(B).to(torch.bfloat16).cuda()
    dY = torch.from_numpy(Y).cuda()
    ref = (A.astype(np.float64) @ B.astype(np.float64).T).T
    bound = K * 2.0 ** -23 * (np.abs(A).astype(np.float64) @ np.abs(B).astype(np.float64).T).T + 1e-5
    Ct, Cb = gb.gemm_bf16_tn(dA, dB, Y=dY, want_bf16=True)
    torch.cuda.synchronize()
    got = Ct.cpu().numpy()
    assert np.all(np.abs(got - (Y - ref)) <= bound), float(np.max(np.abs(got - (Y - ref)) - bound))
    assert np.array_equal(Cb.float().cpu().numpy(), _bf16_round(got))
    os.environ["GB_CS_GEMM"] = "mma"
    try:
        Ct2, _ = gb.gemm_bf16_tn(dA, dB, Y=dY)
        torch.cuda.synchronize()
    finally:
        del os.environ["GB_CS_GEMM"]
    assert np.all(np.abs(got - Ct2.cpu().numpy()) <= 2 * bound)
    os.environ["GB_CS_GEMM_PAIR"] = "0"
    try:
        Ct3, _ = gb.gemm_bf16_tn(dA, dB, Y=dY)
        torch.cuda.synchronize()
    finally:
        del os.environ["GB_CS_GEMM_PAIR"]
    assert np.all(np.abs(got - Ct3.cpu().numpy()) <= 2 * bound)


def test_gemm_rejects_bad_shapes(gb):
    import torch

    a = torch.zeros((100, 64), dtype=torch.bfloat16, device="cuda")
    b = torch.zeros((128, 64), dtype=torch.bfloat16, device="cuda")
    with pytest.raises(gb.GagaError):
        gb.gemm_bf16_tn(a, b)


def _shared_case(gb, gbo, m, n, ks, maxiter):
    import torch

    ns, iters, err, ok, A, Y, X0 = gb.solve_shared_batch(m, n, ks, SEED, tol_rel=1e-4, maxiter=maxiter,
                                                          outputs=True)
    torch.cuda.synchronize()
    # the generated problem is the oracle's: A from SEED (trial 0), x0_t from SEED + 1 + t
    A_o = gbo.gen_dense(m, n, SEED, 0, 1).reshape(n, m)
    np.testing.assert_allclose(A.cpu().numpy(), A_o, rtol=1e-5, atol=1e-6)
    X0h = X0.cpu().numpy()
    for t in (0, len(ks) // 2, len(ks) - 1):
        x_o, _ = gbo.gen_vector(n, int(ks[t]), 1, SEED + 1 + t, 0)
        assert np.array_equal(X0h[t], x_o), t
    return ns, iters, err, ok, A, Y, X0h


def test_shared_batch_matches_plain(gb, gbo):
    import torch

    m, n = 512, 1024
    ks = np.round(np.linspace(0.04, 0.42, 96) * m).astype(np.int32)
    ns, iters, err, ok, A, Y, X0 = _shared_case(gb, gbo, m, n, ks, 1000)
    assert ns == int(ok.sum())
    agree = 0
    for t in range(len(ks)):
        k_t = int(np.count_nonzero(X0[t]))
        opts = gb.gaga_options("tol", 1e-4, "tol_is_relative", 1, "maxiter", 1000)
        x, it, _ = gb.gaga_cs("NIHT", "gen", Y[t].contiguous(), A.t(), k_t, opts)
        x = x.cpu().numpy()
        rel = np.linalg.norm(x - X0[t]) / np.linalg.norm(X0[t])
        agree += int((rel <= 1e-3) == bool(ok[t]))
        if ok[t]:
            assert err[t] <= 1e-3
    assert 0 < ns < len(ks)  # the sample straddles the phase transition
    assert agree >= len(ks) - 1, (agree, len(ks))


def test_shared_batch_debias_accuracy(gb, gbo):
    """Trials well inside the recovery region come back exact to FP32 level after debias."""
    m, n = 1024, 2048
    ks = np.full(40, 60, dtype=np.int32)
    ns, iters, err, ok, A, Y, X0 = _shared_case(gb, gbo, m, n, ks, 500)
    assert ns == len(ks)
    assert float(np.max(err)) < 1e-5
    fl, ms = gb.shared_last_stats()
    assert fl > 0 and ms > 0


def test_shared_batch_rejects_bad_sizes(gb):
    with pytest.raises(gb.GagaError):
        gb.solve_shared_batch(500, 1024, [10], SEED)
    with pytest.raises(gb.GagaError):
        gb.solve_shared_batch(1024, 512, [10], SEED)
    with pytest.raises(gb.GagaError):
        gb.solve_shared_batch(512, 1024, [0], SEED)


def test_shared_batch_debias_matches_fp64_least_squares(gb, gbo):
    """The debias is conjugate gradients on the normal equations restricted to the final
    support, with split-BF16 GEMM products and FP64 scalars -- a deliberate stand-in for an
    FP64 least-squares solve on that support (FP64 arithmetic runs at a small fraction of the
    FP32 rate on this part).  Against numpy's FP64 lstsq on the same support, A and y, the
    debiased x agrees to 1e-5 relative (the CG stops at 1e-12 of its starting gradient)."""
    import torch

    m, n = 1024, 2048
    ks = np.array([40, 80, 120, 160, 200] * 2, dtype=np.int32)
    ns, iters, err, ok, A, Y, X0, X = gb.solve_shared_batch(m, n, ks, SEED + 9, tol_rel=1e-4, maxiter=1000,
                                                             outputs="x")
    torch.cuda.synchronize()
    A64 = A.cpu().numpy().astype(np.float64).T  # m x n
    Yh, Xh = Y.cpu().numpy().astype(np.float64), X.cpu().numpy().astype(np.float64)
    checked = 0
    for t in range(len(ks)):
        if not ok[t]:
            continue
        S = np.flatnonzero(Xh[t])
        z, *_ = np.linalg.lstsq(A64[:, S], Yh[t], rcond=None)
        assert np.linalg.norm(Xh[t][S] - z) <= 1e-5 * np.linalg.norm(z), t
        checked += 1
    assert checked >= 6


def _shared_cgiht_vs_plain(gb, gbo, ks, learned=None):
    import torch

    m, n = 512, 1024
    ns, iters, err, ok, A, Y, X0 = gb.solve_shared_batch(m, n, ks, SEED + 3, tol_rel=1e-4, maxiter=1000,
                                                          outputs=True, alg="CGIHT", learned_params=learned)
    torch.cuda.synchronize()
    X0 = X0.cpu().numpy()
    assert ns == int(ok.sum())
    res = []
    for t in range(len(ks)):
        k_t = int(np.count_nonzero(X0[t]))
        opts = gb.gaga_options("tol", 1e-4, "tol_is_relative", 1, "maxiter", 1000)
        x, it, _ = gb.gaga_cs("CGIHT", "gen", Y[t].contiguous(), A.t(), k_t, opts)
        x = x.cpu().numpy()
        rel = np.linalg.norm(x - X0[t]) / np.linalg.norm(X0[t])
        res.append((bool(rel <= 1e-3), bool(ok[t]), int(it), int(iters[t])))
    return ns, res


def test_shared_cgiht_matches_plain(gb, gbo):
    """CGIHT in lockstep with BF16 tensor-core products (restricted and unrestricted CG
    branches, support evolution) against the FP32 single-trial CGIHT on the same A and y:
    the same verdicts except at the edge of the phase transition, and iteration counts close
    on the trials both recover."""
    ks = np.round(np.linspace(0.04, 0.5, 96) * 512).astype(np.int32)
    ns, res = _shared_cgiht_vs_plain(gb, gbo, ks)
    agree = sum(int(p == s) for p, s, _, _ in res)
    assert 0 < ns < len(ks)
    assert agree >= len(ks) - 2, agree
    both = [(ip, isb) for p, s, ip, isb in res if p and s]
    assert len(both) > 20
    assert np.median([abs(a - b) for a, b in both]) <= 2


def test_shared_cgiht_two_column_blocks(gb, gbo):
    """200 trials: the direction products of the restricted and unrestricted trials (up to
    400 columns) span two 256-column blocks of the joined GEMM, each split as a one-block call
    would be; verdicts against the FP32 single-trial CGIHT as above."""
    ks = np.round(np.linspace(0.04, 0.5, 200) * 512).astype(np.int32)
    ns, res = _shared_cgiht_vs_plain(gb, gbo, ks)
    agree = sum(int(p == s) for p, s, _, _ in res)
    assert 0 < ns < len(ks)
    assert agree >= len(ks) - 4, agree
    both = [(ip, isb) for p, s, ip, isb in res if p and s]
    assert len(both) > 40
    assert np.median([abs(a - b) for a, b in both]) <= 2


def test_shared_cgiht_learned_warm_start(gb, gbo):
    """The learned warm start in the shared-matrix form: the trained network's start, the
    fallback to the plain start after 10 iterations without progress (counted), verdicts
    against the plain FP32 CGIHT, and fewer iterations on the trials both recover."""
    from gaga_gb300 import learned

    params = learned.load_weights()
    ks = np.round(np.linspace(0.05, 0.45, 96) * 512).astype(np.int32)
    ns, res = _shared_cgiht_vs_plain(gb, gbo, ks, learned=params)
    fb = gb.shared_last_fallbacks()
    assert 0 <= fb <= len(ks)
    # the warm start changes which trials near the phase transition recover; it may gain
    # trials over plain CGIHT but should lose almost none
    only_plain = sum(int(p and not s) for p, s, _, _ in res)
    only_learned = sum(int(s and not p) for p, s, _, _ in res)
    assert only_plain <= 2, (only_plain, only_learned, fb)
    both = [(ip, isb) for p, s, ip, isb in res if p and s]
    assert np.mean([b for _, b in both]) <= np.mean([a for a, _ in both]) + 1.0, (only_plain, only_learned, fb)
