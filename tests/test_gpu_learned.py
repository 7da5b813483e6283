"""Learned warm start on the GPU: features, forward pass and gradient against the CPU
oracle (oracle/mlp_ref.py), training on the GPU, and warm-started CGIHT solves."""
import os

import numpy as np
import pytest

from oracle import mlp_ref

pytestmark = pytest.mark.gpu


def _t(a):
    import torch

    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.float32)).cuda()


def test_features_match_oracle(gb):
    from gaga_gb300 import learned

    rng = np.random.default_rng(11)
    g = rng.standard_normal(20000).astype(np.float32)
    g[::97] = g[0]  # ties
    f = learned.features_of(_t(g), 9000, 1234).cpu().numpy()
    np.testing.assert_array_equal(f, mlp_ref.features(g, 9000, 1234))


def test_forward_and_gradient_match_oracle(gb):
    import torch

    L = gb._lib.load()
    rng = np.random.default_rng(12)
    p = mlp_ref.init_params(7)
    F = rng.random((3000, 4)).astype(np.float32)
    t = (rng.standard_normal(3000) * 0.5).astype(np.float32)
    dp, dF, dt = _t(p), _t(F), _t(t)
    out = torch.empty(3000, device="cuda")
    gb._lib.check(L.gb_cs_mlp_forward(dp.data_ptr(), dF.data_ptr(), 3000, out.data_ptr(), None))
    torch.cuda.synchronize()
    ref = mlp_ref.forward(p, F)
    np.testing.assert_allclose(out.cpu().numpy(), ref, rtol=1e-5, atol=1e-5 * np.abs(ref).max())
    grad = torch.empty(mlp_ref.P, device="cuda")
    loss = torch.empty(1, device="cuda")
    gb._lib.check(L.gb_cs_mlp_grad(dp.data_ptr(), dF.data_ptr(), dt.data_ptr(), 3000, grad.data_ptr(),
                                   loss.data_ptr(), None))
    l_ref, g_ref = mlp_ref.loss_and_grad(p, F, t)
    assert abs(loss.item() - l_ref) <= 1e-5 * l_ref
    np.testing.assert_allclose(grad.cpu().numpy(), g_ref, rtol=0, atol=1e-4 * np.abs(g_ref).max())


def test_training_fits_a_teacher(gb):
    """The GPU training loop fits targets made by another network."""
    from gaga_gb300 import learned

    rng = np.random.default_rng(13)
    teacher = mlp_ref.init_params(99) * 0.5
    F = rng.random((20000, 4)).astype(np.float32)
    t = mlp_ref.forward(teacher, F).astype(np.float32)
    p, hist = learned.train_params(_t(F), _t(t), epochs=30, batch=512, lr=2e-3, seed=3)
    assert hist[-1] < 0.1 * hist[0], hist
    _, g = mlp_ref.loss_and_grad(p.cpu().numpy(), F, t)
    assert np.all(np.isfinite(g))


def test_warm_started_cgiht_solves(gb):
    """CGIHT from the learned warm start recovers a problem inside the recovery region."""
    import torch

    from gaga_gb300 import learned

    if not os.path.exists(learned.WEIGHTS):
        pytest.skip("trained parameters not generated yet")
    params = learned.load_weights()
    m, n, k = 2048, 8192, 300
    _, _, _, _, A, Y, X0 = gb.solve_shared_batch(m, n, [k], 4242, maxiter=0, outputs=True)
    ks = int(torch.count_nonzero(X0[0]).item())
    res = {}
    for name, lp in (("plain", None), ("learned", params)):
        opts = gb.gaga_options("tol", 1e-4, "tol_is_relative", 1, "maxiter", 5000, "learnedWarmStart", lp)
        x, r, _ = gb._solve("CGIHT", gb._lib.GB_OP_DENSE, Y[0].contiguous(), ks, m, n, opts, "gen",
                            A=A.contiguous(), lda=m)
        rel = float(torch.linalg.vector_norm(x - X0[0]) / torch.linalg.vector_norm(X0[0]))
        res[name] = (rel, r.iter, r.warm_start)
    assert res["plain"][0] <= 1e-3 and res["learned"][0] <= 1e-3, res
    assert res["plain"][2] == 0 and res["learned"][2] in (1, 2), res


def test_warm_start_gain_over_plain_cgiht(gb):
    """What the trained network gains: on fresh trials of its training distribution (n = 8192,
    delta in [0.1, 0.6], rho in [0.05, 0.45]) the warm-started batched CGIHT recovers at least
    as many trials as zero-initialised CGIHT, loses almost none of plain's recoveries, and
    needs fewer iterations on the trials both recover."""
    from gaga_gb300 import learned

    if not os.path.exists(learned.WEIGHTS):
        pytest.skip("trained parameters not generated yet")
    res = learned.evaluate(learned.load_weights(), count=256, seed=learned.EVAL_SEED + 17)
    assert res["learned"]["recovered"] >= res["plain"]["recovered"], res
    assert res["only_plain_recovers"] <= 2, res
    it = res["mean_iters_both_recovered"]
    assert it["learned"] < it["plain"], res
