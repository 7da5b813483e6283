"""Learned warm start, CPU side: the oracle's network gradient against finite differences,
the feature restatement, and the committed trained parameters."""
import os

import numpy as np
import pytest

from oracle import mlp_ref

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_oracle_gradient_matches_finite_differences():
    rng = np.random.default_rng(3)
    p = mlp_ref.init_params(5).astype(np.float64)
    F = rng.random((40, 4))
    t = rng.standard_normal(40)
    loss, g = mlp_ref.loss_and_grad(p, F, t, round_weights=False)
    idx = np.concatenate([rng.choice(mlp_ref.P, 60, replace=False), [mlp_ref.OFF_B3, mlp_ref.OFF_B1, mlp_ref.OFF_W3]])
    h = 1e-6
    for i in idx:
        e = np.zeros(mlp_ref.P)
        e[i] = h
        lp, _ = mlp_ref.loss_and_grad(p + e, F, t, round_weights=False)
        lm, _ = mlp_ref.loss_and_grad(p - e, F, t, round_weights=False)
        fd = (lp - lm) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 * max(1.0, abs(fd)), (i, fd, g[i])


def test_feature_restatement_properties():
    rng = np.random.default_rng(4)
    g = rng.standard_normal(5000).astype(np.float32)
    f = mlp_ref.features(g, 2000, 300)
    assert f.shape == (5000, 4) and f.dtype == np.float32
    assert np.isclose(f[:, 0].max(), 1.0) and f[:, 0].min() >= 0
    order = np.argsort(-np.abs(g), kind="stable")
    assert np.all(np.diff(f[order, 1]) >= 0)  # rank fraction grows as |g| falls
    assert 0 <= f[:, 1].min() and f[:, 1].max() <= 1
    assert np.all(f[:, 2] == np.float32(2000) / np.float32(5000)) and np.all(f[:, 3] == np.float32(300) / 2000)


def test_trained_weights_committed():
    """The parameters trained on the GPU (python -m gaga_gb300.learned train) are in the tree."""
    path = os.path.join(ROOT, "gaga_gb300", "data", "mlp_warmstart.npz")
    if not os.path.exists(path):
        pytest.skip("trained parameters not generated yet")
    d = np.load(path)
    p = d["params"]
    assert p.shape == (mlp_ref.P,) and np.all(np.isfinite(p))
    loss = d["epoch_loss"]
    assert loss[-1] < loss[0]
