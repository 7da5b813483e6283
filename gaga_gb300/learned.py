"""Learned warm start for CGIHT: training data, training and evaluation.

Training data are (features, target) rows of coordinates of dense Gaussian problems that
plain zero-initialised CGIHT solves (n = 8192, delta in [0.1, 0.6], rho in [0.05, 0.45]):
the features of coordinate i of g = A^T y (gb_cs_mlp_features) and the target
w_i = x_i / g_i of the CGIHT solution (clipped to [-2, 4]).  Only trials that CGIHT
recovers (relative l2 error <= 1e-3) contribute.  Training runs on the GPU with the
library's own kernels (gb_cs_mlp_train); the trained FP32 parameters are stored in
gaga_gb300/data/mlp_warmstart.npz.

Command line (on a GPU):  python -m gaga_gb300.learned train | evaluate
"""
import ctypes as C
import json
import os
import sys
import time

import numpy as np

from . import _lib

HERE = os.path.dirname(os.path.abspath(__file__))
WEIGHTS = os.path.join(HERE, "data", "mlp_warmstart.npz")
N = 8192
DELTA = (0.1, 0.6)
RHO = (0.05, 0.45)
TRAIN_SEED = 910000
EVAL_SEED = 7700000


def draw_sizes(count, seed, n=N):
    """(m, k) of `count` trials with delta, rho uniform in the training ranges; m a multiple of 128."""
    rng = np.random.default_rng(seed)
    d = rng.uniform(*DELTA, count)
    r = rng.uniform(*RHO, count)
    m = np.maximum(128, np.round(d * n / 128).astype(int) * 128)
    k = np.maximum(1, np.round(r * m).astype(int))
    return m, k


def num_params():
    return int(_lib.load().gb_cs_mlp_num_params())


def load_weights(path=WEIGHTS):
    """Trained parameters as a CUDA tensor."""
    import torch

    p = np.load(path)["params"].astype(np.float32)
    assert p.size == num_params()
    return torch.from_numpy(p).cuda()


def features_of(g, m, k):
    """Device features (n x 4) of g (CUDA tensor)."""
    import torch

    L = _lib.load()
    n = g.numel()
    f = torch.empty((n, 4), dtype=torch.float32, device=g.device)
    _lib.check(L.gb_cs_mlp_features(g.data_ptr(), n, int(m), int(k), f.data_ptr(), None))
    return f


def make_data(ntrials=400, per_trial=512, seed=TRAIN_SEED, n=N, log=print):
    """Features and targets from plain CGIHT solves; returns (F, t, info) on the device."""
    import torch

    import gaga_gb300 as gb

    L = _lib.load()
    m_all, k_all = draw_sizes(ntrials, seed, n)
    rng = np.random.default_rng(seed + 1)
    Fs, Ts = [], []
    used = 0
    t0 = time.time()
    for t in range(ntrials):
        m, k = int(m_all[t]), int(k_all[t])
        # one problem drawn on the device (A from seed + t, x0 from seed + t + 1), no solve
        _, _, _, _, A, Y, X0 = gb.solve_shared_batch(m, n, [k], seed + 2 * t, maxiter=0, outputs=True)
        y = Y[0].contiguous()
        x0 = X0[0]
        ks = int(torch.count_nonzero(x0).item())
        g = torch.empty(n, dtype=torch.float32, device="cuda")
        _lib.check(L.gb_cs_dense_apply_noalloc(A.data_ptr(), m, m, n, 1, y.data_ptr(), g.data_ptr(), None))
        opts = gb.gaga_options("tol", 1e-4, "tol_is_relative", 1, "maxiter", 5000)
        x, it, _ = gb.gaga_cs("CGIHT", "gen", y, A.t(), ks, opts)
        rel = float(torch.linalg.vector_norm(x - x0) / torch.linalg.vector_norm(x0))
        if rel > 1e-3:
            continue
        used += 1
        F = features_of(g, m, ks)
        w = torch.where(g.abs() > 1e-12, x / torch.where(g.abs() > 1e-12, g, torch.ones_like(g)),
                        torch.zeros_like(g)).clamp(-2.0, 4.0)
        sel = torch.from_numpy(rng.choice(n, size=per_trial, replace=False)).cuda()
        Fs.append(F[sel])
        Ts.append(w[sel])
    F = torch.cat(Fs).contiguous()
    T = torch.cat(Ts).contiguous()
    info = {"trials": ntrials, "recovered_trials_used": used, "samples": int(T.numel()), "seconds": time.time() - t0}
    log(json.dumps(info))
    return F, T, info


def _init_params(seed):
    """He-style initialisation (float32)."""
    rng = np.random.default_rng(seed)
    P, IN, H = num_params(), 4, 64
    p = np.zeros(P, dtype=np.float32)
    o_b1 = H * IN
    o_w2 = o_b1 + H
    o_b2 = o_w2 + H * H
    o_w3 = o_b2 + H
    p[0:o_b1] = rng.standard_normal(H * IN) * np.sqrt(2.0 / IN)
    p[o_w2:o_b2] = rng.standard_normal(H * H) * np.sqrt(2.0 / H)
    p[o_w3:o_w3 + H] = rng.standard_normal(H) * np.sqrt(1.0 / H)
    return p


def train_params(F, T, epochs=40, batch=1024, lr=2e-3, seed=1):
    """Adam training on the GPU (gb_cs_mlp_train); returns (params tensor, per-epoch loss)."""
    import torch

    L = _lib.load()
    p = torch.from_numpy(_init_params(seed)).cuda()
    hist = np.zeros(epochs, dtype=np.float32)
    _lib.check(L.gb_cs_mlp_train(p.data_ptr(), F.data_ptr(), T.data_ptr(), int(T.numel()), int(batch), int(epochs),
                                 float(lr), int(seed), C.c_void_p(hist.ctypes.data), None))
    return p, hist


def evaluate(params, count=2048, seed=EVAL_SEED, n=N, maxiter=5000):
    """Plain zero-initialised CGIHT against the learned warm start on `count` fresh trials,
    both through the batched form; recovery, iterations and device time of each."""
    import gaga_gb300 as gb

    m, k = draw_sizes(count, seed, n)
    nn = np.full(count, n, dtype=np.int32)
    tid = np.arange(count, dtype=np.uint32)
    out = {}
    for name, lp in (("plain", None), ("learned", params)):
        gb.solve_batch(nn[:16], m[:16], k[:16], seed, tid[:16], alg="CGIHT", maxiter=maxiter, learned_params=lp)
        ns, iters, err, ok = gb.solve_batch(nn, m, k, seed, tid, alg="CGIHT", maxiter=maxiter, learned_params=lp)
        _, ms = gb.batch_last_stats()
        out[name] = {"recovered": int(ns), "mean_iters": float(iters.mean()), "kernel_ms": ms,
                     "recovered_per_s": ns / (ms / 1e3), "ok": ok, "iters": iters}
    both = (out["plain"]["ok"] == 1) & (out["learned"]["ok"] == 1)
    agree = float(np.mean(out["plain"]["ok"] == out["learned"]["ok"]))
    res = {"trials": count, "n": n, "delta": DELTA, "rho": RHO,
           "plain": {k2: v for k2, v in out["plain"].items() if k2 not in ("ok", "iters")},
           "learned": {k2: v for k2, v in out["learned"].items() if k2 not in ("ok", "iters")},
           "verdict_agreement": agree,
           "only_plain_recovers": int(np.sum((out["plain"]["ok"] == 1) & (out["learned"]["ok"] == 0))),
           "only_learned_recovers": int(np.sum((out["plain"]["ok"] == 0) & (out["learned"]["ok"] == 1))),
           "mean_iters_both_recovered": {"plain": float(out["plain"]["iters"][both].mean()) if both.any() else None,
                                         "learned": float(out["learned"]["iters"][both].mean()) if both.any() else None},
           "speedup_recovered_per_s": out["learned"]["recovered_per_s"] / out["plain"]["recovered_per_s"]}
    return res


def main(argv):
    import torch

    cmd = argv[1] if len(argv) > 1 else "train"
    if cmd == "train":
        F, T, info = make_data()
        p, hist = train_params(F, T)
        os.makedirs(os.path.dirname(WEIGHTS), exist_ok=True)
        out = os.environ.get("GB_MLP_OUT", WEIGHTS)
        np.savez(out, params=p.cpu().numpy(), epoch_loss=hist, info=json.dumps(info))
        print(json.dumps({"saved": out, "first_loss": float(hist[0]), "last_loss": float(hist[-1])}))
    elif cmd == "evaluate":
        res = evaluate(load_weights())
        print(json.dumps(res))
    torch.cuda.synchronize()


if __name__ == "__main__":
    main(sys.argv)
