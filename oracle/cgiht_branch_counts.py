"""CGIHT's step kinds over sampled sweep trials, counted by the oracle (CPU).

CGIHT with restartFlag off (GAGA/gaga/algorithms.cu:3689-3942) takes an UnrestrictedCG
step (functions.cu:1107-1220) after a support change and a
RestrictedCGwithSupportEvolution step (functions.cu:1004-1102) otherwise.  This script
solves every third trial of one size class of a sweep step with the oracle and reports
how the iterations split between the two kinds and between recovered and failed trials.
Each trial is a dense Gaussian problem with the trial's (n, m, k), drawn with numpy from a
fixed seed: the split is a property of the algorithm at those sizes, not of one draw.

    python oracle/cgiht_branch_counts.py [n ...]      # default: 1024 2048
"""
import os
import sys

import numpy as np

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))

from gaga_gb300 import sweep  # noqa: E402
from oracle import gbo  # noqa: E402

STEP = 3          # the sweep step whose trials are sampled
TOTAL = 4096 - 1024
PARTS = 4


def counts(n_value, stride=3, seed=0):
    n_all, m_all, k_all, _ = sweep.wave_trials(TOTAL, PARTS, STEP)
    rng = np.random.default_rng(seed)
    out = []
    for j in np.flatnonzero(n_all == n_value)[::stride]:
        n, m, k = int(n_all[j]), int(m_all[j]), int(k_all[j])
        A = (rng.standard_normal((m, n)) / np.sqrt(m)).astype(np.float32)
        x0 = np.zeros(n, np.float32)
        x0[rng.choice(n, k, replace=False)] = rng.choice([-1.0, 1.0], k)
        y = (A @ x0).astype(np.float32)
        op = gbo.Op.dense(np.asfortranarray(A).ravel(order="F"), m, n)
        x, info = gbo.solve("CGIHT", op, y, k, 1e-4 * float(np.linalg.norm(y)), maxiter=5000)
        ok = bool(np.linalg.norm(x - x0) <= 1e-3 * np.linalg.norm(x0))
        out.append((ok, info.ucg_steps, info.rcg_steps, info.iter))
    return out


def main(argv):
    for n_value in [int(a) for a in argv] or [1024, 2048]:
        res = counts(n_value)
        u = sum(r[1] for r in res)
        r_ = sum(r[2] for r in res)
        fail = [r for r in res if not r[0]]
        print("n = %d: %d trials, %d unrestricted + %d restricted steps (%.0f%% unrestricted); "
              "failed trials: %d, with %d of the %d steps" % (n_value, len(res), u, r_, 100.0 * u / max(1, u + r_),
                                                            len(fail), sum(f[1] + f[2] for f in fail), u + r_))


if __name__ == "__main__":
    main(sys.argv[1:])
