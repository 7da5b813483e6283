"""Phase-transition sweep of independent dense Gaussian trials.

The grid is n in {1024, 2048, 4096, 8192, 16384}, delta = m/n in {0.1, ..., 0.9} and
rho = k/m on a 0.02 grid up to 0.5 (1125 points); a sweep of T trials cycles through the
grid with a distinct trial id (and therefore a distinct seeded A and x) per trial.  The
reference sweeps the same grid shape through gaga_cs one trial per call
(GAGA/gaga_for_CS_timings/generate_gpu_gen_timing_data.m, GAGA/CGIHTcode/shared/
tests_delta_fixed.m), with success meaning a small relative error.
"""
import numpy as np

N_VALUES = (1024, 2048, 4096, 8192, 16384)
DELTAS = tuple(round(0.1 * i, 1) for i in range(1, 10))
RHOS = tuple(round(0.02 * i, 2) for i in range(1, 26))


def grid():
    pts = [(n, d, r) for n in N_VALUES for d in DELTAS for r in RHOS]
    return pts


# Rounds of the grid after the first two visit its points in the order t * STRIDE mod 1125
# (STRIDE coprime with 1125 = 3^2 5^3), so a partial round -- 822 of the 1125 points in the
# 3072 independent trials of the sweep -- spreads over every n, delta and rho instead of
# taking the first (smallest-n) points of the grid's n-major order.
ROUND_STRIDE = 409


def grid_point(t, npts):
    """Grid index of trial t: the grid's own order in rounds 0 and 1, strided after."""
    r, q = divmod(t, npts)
    return q if r < 2 else (q * ROUND_STRIDE) % npts


def sweep_trials(total=4096):
    """Arrays (n, m, k, trial_id) of a sweep of `total` trials."""
    pts = grid()
    n = np.empty(total, np.int32)
    m = np.empty(total, np.int32)
    k = np.empty(total, np.int32)
    for t in range(total):
        nn, dd, rr = pts[grid_point(t, len(pts))]
        mm = int(round(dd * nn))
        n[t], m[t], k[t] = nn, mm, max(1, int(round(rr * mm)))
    return n, m, k, np.arange(total, dtype=np.uint32)


def wave(total, waves, w):
    """Indices of wave w when a sweep of `total` trials is split into `waves` interleaved waves."""
    return np.arange(w, total, waves)


def wave_trials(total, waves, w):
    """Arrays (n, m, k, trial_id) of wave w of a sweep of `total` trials split into `waves`
    interleaved waves.  Waves w and w + waves cover the same grid points with distinct
    trials: the trial ids of round w // waves are offset by that many sweeps, so every wave
    index names its own seeded problems (ranks beyond the wave count never repeat a trial)."""
    n, m, k, tid = sweep_trials(total)
    idx = wave(total, waves, w % waves)
    return n[idx], m[idx], k[idx], (tid[idx] + np.uint32((w // waves) * total)).astype(np.uint32)


def shard(indices, rank, world):
    """Trials of one rank: every world-th index starting at rank."""
    indices = np.asarray(indices)
    return indices[rank::world]


def rank_wave(rank, world, step):
    """Wave solved by `rank` at global step `step` (weak scaling: every rank its own wave)."""
    return rank + world * step


# The shared-matrix subset of the sweep: trials that share one dense Gaussian A with
# n = 8192 and delta = 0.5 (m = 4096), rho cycling through the sweep's 0.02 grid.
SHARED_N, SHARED_M = 8192, 4096


def shared_subset(total=1024):
    """k of each trial of a shared-matrix subset of `total` trials."""
    return np.array([max(1, int(round(RHOS[t % len(RHOS)] * SHARED_M))) for t in range(total)], dtype=np.int32)
