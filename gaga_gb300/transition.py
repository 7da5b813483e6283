"""The phase transition of CGIHT on dense Gaussian problems, and the batched form's
transition-aware A^T r operand.

Rounding the operand of A^T r to BF16 (2^-9 relative per entry) leaves y = A x a fixed
point but moves CGIHT's trajectory; a trial's verdict (relative l2 error <= 1e-3) can then
change only where the outcome is sensitive, i.e. near the phase transition rho*(delta),
where about half of the trials recover.  Away from it the verdict does not depend on that
rounding.  `operand_formats` therefore gives each trial the 24-bit operand (2^-16, which
left every verdict unchanged in the oracle's runs) when rho = k/m lies within the band of
rho*(delta), and the BF16 operand elsewhere.  The transition sharpens as n grows (its width
shrinks like a power of 1/n), so the band does too: band0 (1024 / n)^0.3, 0.08 at
n = 1024 and 0.035 at n = 16384 -- wider at every n than the farthest BF16 verdict change
seen (0.06, 0.02, 0.04, 0.00, 0.00 from rho* at n = 1024 ... 16384 over 3072 sweep trials).

RHO_STAR is measured by `calibrate` (plain FP32 CGIHT from the zero start, batched form,
tolerance 1e-4 ||y||, on sweep trials whose ids are disjoint from the benchmark's): for
each delta, the smallest rho of the 0.02 grid where fewer than half of the trials recover.
"""
import numpy as np

from . import sweep

# rho*(delta): GB300, 3072 calibration trials (sweep waves 40-43, n = 1024 ... 16384)
RHO_STAR = {0.1: 0.18, 0.2: 0.22, 0.3: 0.26, 0.4: 0.28, 0.5: 0.32, 0.6: 0.34, 0.7: 0.40, 0.8: 0.44, 0.9: 0.48}

CALIBRATION_WAVES = (40, 41, 42, 43)


def rho_star(delta):
    """rho*(delta) interpolated linearly in delta between the measured points."""
    ds = np.array(sorted(RHO_STAR))
    rs = np.array([RHO_STAR[d] for d in ds])
    return np.interp(np.asarray(delta, dtype=np.float64), ds, rs)


BAND0, BAND_EXP = 0.08, 0.3


def band(n, band0=BAND0, exp=BAND_EXP):
    """Half-width of the transition band at size n: band0 (1024 / n)^exp."""
    return band0 * (1024.0 / np.asarray(n, dtype=np.float64)) ** exp


def operand_formats(n, m, k, band0=BAND0, exp=BAND_EXP):
    """Per trial: "a24" when |k/m - rho*(m/n)| <= band(n), else "bf16"."""
    n, m, k = (np.asarray(a, dtype=np.float64) for a in (n, m, k))
    near = np.abs(k / m - rho_star(m / n)) <= band(n, band0, exp) + 1e-9  # the band's edge is near
    return np.where(near, "a24", "bf16")


def rho_star_from_verdicts(n, m, k, ok):
    """The table's rule applied to verdicts: per delta (m/n rounded to 0.1), the smallest
    rho of the 0.02 grid where fewer than half of the trials recover."""
    n, m, k, ok = (np.asarray(a) for a in (n, m, k, ok))
    delta = np.round(m / n, 1)
    rho = k / m
    out = {}
    for d in sorted(set(delta.tolist())):
        sel = delta == d
        star = 0.5
        for g in np.round(np.arange(0.0, 0.52, 0.02), 2):
            b = sel & (rho >= g) & (rho < g + 0.02)
            if b.any() and ok[b].mean() < 0.5:
                star = float(g)
                break
        out[float(d)] = star
    return out


def calibrate(seed, tol_rel=1e-4, maxiter=5000, waves=CALIBRATION_WAVES, total=3072, parts=4):
    """Measure RHO_STAR on the GPU: plain FP32 CGIHT (batched form, zero start) on the sweep
    waves `waves` (trial ids disjoint from waves 0-39)."""
    import gaga_gb300 as gb

    arrs = [sweep.wave_trials(total, parts, w) for w in waves]
    n, m, k, tid = (np.concatenate([a[i] for a in arrs]) for i in range(4))
    _, _, _, ok = gb.solve_batch(n, m, k, seed, tid, alg="CGIHT", tol_rel=tol_rel, maxiter=maxiter)
    return rho_star_from_verdicts(n, m, k, ok)


def check_band(seed, tol_rel=1e-4, maxiter=5000, waves=CALIBRATION_WAVES, total=3072, parts=4, residual_refresh=8):
    """Verdicts of batched CGIHT with the BF16 operand against the FP32 operand on the sweep
    waves `waves`: (trials, verdict changes, changes outside the band)."""
    import gaga_gb300 as gb

    arrs = [sweep.wave_trials(total, parts, w) for w in waves]
    n, m, k, tid = (np.concatenate([a[i] for a in arrs]) for i in range(4))
    _, _, _, ok32 = gb.solve_batch(n, m, k, seed, tid, alg="CGIHT", tol_rel=tol_rel, maxiter=maxiter)
    _, _, _, ok16 = gb.solve_batch(n, m, k, seed, tid, alg="CGIHT", tol_rel=tol_rel, maxiter=maxiter,
                                   grad_format="bf16", residual_refresh=residual_refresh)
    flip = ok32 != ok16
    outside = operand_formats(n, m, k) == "bf16"
    return int(len(n)), int(flip.sum()), int((flip & outside).sum())
