"""Generate the golden fixtures in tests/golden from the reference's own code.

The reference (GAGA) has no golden vectors or known-answer tests.  This script runs
the reference's own source -- GAGA/gaga/kernels.cu, GAGA/gaga/expander/kernels.cu
and GAGA/gaga/expander/serial_l0.cu compiled unmodified for the CPU by
oracle/build.py (build_ref) -- on seeded inputs and stores inputs and outputs.
The orthonormal DCT fixtures come from scipy.fft (FP64), the published definition
that GAGA/Matrices/dct_gpu.cu implements through cuFFT.

Run from the repository root where the reference tree is present:
    python tests/golden/make_golden.py
"""
import ctypes as C
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
from oracle import gbo  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))


def p(a):
    return C.c_void_p(a.ctypes.data)


def binning_cases(R):
    rng = np.random.default_rng(20240101)
    cases = {}
    specs = [
        ("gauss5000", rng.standard_normal(5000), 1000, None),
        ("gauss_small_maxbin", rng.standard_normal(4096), 1000, 300),
        ("ties_and_tiny", np.concatenate([np.full(300, 0.5), np.full(200, -0.5), rng.standard_normal(800) * 1e-8,
                                          np.zeros(50), rng.uniform(-1, 1, 1000)]), 1000, None),
        ("uniform_keys", rng.uniform(0, 1, 8192), 8192, 8192),
        ("heavy_tail", rng.standard_cauchy(6000), 2000, None),
    ]
    for name, v, num_bins, max_bin in specs:
        v = v.astype(np.float32)
        if max_bin is None:
            max_bin = int(np.float32(num_bins) * (np.float32(1.0) - np.float32(0.25)))
        mx = np.float32(np.abs(v).max())
        slope = np.float32(np.float32(num_bins - 1) / mx)
        bins = np.zeros(len(v), np.int32)
        cnt = np.zeros(num_bins, np.int32)
        R.ref_linear_binning(p(v), p(bins), p(cnt), num_bins, max_bin, len(v), C.c_float(slope), C.c_float(mx))
        cases[name] = dict(v=v, num_bins=num_bins, max_bin=max_bin, slope=slope, intercept=mx, bins=bins, counters=cnt)
    return cases


def threshold_cases(R):
    rng = np.random.default_rng(7)
    n = 3000
    v = rng.standard_normal(n).astype(np.float32)
    bins = rng.integers(0, 1000, n).astype(np.int32)
    out = {}
    for k_bin in (-1, 0, 17, 500, 999):
        a = v.copy()
        R.ref_threshold(p(a), p(bins), k_bin, n)
        b = np.zeros(n, np.float32)
        src = v.copy()
        R.ref_threshold_one(p(src), p(b), p(bins), k_bin, n)
        out[k_bin] = (a, b)
    return v, bins, out


def support_evolution_cases(R):
    rng = np.random.default_rng(11)
    n = 2000
    res = []
    for t in range(6):
        prev = rng.integers(0, 100, n).astype(np.int32)
        cur = prev.copy()
        if t % 2:
            idx = rng.choice(n, 3, replace=False)
            cur[idx] = 99
        kprev, kcur = 10 + t, 10 + t
        if t == 4:
            kcur = kprev - 3
        flag = R.ref_check_support_evolution(p(cur), p(prev), kcur, kprev, n)
        res.append((cur, prev, kcur, kprev, flag))
    return res


def l0_cases(R):
    out = []
    for seed, (m, n, d, ens, vec_dist) in enumerate([(256, 1024, 7, 3, 1), (512, 2048, 5, 3, 1), (300, 900, 7, 1, 2)]):
        rows, vals = gbo.gen_smv(m, n, d, ens, seed=100 + seed)
        x0, ks = gbo.gen_vector(n, max(4, m // 20), vec_dist, seed=100 + seed)
        op = gbo.Op.smv(m, n, d, rows, vals)
        y = gbo.A(op, x0)
        for shift in range(min(d, 3)):
            res = y.copy()
            x = np.zeros(n, np.float32)
            scores = np.zeros(n, np.float32)
            upd = np.zeros(n, np.float32)
            found = R.ref_l0_scores(p(scores), p(res), p(x), p(upd), p(rows), n, d, 1, shift)
            res2 = res.copy()
            R.ref_update_residual(p(res2), p(rows), p(upd), n, d)
            out.append(dict(m=m, n=n, d=d, shift=shift, rows=rows, res=res, x_after=x, updates=upd, found=found,
                            res_after=res2))
    return out


def serial_l0_cases(R):
    out = []
    for seed, (m, n, d, kdiv) in enumerate([(512, 2048, 7, 20), (1024, 4096, 7, 10), (400, 1600, 5, 8)]):
        rows, vals = gbo.gen_smv(m, n, d, 3, seed=200 + seed)
        x0, ks = gbo.gen_vector(n, m // kdiv, 1, seed=200 + seed)
        op = gbo.Op.smv(m, n, d, rows, vals)
        y = gbo.A(op, x0)
        cols = np.repeat(np.arange(n, dtype=np.int32), d)
        maxiter = 300
        x = np.zeros(n, np.float32)
        res = y.copy()
        rec = np.zeros(maxiter + 1, np.float32)
        trec = np.zeros(maxiter + 2, np.float32)
        it = R.ref_serial_l0(p(x), p(y), p(res), p(rows), p(cols), n, m, ks, d, 1, C.c_float(1e-6), maxiter,
                             p(rec), p(trec))
        out.append(dict(m=m, n=n, d=d, k=ks, rows=rows, y=y, x0=x0, x=x, res=res, rec=rec, iter=it, maxiter=maxiter))
    return out


def dct_cases():
    import scipy.fft as sf

    rng = np.random.default_rng(3)
    out = {}
    for N in (16, 64, 1024, 4096):
        v = rng.standard_normal(N).astype(np.float32)
        out[N] = (v, sf.dct(v.astype(np.float64), type=2, norm="ortho"), sf.dct(v.astype(np.float64), type=3, norm="ortho"))
    return out


def main():
    R = gbo.ref_lib()
    if R is None:
        raise SystemExit("reference tree not found; set GAGA_REFERENCE_ROOT")
    b = binning_cases(R)
    flat = {}
    for name, c in b.items():
        for key, val in c.items():
            flat[f"{name}__{key}"] = np.asarray(val)
    np.savez_compressed(os.path.join(OUT, "linear_binning.npz"), names=np.array(list(b)), **flat)

    v, bins, th = threshold_cases(R)
    flat = {"v": v, "bins": bins, "k_bins": np.array(list(th), np.int32)}
    for kb, (a, bb) in th.items():
        flat[f"threshold_{kb}"] = a
        flat[f"threshold_one_{kb}"] = bb
    np.savez_compressed(os.path.join(OUT, "threshold.npz"), **flat)

    se = support_evolution_cases(R)
    flat = {}
    for i, (cur, prev, kc, kp, fl) in enumerate(se):
        flat.update({f"c{i}__cur": cur, f"c{i}__prev": prev, f"c{i}__kcur": np.int32(kc), f"c{i}__kprev": np.int32(kp),
                     f"c{i}__flag": np.int32(fl)})
    np.savez_compressed(os.path.join(OUT, "support_evolution.npz"), count=np.int32(len(se)), **flat)

    for fname, cases in (("l0_step.npz", l0_cases(R)), ("serial_l0.npz", serial_l0_cases(R))):
        flat = {}
        for i, c in enumerate(cases):
            for key, val in c.items():
                flat[f"c{i}__{key}"] = np.asarray(val)
        np.savez_compressed(os.path.join(OUT, fname), count=np.int32(len(cases)), **flat)

    dc = dct_cases()
    flat = {}
    for N, (v, d2, d3) in dc.items():
        flat.update({f"N{N}__x": v, f"N{N}__dct2": d2, f"N{N}__dct3": d3})
    np.savez_compressed(os.path.join(OUT, "dct_scipy.npz"), sizes=np.array(list(dc), np.int32), **flat)
    for f in sorted(os.listdir(OUT)):
        if f.endswith(".npz"):
            print(f, os.path.getsize(os.path.join(OUT, f)))


if __name__ == "__main__":
    main()
