"""Golden fixtures of the reference's own recovery loops (test infrastructure).

Runs the reference's MEX gateways gaga_gen / gaga_dct / gaga_smv -- GAGA/gaga/gaga_gen.cu,
gaga_dct.cu, gaga_smv.cu with everything they include, unmodified, compiled for the CPU by
oracle/build.py:build_ref_gateways over the host emulation in oracle/ref_shim/host -- in
their "solve given data" usage (gaga_gen.cu:115-134, gaga_dct.cu:112-127,
gaga_smv.cu:159-195) on seeded problems, and stores each call's outputs in
tests/golden/ref_loops.npz:

  dense     n = 4096, m = 1024 (the single-trial configuration), +-1 signals, k = 20, 102,
            230: every gaga_gen algorithm, CGIHT with restartFlag on and off, and the NIHT
            and HTP timing variants with supportFlag 0-3
  dct       n = 2^14, m = 2^12, Gaussian signals, k = 100, 400: every algorithm and the
            timing variants
  expander  n = 2^14, m = 2^12, d = 7: values 1/sqrt(7) with Gaussian signals (k = 60, 200)
            for every algorithm and the timing variants; unit values with +-1 signals
            (k = 204, 512) for parallel_l0, parallel_lddsr, parallel_l0_swipe, serial_l0, smp,
            ssmp, er, ssmp_naive, er_naive (with their residual records)

Each call is repeated PROBES times with every entry of y moved by one ulp up or down (seeded
signs, the size of the operator's own rounding), and the case records how far the
reference's own outputs moved at most (x_spread = relative l2 distance between the x,
iter_spread, conv_spread, and whether the verdict held): the tests widen their bars to that spread, so a
case whose trajectory is sensitive to rounding is held to what the reference itself
reproduces.

The problems come from the oracle's seeded generators (oracle/gbo.py), so a test rebuilds
A, the DCT rows and the expander pattern from the seed; y is stored.  The tolerance of the
residual test is 1e-4 ||y|| (absolute, as the gateways take it); maxiter is 5000 (300 for
HTP, 200 for the expander decoders).

Run from the repository root where the reference tree is available:
    python tests/golden/make_ref_loops.py
"""
import json
import os
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle import gbo  # noqa: E402
from oracle import ref_gateway as rg  # noqa: E402

OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "ref_loops.npz")
ALGS = ["NIHT", "HTP", "IHT", "ThresholdSD", "ThresholdCG", "CSMPSP", "CGIHT", "FIHT", "ALPS", "CGIHTprojected"]
PROBES = 3
DECODERS = ["parallel_l0", "parallel_lddsr", "parallel_l0_swipe", "serial_l0", "smp", "ssmp", "er", "ssmp_naive",
            "er_naive"]


def variants(extra_timing=True):
    out = [(a, ()) for a in ALGS] + [("CGIHT", (("restartFlag", "on"),))]
    if extra_timing:
        for a in ("NIHT", "HTP"):
            for f in range(4):
                out.append((a, (("timing", "on"), ("supportFlag", f))))
    return out


def problem(kind, n, m, k, seed, d=7, ens=1):
    vd = 1 if kind == "dense" or ens == 3 else 2
    if kind == "dense":
        op = gbo.Op.dense(gbo.gen_dense(m, n, seed=seed), m, n)
    elif kind == "dct":
        op = gbo.Op.dct(n, gbo.gen_dct_rows(n, m, seed))
    else:
        rows, vals = gbo.gen_smv(m, n, d, ens, seed)
        op = gbo.Op.smv(m, n, d, rows, vals)
    x0, ks = gbo.gen_vector(n, k, vd, seed=seed)
    return op, x0, ks, gbo.A(op, x0), vd


def run(kind, op, y, ks, alg, opts):
    n, m = op.n, op.m
    if kind == "dense":
        return rg.gaga_gen(alg, y, op.A.reshape(n, m).T, ks, opts) + (None,)
    if kind == "dct":
        return rg.gaga_dct(alg, y, op.dct_rows + 1, ks, m, n, opts) + (None,)
    cols = np.repeat(np.arange(n, dtype=np.int32), op.d)
    return rg.gaga_smv(alg, y, op.smv_rows + 1, cols + 1, op.smv_vals, ks, opts)


def main():
    cases, arrays = [], {}
    plan = []
    for k, seed in ((102, 1), (230, 2), (20, 4)):
        plan.append(("dense", 4096, 1024, k, seed, 1, variants(k == 102) if k != 20 else
                     [("NIHT", ()), ("HTP", ()), ("CGIHT", ())]))
    for k, seed in ((100, 3), (400, 6)):
        plan.append(("dct", 1 << 14, 1 << 12, k, seed, 1, variants(k == 100)))
    for k, seed in ((60, 5), (200, 9)):
        plan.append(("smv", 1 << 14, 1 << 12, k, seed, 1, variants(k == 60)))
    for k, seed in ((204, 7), (512, 8)):
        plan.append(("smv", 1 << 14, 1 << 12, k, seed, 3, [(a, ()) for a in DECODERS]))
    for kind, n, m, k, seed, ens, runs in plan:
        op, x0, ks, y, vd = problem(kind, n, m, k, seed, ens=ens)
        tol = 1e-4 * float(np.linalg.norm(y.astype(np.float64)))
        pid = "%s_n%d_m%d_k%d_s%d_e%d" % (kind, n, m, k, seed, ens)
        arrays[pid + "/y"] = y
        if kind == "dense":
            arrays[pid + "/A_sample"] = op.A[:64].copy()
            arrays[pid + "/A_sum"] = np.array([op.A.astype(np.float64).sum()])
        for alg, opts in runs:
            maxiter = 200 if alg in DECODERS else (300 if alg == "HTP" else 5000)
            o = [("tol", tol), ("maxiter", maxiter)] + list(opts)
            t = time.time()
            x, it, conv, rec = run(kind, op, y, ks, alg, o)
            err = float(np.linalg.norm(x.astype(np.float64) - x0) / np.linalg.norm(x0.astype(np.float64)))
            spread = {"x_spread": 0.0, "iter_spread": 0, "conv_spread": 0.0, "verdict_stable": True}
            for probe in range(PROBES):
                sgn = np.random.default_rng([seed, probe]).integers(0, 2, y.size).astype(bool)
                y2 = np.where(sgn, np.nextafter(y, np.float32(np.inf)), np.nextafter(y, np.float32(-np.inf)))
                x2, it2, conv2, _ = run(kind, op, y2.astype(np.float32), ks, alg, o)
                err2 = float(np.linalg.norm(x2.astype(np.float64) - x0) / np.linalg.norm(x0.astype(np.float64)))
                spread["x_spread"] = max(spread["x_spread"], float(np.linalg.norm(x2.astype(np.float64) - x) /
                                                                   max(np.linalg.norm(x.astype(np.float64)), 1e-30)))
                spread["iter_spread"] = max(spread["iter_spread"], abs(it2 - it))
                spread["conv_spread"] = max(spread["conv_spread"], abs(conv2 - conv))
                spread["verdict_stable"] &= (err <= 1e-3) == (err2 <= 1e-3)
            cid = "%s/%s%s" % (pid, alg, "".join("_%s=%s" % (a, b) for a, b in opts))
            arrays[cid + "/x"] = x
            if rec is not None:
                arrays[cid + "/rec"] = rec[: it + 1]
            cases.append({"id": cid, "problem": pid, "kind": kind, "n": n, "m": m, "k": k, "k_used": int(ks),
                          "seed": seed, "ens": ens, "vec_dist": vd, "alg": alg, "opts": [list(p) for p in opts],
                          "tol": tol, "maxiter": maxiter, "iter": it, "conv_rate": conv, "rel_err": err, **spread})
            print("%-60s it %4d err %.2e  spread x %.1e it %d conv %.3f  %.1fs" % (
                cid, it, err, spread["x_spread"], spread["iter_spread"], spread["conv_spread"], time.time() - t),
                flush=True)
    arrays["manifest"] = np.array(json.dumps(cases))
    np.savez_compressed(OUT, **arrays)
    print("wrote", OUT, os.path.getsize(OUT), "bytes,", len(cases), "cases")


if __name__ == "__main__":
    main()
