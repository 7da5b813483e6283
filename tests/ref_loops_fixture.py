"""Reads tests/golden/ref_loops.npz -- outputs of the reference's own MEX gateways
(GAGA/gaga/gaga_{gen,dct,smv}.cu, compiled for the CPU; tests/golden/make_ref_loops.py) --
rebuilds each case's problem from its seed with the oracle's generators, and checks a
solver's outputs against the reference's.

The bar (one place, used by the oracle's and the GPU path's tests):
  * every case: the same verdict (relative l2 error to the planted signal <= 1e-3);
  * the expander decoders (integer scores on unit values, +-1 signals): x, the iteration
    count and the residual record bit for bit;
  * the other algorithms on cases the reference recovers: relative l2 distance to the
    reference's x <= 1e-4, the same support (entries above 1e-4 max|x|), iterations within
    +-2 and the convergence rate within 0.02.  Failing cases are compared by verdict only:
    their trajectories are chaotic (a 1-ulp change of one entry of y moves the reference's
    failing HTP run at k = 230 between 8 and 15 iterations).
  * Each case also records how far the reference's own outputs move when every entry of y
    moves by one ulp, up or down (x_spread, iter_spread, conv_spread, verdict_stable): noise
    of the size of the operators' own rounding, in which the reference's FP32 operators and
    any other implementation differ.  The bars widen
    to that measured spread -- x to 4 x_spread, iterations to 2 iter_spread, the rate to
    2 conv_spread -- and a verdict the reference itself does not hold under the nudge is not
    compared.  (Example: at n = 4096, k = 102 HTP's x moves by 1e-4 under the nudge.)
"""
import json
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PATH = os.path.join(HERE, "golden", "ref_loops.npz")
DECODERS = {"parallel_l0", "parallel_lddsr", "parallel_l0_swipe", "serial_l0", "smp", "ssmp", "er", "ssmp_naive",
            "er_naive"}
REL_X_TOL = 1e-4
VERDICT_TOL = 1e-3

_data = None


def data():
    global _data
    if _data is None:
        z = np.load(PATH)
        _data = ({k: z[k] for k in z.files if k != "manifest"}, json.loads(str(z["manifest"])))
    return _data


def cases(kind=None, decoders=None):
    arrays, manifest = data()
    out = []
    for c in manifest:
        if kind and c["kind"] != kind:
            continue
        if decoders is not None and (c["alg"] in DECODERS) != decoders:
            continue
        out.append(c)
    return out


_problems = {}


def problem(gbo, case):
    """(op, x0, y) of a case, rebuilt from its seed (y as stored)."""
    pid = case["problem"]
    if pid not in _problems:
        arrays, _ = data()
        n, m, k, seed, ens = case["n"], case["m"], case["k"], case["seed"], case["ens"]
        if case["kind"] == "dense":
            A = gbo.gen_dense(m, n, seed=seed)
            np.testing.assert_allclose(A[:64], arrays[pid + "/A_sample"], rtol=1e-6)
            np.testing.assert_allclose(A.astype(np.float64).sum(), arrays[pid + "/A_sum"][0], rtol=1e-7)
            op = gbo.Op.dense(A, m, n)
        elif case["kind"] == "dct":
            op = gbo.Op.dct(n, gbo.gen_dct_rows(n, m, seed))
        else:
            rows, vals = gbo.gen_smv(m, n, 7, ens, seed)
            op = gbo.Op.smv(m, n, 7, rows, vals)
        x0, ks = gbo.gen_vector(n, k, case["vec_dist"], seed=seed)
        assert ks == case["k_used"]
        _problems[pid] = (op, x0, arrays[pid + "/y"])
    return _problems[pid]


def options(case):
    """The case's options as a dict of gagaOptions names."""
    o = {"tol": case["tol"], "maxiter": case["maxiter"]}
    for name, val in case["opts"]:
        o[name] = val
    return o


def rel(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30))


def support(x):
    x = np.abs(np.asarray(x, np.float64))
    mx = x.max() if x.size else 0.0
    return set(np.flatnonzero(x > 1e-4 * mx)) if mx > 0 else set()


def check(case, x0, x, iters, conv=None, rec=None, label=""):
    arrays, _ = data()
    ref_x = arrays[case["id"] + "/x"]
    where = "%s %s" % (label, case["id"])
    ref_ok = case["rel_err"] <= VERDICT_TOL
    ok = rel(x, x0) <= VERDICT_TOL
    if case["verdict_stable"] or case["alg"] in DECODERS:
        assert ok == ref_ok, "%s: verdict %s, the reference's %s (err %.3g vs %.3g)" % (where, ok, ref_ok,
                                                                                      rel(x, x0), case["rel_err"])
    if case["alg"] in DECODERS:
        assert np.array_equal(np.asarray(x, np.float32), ref_x), "%s: x differs from the reference's" % where
        assert iters == case["iter"], "%s: %d iterations, the reference %d" % (where, iters, case["iter"])
        if rec is not None:
            ref_rec = arrays[case["id"] + "/rec"]
            assert np.array_equal(np.asarray(rec[: len(ref_rec)], np.float32), ref_rec), \
                "%s: residual record differs" % where
        return
    if not (ref_ok and ok):
        return
    d = rel(x, ref_x)
    x_tol = max(REL_X_TOL, 4.0 * case["x_spread"])
    assert d <= x_tol, "%s: rel l2 distance to the reference's x %.3g (bar %.3g)" % (where, d, x_tol)
    assert support(x) == support(ref_x), "%s: support differs from the reference's" % where
    it_tol = max(2, 2 * case["iter_spread"])
    assert abs(iters - case["iter"]) <= it_tol, "%s: %d iterations, the reference %d" % (where, iters, case["iter"])
    if conv is not None:
        c_tol = max(0.02, 2.0 * case["conv_spread"])
        assert abs(conv - case["conv_rate"]) <= c_tol, "%s: convRate %.4f, the reference %.4f" % (
            where, conv, case["conv_rate"])
