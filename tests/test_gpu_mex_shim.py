"""This library's MEX gateways (gaga_gb300/mex/gb_gaga_mex.cpp) called as MATLAB calls the
reference's: the same argument arrays and gagaOptions cell (1-based indices, typed option
values) that produced tests/golden/ref_loops.npz from the reference's own gaga_gen /
gaga_dct / gaga_smv, and the outputs checked against the reference's by the bar of
tests/ref_loops_fixture.py, with the reference's output classes (iters int32, x and
convRate single).  The gateways are built against the stand-in MATLAB API
(tests/mex_shim.py)."""
import numpy as np
import pytest

import mex_shim
import ref_loops_fixture as F

pytestmark = pytest.mark.gpu

PICK = {("dense", "NIHT"), ("dense", "HTP"), ("dense", "CGIHT"), ("dense", "CSMPSP"), ("dct", "NIHT"),
        ("dct", "CGIHT"), ("dct", "HTP"), ("smv", "NIHT"), ("smv", "CGIHT"), ("smv", "parallel_l0"), ("smv", "smp")}
CASES = [c for c in F.cases() if (c["kind"], c["alg"]) in PICK]
mxSINGLE, mxINT32 = 7, 12


@pytest.mark.parametrize("case", CASES, ids=[c["id"] for c in CASES])
def test_mex_gateway_matches_reference(gbo, case):
    from oracle import ref_gateway as rg

    op, x0, y = F.problem(gbo, case)
    opts = [("tol", case["tol"]), ("maxiter", case["maxiter"])] + [tuple(p) for p in case["opts"]]
    ks = case["k_used"]
    if case["kind"] == "dense":
        L = mex_shim.load("gen")
        args = lambda: rg.gen_args(L, case["alg"], y, op.A.reshape(op.n, op.m).T, ks, opts)  # noqa: E731
        nlhs = 3
    elif case["kind"] == "dct":
        L = mex_shim.load("dct")
        args = lambda: rg.dct_args(L, case["alg"], y, op.dct_rows + 1, ks, op.m, op.n, opts)  # noqa: E731
        nlhs = 3
    else:
        L = mex_shim.load("smv")
        cols = np.repeat(np.arange(op.n, dtype=np.int32), op.d) + 1
        args = lambda: rg.smv_args(L, case["alg"], y, op.smv_rows + 1, cols, op.smv_vals, ks, opts)  # noqa: E731
        nlhs = 5
    L.gbmx_clear_error()
    outs = rg.call(L, nlhs, args())
    assert L.gbmx_last_error() == b"", L.gbmx_last_error()
    x, it, conv = outs[0], int(outs[1][0]), float(outs[2][0])
    rec = outs[3] if case["alg"] in F.DECODERS else None
    F.check(case, x0, x, it, conv, rec, label="mex")
    classes = rg.out_classes(L, nlhs, args())
    assert classes[:3] == [mxSINGLE, mxINT32, mxSINGLE]
