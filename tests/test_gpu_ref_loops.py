"""The CUDA path against the reference's own MEX gateways run on the CPU
(tests/golden/ref_loops.npz, made by tests/golden/make_ref_loops.py): every gaga_gen,
gaga_dct and gaga_smv algorithm through gaga_cs's solve-given-data usage (the C ABI), CGIHT's
restartFlag, the NIHT / HTP timing variants with supportFlag 0-3, and the expander decoders
bit for bit with their residual records.  Dense NIHT, HTP and CGIHT at n = 4096 run on the
single-trial cluster kernel, the rest as per-step kernels in CUDA graphs.  The bar is in
tests/ref_loops_fixture.py."""
import numpy as np
import pytest

import ref_loops_fixture as F

pytestmark = pytest.mark.gpu

# serial_l0 is Gauss-Seidel, sequential by construction; the reference runs it on the host
# (GAGA/gaga/gaga_smv.cu:951) and this library does not offer it on the GPU (the oracle's
# restatement is pinned to the reference in tests/test_oracle_ref_loops.py)
ALL = [c for c in F.cases() if c["alg"] != "serial_l0"]


@pytest.mark.parametrize("case", ALL, ids=[c["id"] for c in ALL])
def test_gpu_matches_reference_loops(gb, gbo, case):
    op, x0, y = F.problem(gbo, case)
    o = F.options(case)
    opts = gb.gaga_options(*[v for kv in o.items() for v in kv])
    alg, ks = case["alg"], case["k_used"]
    rec = None
    if case["kind"] == "dense":
        x, it, conv = gb.gaga_cs(alg, "gen", y, op.A.reshape(op.n, op.m).T.copy(), ks, opts)
    elif case["kind"] == "dct":
        x, it, conv = gb.gaga_cs(alg, "dct", y, op.dct_rows, ks, op.m, op.n, opts, index_base=0)
    else:
        cols = np.repeat(np.arange(op.n, dtype=np.int32), op.d)
        x, it, conv, rec, _ = gb.gaga_cs(alg, "smv", y, op.smv_rows, cols, op.smv_vals, ks, opts, index_base=0)
        if alg not in F.DECODERS:
            rec = None
    F.check(case, x0, np.asarray(x), int(it), float(conv), None if rec is None else np.asarray(rec), label="gpu")
