"""The oracle's loops (oracle/gbo.c) against the reference's own MEX gateways run on the
CPU (tests/golden/ref_loops.npz, made by tests/golden/make_ref_loops.py): every gaga_gen,
gaga_dct and gaga_smv algorithm, CGIHT's restartFlag, the NIHT / HTP timing variants with
supportFlag 0-3, and the expander decoders bit for bit.  The bar is in
tests/ref_loops_fixture.py."""
import pytest

import ref_loops_fixture as F

ALL = F.cases()


@pytest.mark.parametrize("case", ALL, ids=[c["id"] for c in ALL])
def test_oracle_matches_reference_loops(gbo, case):
    op, x0, y = F.problem(gbo, case)
    o = F.options(case)
    alg = case["alg"]
    if alg in ("parallel_l0", "parallel_lddsr", "parallel_l0_swipe"):
        x, _, rec, info = gbo.parallel_l0(op, y, o["tol"], o["maxiter"], variant=alg)
    elif alg == "serial_l0":
        x, _, rec, info = gbo.serial_l0(op, y, o["tol"], o["maxiter"])
    elif alg == "smp":
        x, _, rec, info = gbo.smp(op, y, case["k_used"], o["tol"], o["maxiter"])
    elif alg in F.DECODERS:
        x, _, rec, info = gbo.seq_decode(alg, op, y, case["k_used"], o["tol"], o["maxiter"])
    else:
        rec = None
        x, info = gbo.solve(alg, op, y, case["k_used"], o["tol"], maxiter=o["maxiter"],
                            restart=1 if o.get("restartFlag") == "on" else 0,
                            timing=1 if o.get("timing") == "on" else 0, supp_flag=int(o.get("supportFlag", 0)))
    F.check(case, x0, x, info.iter, info.conv_rate, rec, label="oracle")
