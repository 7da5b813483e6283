"""Defined statuses at the C ABI boundary (include/gb_cs.h): the pass watchdog of the
device-side loops (GB_WATCHDOG) and non-finite data (GB_BAD_ARG), on the single-trial
cluster kernel (dense), the per-step graph path (DCT, expander) and the expander decoders.
Every case ends by a bound the host sets or by the stopping rules; nothing here faults or
spins on the GPU, and a normal solve after each failure checks that the context is usable.
The reference has neither check: its host loop ends on a NaN residual through the
comparisons of its stopping rules (GAGA/gaga/algorithms.cu:1365) and returns normally."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _dense(gbo, n=4096, m=1024, k=102, seed=3):
    A = gbo.gen_dense(m, n, seed)
    x0, ks = gbo.gen_vector(n, k, 1, seed)
    op = gbo.Op.dense(A, m, n)
    return op, A.reshape(n, m).T.copy(), x0, ks, gbo.A(op, x0)


def _dct(gbo, n=1 << 14, m=1 << 12, k=100, seed=4):
    rows = gbo.gen_dct_rows(n, m, seed)
    x0, ks = gbo.gen_vector(n, k, 2, seed)
    op = gbo.Op.dct(n, rows)
    return op, rows, x0, ks, gbo.A(op, x0)


def _smv(gbo, n=1 << 14, m=1 << 12, k=60, seed=5, ens=1):
    rows, vals = gbo.gen_smv(m, n, 7, ens, seed)
    x0, ks = gbo.gen_vector(n, k, 1 if ens == 3 else 2, seed)
    op = gbo.Op.smv(m, n, 7, rows, vals)
    return op, rows, vals, x0, ks, gbo.A(op, x0)


def _status(gb, fn):
    try:
        fn()
    except gb.GagaError as e:
        return e.status, str(e)
    return gb._lib.GB_OK, ""


def _solve(gb, gbo, kind, alg, y=None, A=None, **opt):
    if kind == "gen":
        op, Am, x0, ks, y0 = _dense(gbo)
        y = y0 if y is None else y
        Am = Am if A is None else A
        tol = 1e-4 * float(np.linalg.norm(y0))
        opts = gb.gaga_options("tol", tol, *[v for kv in opt.items() for v in kv])
        return lambda: gb.gaga_cs(alg, "gen", y, Am, ks, opts)
    if kind == "dct":
        op, rows, x0, ks, y0 = _dct(gbo)
        y = y0 if y is None else y
        opts = gb.gaga_options("tol", 1e-4 * float(np.linalg.norm(y0)), *[v for kv in opt.items() for v in kv])
        return lambda: gb.gaga_cs(alg, "dct", y, rows, ks, op.m, op.n, opts, index_base=0)
    ens = 3 if alg == "parallel_l0" else 1
    # parallel_l0 at k = 204 takes 7 iterations (at k = 60, 2)
    op, rows, vals, x0, ks, y0 = _smv(gbo, k=204, seed=7, ens=3) if ens == 3 else _smv(gbo)
    y = y0 if y is None else y
    cols = np.repeat(np.arange(op.n, dtype=np.int32), 7)
    opts = gb.gaga_options("tol", 1e-6 if ens == 3 else 1e-4 * float(np.linalg.norm(y0)),
                           *[v for kv in opt.items() for v in kv])
    return lambda: gb.gaga_cs(alg, "smv", y, rows, cols, vals, ks, opts, index_base=0)


@pytest.mark.parametrize("kind,alg", [("gen", "NIHT"), ("gen", "CGIHT"), ("gen", "HTP"), ("dct", "NIHT"),
                                      ("dct", "CGIHT"), ("smv", "NIHT"), ("smv", "parallel_l0")])
def test_pass_watchdog_returns_status(gb, gbo, kind, alg):
    """watchdog_passes bounds the passes of the device-side loop: a solve that needs more
    stops with GB_WATCHDOG; the same solve without the bound then completes."""
    st, msg = _status(gb, _solve(gb, gbo, kind, alg, watchdogPasses=1))
    assert st == gb._lib.GB_WATCHDOG, (st, msg)
    assert "iteration bound" in msg
    st, msg = _status(gb, _solve(gb, gbo, kind, alg))
    assert st == gb._lib.GB_OK, msg


@pytest.mark.parametrize("kind", ["gen", "dct", "smv"])
@pytest.mark.parametrize("bad", [np.nan, np.inf])
def test_non_finite_host_y(gb, gbo, kind, bad):
    """NaN or Inf in a host y: GB_BAD_ARG before any device work."""
    y = {"gen": _dense, "dct": _dct, "smv": _smv}[kind](gbo)[-1].copy()
    y[7] = bad
    alg = "NIHT"
    st, msg = _status(gb, _solve(gb, gbo, kind, alg, y=y))
    assert st == gb._lib.GB_BAD_ARG and "non-finite" in msg, (st, msg)


def test_non_finite_device_y(gb, gbo):
    """NaN in a device y: the solve runs to its stopping rules (a NaN residual ends the loop
    at once) and returns GB_BAD_ARG; the next solve is unaffected."""
    torch = pytest.importorskip("torch")
    op, Am, x0, ks, y0 = _dense(gbo)
    y = y0.copy()
    y[11] = np.nan
    dy, dA = torch.tensor(y, device="cuda"), torch.tensor(np.asfortranarray(Am).ravel(order="F"), device="cuda")
    dx = torch.zeros(op.n, device="cuda")
    p = gb._lib.Problem(gb._lib.GB_OP_DENSE, op.m, op.n, ks, dy.data_ptr(), dA.data_ptr(), op.m, None, None, None,
                        0, 0, gb._lib.GB_DEVICE, None)
    L = gb._lib.load()
    o = gb._lib.Options()
    L.gb_cs_default_options(o, b"NIHT", op.n)
    o.tol = 1e-4 * float(np.linalg.norm(y0))
    import ctypes as C
    r = gb._lib.Result()
    assert L.gb_cs_solve(b"NIHT", C.byref(p), C.byref(o), dx.data_ptr(), C.byref(r)) == gb._lib.GB_BAD_ARG
    assert b"non-finite" in L.gb_cs_last_error()
    st, msg = _status(gb, _solve(gb, gbo, "gen", "NIHT"))
    assert st == gb._lib.GB_OK, msg


def test_non_finite_A(gb, gbo):
    """NaN in a column of A that the support picks up: the residual turns non-finite, the
    loop ends by its stopping rules and the call returns GB_BAD_ARG."""
    op, Am, x0, ks, y0 = _dense(gbo)
    j = int(np.flatnonzero(x0)[0])
    Am = Am.copy()
    Am[:, j] = np.nan
    st, msg = _status(gb, _solve(gb, gbo, "gen", "NIHT", A=Am))
    assert st == gb._lib.GB_BAD_ARG and "non-finite" in msg, (st, msg)
