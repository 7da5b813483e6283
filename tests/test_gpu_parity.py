"""GPU parity: the CUDA path (through the C ABI) against the oracle and the golden
fixtures made from the reference's own code.

Tolerances: support selection, binning, k-th bin and l0 decoding are integer work and
must match bit for bit.  Recovered x (FP32) must match the oracle's within a relative
l2 distance of 1e-4 when both converge, and recover the planted signal to 1e-3.
"""
import ctypes as C
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
REL_X_TOL = 1e-4


def _torch():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def dense_problem(gbo, n, m, k, seed, vec_dist=1):
    A = gbo.gen_dense(m, n, seed=seed)
    x0, ks = gbo.gen_vector(n, k, vec_dist, seed=seed)
    op = gbo.Op.dense(A, m, n)
    y = gbo.A(op, x0)
    return A, x0, ks, op, y


@pytest.mark.parametrize("alg", ["NIHT", "HTP", "CGIHT"])
def test_dense_config1(gb, gbo, alg):
    """Dense Gaussian n=4096, m=1024, k=102, +-1 signal, tol 1e-4*||y|| (first workload)."""
    n, m, k = 4096, 1024, 102
    A, x0, ks, op, y = dense_problem(gbo, n, m, k, seed=1234)
    tol = 1e-4 * float(np.linalg.norm(y))
    opts = gb.gaga_options("tol", tol)
    x, iters, conv = gb.gaga_cs(alg, "gen", y, A.reshape(n, m).T, ks, opts)
    xo, info = gbo.solve(alg, op, y, ks, tol)
    assert np.linalg.norm(x - x0) / np.linalg.norm(x0) < 1e-3
    assert np.linalg.norm(x - xo) / np.linalg.norm(xo) < REL_X_TOL
    assert np.array_equal(np.flatnonzero(x), np.flatnonzero(xo))
    assert abs(iters - info.iter) <= 2


@pytest.mark.parametrize("alg", ["NIHT", "HTP", "CGIHT"])
def test_dct_small(gb, gbo, alg):
    n = 2 ** 14
    m, k = n // 4, n // 40
    rows = gbo.gen_dct_rows(n, m, seed=77)
    x0, ks = gbo.gen_vector(n, k, 2, seed=77)
    op = gbo.Op.dct(n, rows)
    y = gbo.A(op, x0)
    tol = 1e-5 * float(np.linalg.norm(y))
    opts = gb.gaga_options("tol", tol)
    x, iters, conv = gb.gaga_cs(alg, "dct", y, rows, ks, m, n, opts, index_base=0)
    xo, info = gbo.solve(alg, op, y, ks, tol)
    assert np.linalg.norm(x - x0) / np.linalg.norm(x0) < 1e-3
    assert np.linalg.norm(x - xo) / np.linalg.norm(xo) < 1e-4


@pytest.mark.parametrize("alg", ["NIHT", "CGIHT"])
def test_smv_small(gb, gbo, alg):
    n, m, d = 2 ** 14, 2 ** 12, 7
    k = m // 20
    rows, vals = gbo.gen_smv(m, n, d, 1, seed=5)
    x0, ks = gbo.gen_vector(n, k, 1, seed=5)
    op = gbo.Op.smv(m, n, d, rows, vals)
    y = gbo.A(op, x0)
    tol = 1e-4 * float(np.linalg.norm(y))
    opts = gb.gaga_options("tol", tol)
    cols = np.repeat(np.arange(n, dtype=np.int32), d)
    x, iters, conv, rec, trec = gb.gaga_cs(alg, "smv", y, rows, cols, vals, ks, opts, index_base=0)
    xo, info = gbo.solve(alg, op, y, ks, tol)
    assert np.linalg.norm(x - x0) / np.linalg.norm(x0) < 1e-3
    assert np.linalg.norm(x - xo) / np.linalg.norm(xo) < REL_X_TOL


def test_parallel_l0_bit_exact(gb, gbo):
    """Unit-valued expander and a +-1 signal: every residual value is an integer, so the
    decoder is exact and must reproduce the oracle bit for bit (x, iterations, record)."""
    n, m, d = 2 ** 14, 2 ** 12, 7
    k = m // 20
    rows, vals = gbo.gen_smv(m, n, d, 3, seed=9)
    x0, ks = gbo.gen_vector(n, k, 1, seed=9)
    op = gbo.Op.smv(m, n, d, rows, vals)
    y = gbo.A(op, x0)
    cols = np.repeat(np.arange(n, dtype=np.int32), d)
    opts = gb.gaga_options("tol", 1e-6, "maxiter", 300)
    x, iters, conv, rec, trec = gb.gaga_cs("parallel_l0", "smv", y, rows, cols, vals, ks, opts, index_base=0)
    xo, reso, reco, info = gbo.parallel_l0(op, y, tol=1e-6, maxiter=300)
    assert iters == info.iter
    assert np.array_equal(x, xo)
    assert np.array_equal(rec[: iters + 1], reco[: iters + 1])
    assert np.array_equal(x, x0)


def test_linear_binning_golden(gb):
    """gb_cs_linear_binning against LinearBinning of the reference run on the CPU."""
    torch = _torch()
    z = np.load(os.path.join(GOLD, "linear_binning.npz"))
    L = gb._lib.load()
    for name in z["names"]:
        v = torch.tensor(z[f"{name}__v"], device="cuda")
        nb = int(z[f"{name}__num_bins"])
        mb = int(z[f"{name}__max_bin"])
        bins = torch.zeros(len(v), dtype=torch.int32, device="cuda")
        cnt = torch.zeros(nb, dtype=torch.int32, device="cuda")
        st = L.gb_cs_linear_binning(v.data_ptr(), len(v), nb, mb, float(z[f"{name}__slope"]),
                                    float(z[f"{name}__intercept"]), bins.data_ptr(), cnt.data_ptr(), None)
        assert st == 0
        torch.cuda.synchronize()
        assert np.array_equal(bins.cpu().numpy(), z[f"{name}__bins"]), name
        assert np.array_equal(cnt.cpu().numpy(), z[f"{name}__counters"]), name


def test_find_support_set_vs_oracle(gb, gbo):
    torch = _torch()
    L = gb._lib.load()
    rng = np.random.default_rng(5)
    for n, k, nb in ((5000, 100, 1000), (2 ** 16, 3000, 3276), (777, 700, 1000)):
        v = rng.standard_normal(n).astype(np.float32)
        mx = np.float32(np.abs(v).max())
        slope = np.float32(np.float32(nb - 1) / mx)
        s_o, bins_o, cnt_o, st_o = gbo.find_support_set(v, k, nb, slope, mx, 1.0)
        vt = torch.tensor(v, device="cuda")
        bins = torch.zeros(n, dtype=torch.int32, device="cuda")
        st = gb._lib.BinState(nb, int(np.float32(nb) * np.float32(0.75)), 0, 0, 0.25, 0.0)
        rc = L.gb_cs_find_support_set(vt.data_ptr(), n, k, float(slope), float(mx), 1.0, C.byref(st),
                                      bins.data_ptr(), None, 1, None)
        assert rc == 0
        torch.cuda.synchronize()
        assert np.array_equal(bins.cpu().numpy(), bins_o)
        assert (st.k_bin, st.sum, st.max_bin) == (st_o.k_bin, st_o.sum, st_o.max_bin)
        assert np.float32(st.min_val) == np.float32(st_o.min_val)
        vo = v.copy()
        gbo.lib().gbo_threshold(vo.ctypes.data, bins_o.ctypes.data, st_o.k_bin, n)
        assert np.array_equal(vt.cpu().numpy(), vo)


def test_l0_step_golden(gb):
    torch = _torch()
    z = np.load(os.path.join(GOLD, "l0_step.npz"))
    L = gb._lib.load()
    for i in range(int(z["count"])):
        g = lambda key: z[f"c{i}__{key}"]
        m, n, d, shift = int(g("m")), int(g("n")), int(g("d")), int(g("shift"))
        res = torch.tensor(g("res"), device="cuda")
        x = torch.zeros(n, device="cuda")
        upd = torch.zeros(n, device="cuda")
        rows = torch.tensor(g("rows"), device="cuda")
        found = C.c_int(0)
        rc = L.gb_cs_l0_step(res.data_ptr(), x.data_ptr(), upd.data_ptr(), rows.data_ptr(), m, n, d, 1, shift,
                             C.byref(found), None)
        assert rc == 0
        assert found.value == int(g("found"))
        assert np.array_equal(x.cpu().numpy(), g("x_after"))
        assert np.array_equal(upd.cpu().numpy(), g("updates"))
        # updates are applied to each row in ascending column order, as the reference's
        # kernel run sequentially does: bit-exact for integer and real residuals alike
        assert np.array_equal(res.cpu().numpy(), g("res_after"))


@pytest.mark.parametrize("m,n,frac", [(257, 700, 0.5), (513, 2000, 1.0), (1001, 3000, 0.05), (1001, 1200, 1.0),
                                      (4099, 1500, 0.9)])
def test_dense_apply_row_tiles(gb, gbo, m, n, frac):
    """A x_S of the drop-in's operator apply (256-row tiles, the support split down to 64
    columns per CTA when there are few tiles): m one past a tile boundary, m not a multiple
    of 4 (scalar loads), tiny and full supports, many tiles; against the oracle's product."""
    torch = _torch()
    L = gb._lib.load()
    rng = np.random.default_rng(m + n)
    A = gbo.gen_dense(m, n, seed=m)
    op = gbo.Op.dense(A, m, n)
    dA = torch.tensor(A, device="cuda")
    p = gb._lib.Problem(0, m, n, 0, None, dA.data_ptr(), m, None, None, None, 0, 0, 1, None)
    x = rng.standard_normal(n).astype(np.float32)
    x[rng.random(n) >= frac] = 0.0
    dx = torch.tensor(x, device="cuda")
    out = torch.full((m,), 7.0, device="cuda")
    assert L.gb_cs_operator_apply(C.byref(p), 0, dx.data_ptr(), out.data_ptr()) == 0
    yo = gbo.A(op, x)
    np.testing.assert_allclose(out.cpu().numpy(), yo, rtol=0, atol=2e-5 * max(np.abs(yo).max(), 1e-30))


@pytest.mark.parametrize("kind", ["dense", "dct", "smv"])
def test_operator_apply(gb, gbo, kind):
    torch = _torch()
    L = gb._lib.load()
    rng = np.random.default_rng(3)
    if kind == "dense":
        m, n = 300, 1000
        A = gbo.gen_dense(m, n, seed=4)
        op = gbo.Op.dense(A, m, n)
        dA = torch.tensor(A, device="cuda")
        p = gb._lib.Problem(0, m, n, 0, None, dA.data_ptr(), m, None, None, None, 0, 0, 1, None)
        keep = [dA]
    elif kind == "dct":
        n = 4096
        m = 1024
        rows = gbo.gen_dct_rows(n, m, seed=8)
        op = gbo.Op.dct(n, rows)
        dr = torch.tensor(rows, device="cuda")
        p = gb._lib.Problem(1, m, n, 0, None, None, 0, dr.data_ptr(), None, None, 0, 0, 1, None)
        keep = [dr]
    else:
        m, n, d = 512, 2048, 7
        rows, vals = gbo.gen_smv(m, n, d, 1, seed=6)
        op = gbo.Op.smv(m, n, d, rows, vals)
        dr, dv = torch.tensor(rows, device="cuda"), torch.tensor(vals, device="cuda")
        p = gb._lib.Problem(2, m, n, 0, None, None, 0, dr.data_ptr(), None, dv.data_ptr(), d, 0, 1, None)
        keep = [dr, dv]
    x = rng.standard_normal(n).astype(np.float32)
    x[rng.random(n) < 0.7] = 0.0
    r = rng.standard_normal(m).astype(np.float32)
    dx, dr_ = torch.tensor(x, device="cuda"), torch.tensor(r, device="cuda")
    out_m = torch.zeros(m, device="cuda")
    out_n = torch.zeros(n, device="cuda")
    assert L.gb_cs_operator_apply(C.byref(p), 0, dx.data_ptr(), out_m.data_ptr()) == 0
    assert L.gb_cs_operator_apply(C.byref(p), 1, dr_.data_ptr(), out_n.data_ptr()) == 0
    ya, ga = out_m.cpu().numpy(), out_n.cpu().numpy()
    yo, go = gbo.A(op, x), gbo.AT(op, r)
    if kind == "smv":
        assert np.array_equal(ya, yo)
        assert np.array_equal(ga, go)
    else:
        np.testing.assert_allclose(ya, yo, rtol=0, atol=2e-5 * np.abs(yo).max())
        np.testing.assert_allclose(ga, go, rtol=0, atol=2e-5 * np.abs(go).max())
    del keep


@pytest.mark.parametrize("m,n,d,ens", [(512, 2048, 7, 2), (512, 2048, 7, 3), (65536, 4096, 7, 1),
                                        (65537, 4096, 7, 1), (70000, 4096, 5, 2), (3000, 4096, 12, 1),
                                        (3000, 4096, 12, 2), (3000, 1024, 20, 1), (4000, 2 ** 19 + 7, 3, 2),
                                        (4000, 2 ** 19, 3, 1)])
def test_smv_operator_layouts(gb, gbo, m, n, d, ens):
    """Every layout of the expander kernels, bit for bit against the oracle: 16-bit row
    indices (m <= 65536) or 32-bit, one value for all entries (ensembles 1 and 3: no value
    stream) or the +-1/sqrt(d) values streamed (ensemble 2), d up to 8, up to 16 and above
    (one entry after another), n up to and beyond 2^19."""
    torch = _torch()
    L = gb._lib.load()
    rng = np.random.default_rng(m + d)
    rows, vals = gbo.gen_smv(m, n, d, ens, seed=m + 3 * d + ens)
    op = gbo.Op.smv(m, n, d, rows, vals)
    dr, dv = torch.tensor(rows, device="cuda"), torch.tensor(vals, device="cuda")
    p = gb._lib.Problem(2, m, n, 0, None, None, 0, dr.data_ptr(), None, dv.data_ptr(), d, 0, 1, None)
    x = rng.standard_normal(n).astype(np.float32)
    x[rng.random(n) < 0.5] = 0.0
    r = rng.standard_normal(m).astype(np.float32)
    dx, dr_ = torch.tensor(x, device="cuda"), torch.tensor(r, device="cuda")
    out_m = torch.zeros(m, device="cuda")
    out_n = torch.zeros(n, device="cuda")
    assert L.gb_cs_operator_apply(C.byref(p), 0, dx.data_ptr(), out_m.data_ptr()) == 0
    assert L.gb_cs_operator_apply(C.byref(p), 1, dr_.data_ptr(), out_n.data_ptr()) == 0
    assert np.array_equal(out_m.cpu().numpy(), gbo.A(op, x))
    assert np.array_equal(out_n.cpu().numpy(), gbo.AT(op, r))


@pytest.mark.parametrize("logn", [5, 6, 7, 8, 9, 10, 11, 13, 16, 20, 22, 24])
def test_dct_operator_large(gb, gbo, logn):
    """The subsampled DCT against the oracle's FP64 DCT, A and A^T.  n < 128 runs the
    n-point shared-memory transform; from n = 128 on, the n/2-point transform in two passes
    of 2^l1 x 2^l2 (l1 + l2 = log2 n - 1) Stockham sequences with 8 elements per thread:
    every pass-length class from 8 (radix-8 only) through 16 and 32 (a radix-2 / radix-4
    tail) up to 4096 (512 threads per sequence, n = 2^24), and the workload size 2^20."""
    torch = _torch()
    L = gb._lib.load()
    n = 2 ** logn
    m = max(1, n // 4)
    rows = gbo.gen_dct_rows(n, m, seed=logn)
    op = gbo.Op.dct(n, rows)
    rng = np.random.default_rng(logn)
    x = rng.standard_normal(n).astype(np.float32)
    x[rng.random(n) < 0.5] = 0.0
    r = rng.standard_normal(m).astype(np.float32)
    dr = torch.tensor(rows, device="cuda")
    p = gb._lib.Problem(1, m, n, 0, None, None, 0, dr.data_ptr(), None, None, 0, 0, 1, None)
    dx, drr = torch.tensor(x, device="cuda"), torch.tensor(r, device="cuda")
    out_m, out_n = torch.zeros(m, device="cuda"), torch.zeros(n, device="cuda")
    assert L.gb_cs_operator_apply(C.byref(p), 0, dx.data_ptr(), out_m.data_ptr()) == 0
    assert L.gb_cs_operator_apply(C.byref(p), 1, drr.data_ptr(), out_n.data_ptr()) == 0
    ya, ga = out_m.cpu().numpy(), out_n.cpu().numpy()
    yo, go = gbo.A(op, x), gbo.AT(op, r)
    np.testing.assert_allclose(ya, yo, rtol=0, atol=2e-5 * np.abs(yo).max())
    np.testing.assert_allclose(ga, go, rtol=0, atol=2e-5 * np.abs(go).max())
    assert np.linalg.norm(ya - yo) / np.linalg.norm(yo) < 1e-5
    assert np.linalg.norm(ga - go) / np.linalg.norm(go) < 1e-5


@pytest.mark.parametrize("tr,drop", [(2, 8), (3, 16)])
def test_dense_compact_gradient_operand(gb, tr, drop):
    """A^T r over the batched form's compact operand (A rounded to nearest even at bit 8:
    24-bit entries, or at bit 16: BF16) against the same rounding done in numpy and an FP64
    product; FP32 accumulation, so within 1e-5 of max |A^T r|.  Ragged m (a tail inside the
    last group of 8 rows) and n not a multiple of 4."""
    torch = _torch()
    L = gb._lib.load()
    m, n, lda = 301, 1003, 304
    rng = np.random.default_rng(tr)
    A = np.zeros((n, lda), dtype=np.float32)
    A[:, :m] = rng.standard_normal((n, m)).astype(np.float32) / np.sqrt(m)
    r = rng.standard_normal(m).astype(np.float32)
    b = A[:, :m].view(np.uint32).astype(np.uint64)
    half = (1 << (drop - 1)) - 1
    q = ((b + half + ((b >> drop) & 1)) & ~np.uint64((1 << drop) - 1)).astype(np.uint32).view(np.float32)
    want = q.astype(np.float64) @ r.astype(np.float64)
    dA, dr = torch.tensor(A.ravel(), device="cuda"), torch.tensor(r, device="cuda")
    out = torch.zeros(n, device="cuda")
    p = gb._lib.Problem(0, m, n, 0, None, dA.data_ptr(), lda, None, None, None, 0, 0, 1, None)
    ms = C.c_float(0)
    assert L.gb_cs_operator_time(C.byref(p), tr, dr.data_ptr(), out.data_ptr(), 0, 1, None, 0, C.byref(ms)) == 0
    got = out.cpu().numpy()
    assert np.abs(got - want).max() <= 1e-5 * np.abs(want).max()
    # and it is not the FP32 product: the rounding is visible at this tolerance for BF16
    if drop == 16:
        full = A[:, :m].astype(np.float64) @ r.astype(np.float64)
        assert np.abs(got - full).max() > 1e-4 * np.abs(full).max()
