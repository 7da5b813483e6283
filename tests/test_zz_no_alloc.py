"""gb_cs_dense_apply_noalloc: the dense operator apply for callers that cannot allocate
device memory during a call (inside a CUDA stream capture, under an up-front memory
budget, or behind an allocator that is not CUDA's).  Its scratch is a fixed device array
inside the library.  It must give the same products as gb_cs_operator_apply, which
allocates a workspace per call, on consecutive calls that reuse the shared scratch.

This file is collected last so that a failure here leaves every other test already run.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _torch():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def test_noalloc_matches_allocating_apply(gb, gbo):
    torch = _torch()
    L = gb._lib.load()
    rng = np.random.default_rng(21)
    for (m, n) in ((300, 1000), (1024, 4096)):
        A = gbo.gen_dense(m, n, seed=5 + m)
        dA = torch.tensor(A, device="cuda")
        p = gb._lib.Problem(0, m, n, 0, None, dA.data_ptr(), m, None, None, None, 0, 0, 1, None)
        for call in range(2):  # two calls in a row share (and reuse) the scratch
            x = rng.standard_normal(n).astype(np.float32)
            x[rng.random(n) < 0.6] = 0.0
            r = rng.standard_normal(m).astype(np.float32)
            dx, dr = torch.tensor(x, device="cuda"), torch.tensor(r, device="cuda")
            ref_m, ref_n = torch.zeros(m, device="cuda"), torch.zeros(n, device="cuda")
            assert L.gb_cs_operator_apply(C.byref(p), 0, dx.data_ptr(), ref_m.data_ptr()) == 0
            assert L.gb_cs_operator_apply(C.byref(p), 1, dr.data_ptr(), ref_n.data_ptr()) == 0
            out_m, out_n = torch.full((m,), 7.0, device="cuda"), torch.full((n,), 7.0, device="cuda")
            assert L.gb_cs_dense_apply_noalloc(dA.data_ptr(), m, m, n, 0, dx.data_ptr(), out_m.data_ptr(), None) == 0
            assert L.gb_cs_dense_apply_noalloc(dA.data_ptr(), m, m, n, 1, dr.data_ptr(), out_n.data_ptr(), None) == 0
            torch.cuda.synchronize()
            for got, want in ((out_m, ref_m), (out_n, ref_n)):
                g, w = got.cpu().numpy(), want.cpu().numpy()
                np.testing.assert_allclose(g, w, rtol=0, atol=2e-5 * np.abs(w).max())


def _alloc_apply(gb, L, dA, lda, m, n, transpose, d_in, d_out):
    p = gb._lib.Problem(0, m, n, 0, None, dA.data_ptr(), lda, None, None, None, 0, 0, 1, None)
    assert L.gb_cs_operator_apply(C.byref(p), transpose, d_in.data_ptr(), d_out.data_ptr()) == 0


def _close(got, want):
    g, w = got.cpu().numpy(), want.cpu().numpy()
    np.testing.assert_allclose(g, w, rtol=0, atol=2e-5 * max(np.abs(w).max(), 1e-30))


@pytest.mark.parametrize("m,lda,n", [(301, 301, 700), (301, 304, 700), (14746, 14748, 40), (20000, 20000, 48),
                                     (65536, 65536, 24)])
def test_noalloc_ragged_padded_and_large_m(gb, m, lda, n):
    """Ragged m (scalar path), padded lda (float4 path), and m up to the documented limit:
    the support-split count is lowered until the partial tiles fit the scratch, so every
    m <= 65536 is accepted.  Two calls of each direction in a row."""
    torch = _torch()
    L = gb._lib.load()
    g = torch.Generator(device="cpu").manual_seed(m + lda)
    Afull = torch.randn(n, lda, generator=g) / np.sqrt(m)
    dA = Afull.to("cuda").contiguous()
    for call in range(2):
        x = torch.randn(n, generator=g)
        x[torch.rand(n, generator=g) < 0.5] = 0.0
        r = torch.randn(m, generator=g)
        dx, dr = x.to("cuda"), r.to("cuda")
        ref_m, ref_n = torch.zeros(m, device="cuda"), torch.zeros(n, device="cuda")
        _alloc_apply(gb, L, dA, lda, m, n, 0, dx, ref_m)
        _alloc_apply(gb, L, dA, lda, m, n, 1, dr, ref_n)
        out_m, out_n = torch.full((m,), 7.0, device="cuda"), torch.full((n,), 7.0, device="cuda")
        assert L.gb_cs_dense_apply_noalloc(dA.data_ptr(), lda, m, n, 0, dx.data_ptr(), out_m.data_ptr(), None) == 0, \
            L.gb_cs_last_error()
        assert L.gb_cs_dense_apply_noalloc(dA.data_ptr(), lda, m, n, 1, dr.data_ptr(), out_n.data_ptr(), None) == 0, \
            L.gb_cs_last_error()
        torch.cuda.synchronize()
        _close(out_m, ref_m)
        _close(out_n, ref_n)


def test_noalloc_transpose_input_not_16_byte_aligned(gb):
    """A^T r with r starting 4 bytes into an allocation (a tensor slice): the float4 path
    is for 16-byte aligned inputs only, so this call takes the scalar path."""
    torch = _torch()
    L = gb._lib.load()
    m, n = 1024, 512
    g = torch.Generator(device="cpu").manual_seed(3)
    dA = (torch.randn(n, m, generator=g) / 32.0).to("cuda").contiguous()
    base = torch.randn(m + 1, generator=g).to("cuda")
    dr = base[1:]
    assert dr.data_ptr() % 16 == 4
    ref = torch.zeros(n, device="cuda")
    _alloc_apply(gb, L, dA, m, m, n, 1, dr.contiguous(), ref)
    for call in range(2):
        out = torch.full((n,), 7.0, device="cuda")
        assert L.gb_cs_dense_apply_noalloc(dA.data_ptr(), m, m, n, 1, dr.data_ptr(), out.data_ptr(), None) == 0
        torch.cuda.synchronize()
        _close(out, ref)


def test_noalloc_fixed_support_mode_call_order(gb):
    """transpose 2 is accepted only right after a transpose 0 call on the same A, lda, m
    and n: a transpose 1 call in between, or another m / lda / A, is rejected."""
    torch = _torch()
    L = gb._lib.load()
    m, n = 600, 1500
    g = torch.Generator(device="cpu").manual_seed(9)
    dA = (torch.randn(n, 608, generator=g) / 25.0).to("cuda").contiguous()
    x = torch.randn(n, generator=g)
    x[torch.rand(n, generator=g) < 0.6] = 0.0
    dx = x.to("cuda")
    r = torch.randn(m, device="cuda")
    out_m, out_n = torch.zeros(m, device="cuda"), torch.zeros(n, device="cuda")
    P = dA.data_ptr()
    assert L.gb_cs_dense_apply_noalloc(P, 608, m, n, 0, dx.data_ptr(), out_m.data_ptr(), None) == 0
    assert L.gb_cs_dense_apply_noalloc(P, 608, m, n, 1, r.data_ptr(), out_n.data_ptr(), None) == 0
    assert L.gb_cs_dense_apply_noalloc(P, 608, m, n, 2, dx.data_ptr(), out_m.data_ptr(), None) == gb._lib.GB_BAD_ARG
    assert b"transpose == 1" in L.gb_cs_last_error()
    assert L.gb_cs_dense_apply_noalloc(P, 608, m, n, 0, dx.data_ptr(), out_m.data_ptr(), None) == 0
    for bad in ((P, 608, m - 8, n), (P, 604, m, n), (P + 16 * 608, 608, m, n - 1)):
        assert L.gb_cs_dense_apply_noalloc(bad[0], bad[1], bad[2], bad[3], 2, dx.data_ptr(), out_m.data_ptr(),
                                           None) == gb._lib.GB_BAD_ARG
    x2 = (x * 2.0 + torch.sign(x)).to("cuda")  # same support, new values
    assert L.gb_cs_dense_apply_noalloc(P, 608, m, n, 2, x2.data_ptr(), out_m.data_ptr(), None) == 0
    torch.cuda.synchronize()
    want = dA.double()[:, :m].T @ x2.double()
    _close(out_m, want.float())


def test_noalloc_rejects_sizes_beyond_the_scratch(gb):
    L = gb._lib.load()
    assert L.gb_cs_dense_apply_noalloc(None, 10, 10, 10, 0, None, None, None) == gb._lib.GB_BAD_ARG
    big = 1 << 17
    fake = C.c_void_p(256)
    assert L.gb_cs_dense_apply_noalloc(fake, big, big, 8, 0, fake, fake, None) == gb._lib.GB_BAD_ARG
    assert b"65536" in L.gb_cs_last_error()


def test_noalloc_fixed_support_mode(gb, gbo):
    """transpose 2 reuses the support of the previous transpose 0 call (same n)."""
    torch = _torch()
    L = gb._lib.load()
    rng = np.random.default_rng(22)
    m, n = 640, 2048
    A = gbo.gen_dense(m, n, seed=77)
    dA = torch.tensor(A, device="cuda")
    x = rng.standard_normal(n).astype(np.float32)
    x[rng.random(n) < 0.7] = 0.0
    x2 = (x * 3.0 - np.sign(x)).astype(np.float32)  # same support, new values
    out = torch.zeros(m, device="cuda")
    assert L.gb_cs_dense_apply_noalloc(dA.data_ptr(), m, m, n, 0, torch.tensor(x, device="cuda").data_ptr(),
                                       out.data_ptr(), None) == 0
    dx2 = torch.tensor(x2, device="cuda")
    assert L.gb_cs_dense_apply_noalloc(dA.data_ptr(), m, m, n, 2, dx2.data_ptr(), out.data_ptr(), None) == 0
    torch.cuda.synchronize()
    want = A.reshape(n, m).T.astype(np.float64) @ x2.astype(np.float64)
    np.testing.assert_allclose(out.cpu().numpy(), want, rtol=0, atol=2e-5 * np.abs(want).max())
    # a different n has no support list to reuse
    assert L.gb_cs_dense_apply_noalloc(dA.data_ptr(), m, m, n // 2, 2, dx2.data_ptr(), out.data_ptr(),
                                       None) == gb._lib.GB_BAD_ARG
    assert L.gb_cs_dense_apply_noalloc(dA.data_ptr(), m, m, n, 3, dx2.data_ptr(), out.data_ptr(),
                                       None) == gb._lib.GB_BAD_ARG
