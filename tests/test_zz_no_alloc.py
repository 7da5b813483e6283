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
