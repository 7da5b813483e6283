"""CPU oracle of the learned warm start's network (test infrastructure only).

Restates in float64 numpy what gaga_gb300/csrc/gb_learned.cu computes, so the GPU kernels
can be checked against it:
  - the features of a coordinate of g = A^T y (float32 arithmetic, as on the device):
    |g_i| / max|g|, rank fraction from a 4096-bin histogram of |g|, delta = m/n, rho = k/m;
  - the MLP 4 -> 64 -> 64 -> 1 with exact (erf) GELU and weights rounded to BF16;
  - the mean squared error against targets and its gradient with respect to the FP32
    parameters (the forward pass uses their BF16 rounding, the gradient flows to them
    unchanged, as in mixed-precision training).
The network has no counterpart in the reference; the warm start it feeds replaces the
H_k(A^T y) start of CGIHT (GAGA/gaga/algorithms.cu:3776).
"""
import numpy as np
from scipy.special import erf

IN, H = 4, 64
OFF_W1 = 0
OFF_B1 = OFF_W1 + H * IN
OFF_W2 = OFF_B1 + H
OFF_B2 = OFF_W2 + H * H
OFF_W3 = OFF_B2 + H
OFF_B3 = OFF_W3 + H
P = OFF_B3 + 1
RANK_BINS = 4096


def bf16(a):
    """Round float32 values to the nearest BF16 (ties to even), returned as float32."""
    u = np.ascontiguousarray(a, dtype=np.float32).view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) >> 16 << 16
    return u.astype(np.uint32).view(np.float32)


def unpack(p):
    p = np.asarray(p, dtype=np.float64)
    return (p[OFF_W1:OFF_B1].reshape(H, IN), p[OFF_B1:OFF_W2], p[OFF_W2:OFF_B2].reshape(H, H), p[OFF_B2:OFF_W3],
            p[OFF_W3:OFF_B3], p[OFF_B3])


def init_params(seed=0):
    """He-style initialisation (float32)."""
    rng = np.random.default_rng(seed)
    p = np.zeros(P, dtype=np.float32)
    p[OFF_W1:OFF_B1] = rng.standard_normal(H * IN) * np.sqrt(2.0 / IN)
    p[OFF_W2:OFF_B2] = rng.standard_normal(H * H) * np.sqrt(2.0 / H)
    p[OFF_W3:OFF_B3] = rng.standard_normal(H) * np.sqrt(1.0 / H)
    return p


def gelu(a):
    return 0.5 * a * (1.0 + erf(a / np.sqrt(2.0)))


def gelu_grad(a):
    return 0.5 * (1.0 + erf(a / np.sqrt(2.0))) + a * np.exp(-0.5 * a * a) / np.sqrt(2.0 * np.pi)


def forward(p, F, keep=False, round_weights=True):
    W1, b1, W2, b2, W3, b3 = unpack(bf16(p) if round_weights else p)
    F = np.asarray(F, dtype=np.float64)
    A1 = F @ W1.T + b1
    H1 = gelu(A1)
    A2 = H1 @ W2.T + b2
    H2 = gelu(A2)
    out = H2 @ W3 + b3
    if keep:
        return out, (F, A1, H1, A2, H2, W2, W3)
    return out


def loss_and_grad(p, F, t, round_weights=True):
    """Mean squared error over the rows of F and its gradient (float64)."""
    out, (F, A1, H1, A2, H2, W2, W3) = forward(p, F, keep=True, round_weights=round_weights)
    t = np.asarray(t, dtype=np.float64)
    ns = len(t)
    r = out - t
    loss = float(np.sum(r * r) / ns)
    dout = 2.0 * r / ns
    g = np.zeros(P, dtype=np.float64)
    g[OFF_W3:OFF_B3] = H2.T @ dout
    g[OFF_B3] = dout.sum()
    dA2 = np.outer(dout, W3) * gelu_grad(A2)
    g[OFF_W2:OFF_B2] = (dA2.T @ H1).ravel()
    g[OFF_B2:OFF_W3] = dA2.sum(0)
    dA1 = (dA2 @ W2) * gelu_grad(A1)
    g[OFF_W1:OFF_B1] = (dA1.T @ F).ravel()
    g[OFF_B1:OFF_W2] = dA1.sum(0)
    return loss, g


def features(g, m, k):
    """Features (n x 4, float32) of g = A^T y in the device's float32 arithmetic."""
    g = np.asarray(g, dtype=np.float32)
    n = len(g)
    a = np.abs(g)
    mx = np.float32(a.max())
    slope = np.float32(RANK_BINS - 1) / mx if mx > 0 else np.float32(0.0)
    b = ((mx - a) * slope).astype(np.float32)
    b = np.clip(np.trunc(b).astype(np.int64), 0, RANK_BINS - 1)
    cnt = np.bincount(b, minlength=RANK_BINS)
    cum = np.concatenate([[0], np.cumsum(cnt)[:-1]])
    f = np.empty((n, IN), dtype=np.float32)
    f[:, 0] = a / mx if mx > 0 else 0.0
    f[:, 1] = (cum[b].astype(np.float32) + np.float32(0.5) * cnt[b].astype(np.float32)) / np.float32(n)
    f[:, 2] = np.float32(m) / np.float32(n)
    f[:, 3] = np.float32(k) / np.float32(m)
    return f
