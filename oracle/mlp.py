"""TEST INFRASTRUCTURE ONLY -- CPU oracle of the learned bond-integral surrogate.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may import this.

The surrogate replaces the quadrature of the bond integral (the reference's
FixedPointCGFunc / AdaptiveCGFunc::getBondFunc, irvingkirkwood/cgfunc/
CoarseGrainFunction.h:85-88 and :124-127) for a Gaussian kernel truncated at 3
widths, on bonds that cross the edge of its support.  In units of the width w:

    B(d, a, b) = int_0^1 exp(-(d^2 + (a + s (b - a))^2) / 2) [r < 3] ds

with d the distance of the grid point from the bond's line and a, b the signed
positions of the two ends along it.  This module holds

* ``label``: B in closed form (clip the segment to the ball, then the error function
  along the line) -- the exact answer the GPU's adaptive-quadrature labels must match;
* ``base`` / ``targets``: four-point Gauss-Legendre on the clipped segment, and the
  scaled relative correction y = (B / base - 1) * YSCALE the network predicts;
* ``inputs`` / ``forward`` / ``loss_and_grad``: the network 4 -> 64 -> 64 -> 64 -> 1
  with SiLU in FP64 and its exact gradient by reverse-mode differentiation, in the
  parameter layout of the C ABI (W1[64][4], b1, W2[64][64], b2, W3[64][64], b3, w4, b4);
* ``forward_bf16``: the deployed arithmetic (BF16 weights and activations, the first
  layer split three ways, SiLU through tanh), accumulated in FP64.

The mirrored kernels are in pyglasstools_gb300/csrc/ik_mlp.cu (mlp_base, k_mlp_samples,
k_mlp_infer_simt, k_mlp_infer_tc).
"""
from __future__ import annotations

import math

import numpy as np

H = 64
O_W1 = 0
O_B1 = O_W1 + H * 4
O_W2 = O_B1 + H
O_B2 = O_W2 + H * H
O_W3 = O_B2 + H
O_B3 = O_W3 + H * H
O_W4 = O_B3 + H
O_B4 = O_W4 + H
NPAR = O_B4 + 1
YSCALE = 1.0e4  # network output = (B / base - 1) * YSCALE

_erf = np.vectorize(math.erf)


def label(d, a, b):
    """Exact B(d, a, b) (units of w, un-normalised Gaussian, support r < 3)."""
    d, a, b = (np.asarray(v, dtype=np.float64) for v in (d, a, b))
    lo, hi = np.minimum(a, b), np.maximum(a, b)
    tc = np.sqrt(np.maximum(9.0 - d * d, 0.0))
    t0, t1 = np.maximum(lo, -tc), np.minimum(hi, tc)
    length = hi - lo
    val = np.sqrt(np.pi / 2.0) * (_erf(t1 / np.sqrt(2.0)) - _erf(t0 / np.sqrt(2.0)))
    out = np.exp(-0.5 * d * d) * val / np.where(length > 0, length, 1.0)
    return np.where((t1 > t0) & (length > 0), out, 0.0)


def split(p):
    p = np.asarray(p, dtype=np.float64)
    return (p[O_W1:O_B1].reshape(H, 4), p[O_B1:O_W2], p[O_W2:O_B2].reshape(H, H), p[O_B2:O_W3],
            p[O_W3:O_B3].reshape(H, H), p[O_B3:O_W4], p[O_W4:O_B4], p[O_B4])


def inputs(feats):
    """x = (sqrt(1 - (d/3)^2), a/4, b/4, 2 (w - 1.5)) from float32 features {d, a, b, w}."""
    f = np.asarray(feats, dtype=np.float32).astype(np.float64)
    d, a, b, w = f[:, 0], f[:, 1], f[:, 2], f[:, 3]
    return np.stack([np.sqrt(np.maximum(1.0 - (d / 3.0) ** 2, 0.0)), a / 4.0, b / 4.0, 2.0 * (w - 1.5)], axis=1)


def _silu(z):
    return z / (1.0 + np.exp(-z))


def _silu_grad(z):
    s = 1.0 / (1.0 + np.exp(-z))
    return s * (1.0 + z * (1.0 - s))


def forward(p, feats):
    W1, b1, W2, b2, W3, b3, w4, b4 = split(p)
    x = inputs(feats)
    h1 = _silu(x @ W1.T + b1)
    h2 = _silu(h1 @ W2.T + b2)
    h3 = _silu(h2 @ W3.T + b3)
    return h3 @ w4 + b4


def loss_and_grad(p, feats, targets):
    """Mean squared error of y over the batch and its gradient (FP64)."""
    W1, b1, W2, b2, W3, b3, w4, b4 = split(p)
    x = inputs(feats)
    y = np.asarray(targets, dtype=np.float32).astype(np.float64)
    n = len(x)
    z1 = x @ W1.T + b1
    h1 = _silu(z1)
    z2 = h1 @ W2.T + b2
    h2 = _silu(z2)
    z3 = h2 @ W3.T + b3
    h3 = _silu(z3)
    out = h3 @ w4 + b4
    r = out - y
    loss = float(np.mean(r * r))
    dy = 2.0 * r / n
    g = np.zeros(NPAR)
    g[O_W4:O_B4] = h3.T @ dy
    g[O_B4] = dy.sum()
    dz3 = np.outer(dy, w4) * _silu_grad(z3)
    g[O_W3:O_B3] = (dz3.T @ h2).ravel()
    g[O_B3:O_W4] = dz3.sum(0)
    dz2 = (dz3 @ W3) * _silu_grad(z2)
    g[O_W2:O_B2] = (dz2.T @ h1).ravel()
    g[O_B2:O_W3] = dz2.sum(0)
    dz1 = (dz2 @ W2) * _silu_grad(z1)
    g[O_W1:O_B1] = (dz1.T @ x).ravel()
    g[O_B1:O_W2] = dz1.sum(0)
    return loss, g


def bf16(v):
    """Round float32 values to the nearest BF16 (ties to even), returned as float64."""
    u = np.asarray(v, dtype=np.float32).view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def base(feats):
    """Four-point Gauss-Legendre on the part of the bond inside the support:
    s1/2 sum_k w_k exp(-(d^2 + t_k^2)/2), t_k = a + s1 (b - a)(1 + x_k)/2, with
    t_c = sqrt(9 - d^2) and s1 = (t_c - a)/(b - a) clipped to [0, 1]."""
    f = np.asarray(feats, dtype=np.float32).astype(np.float64)
    d, a, b = f[:, 0], f[:, 1], f[:, 2]
    tc = np.sqrt(np.maximum(9.0 - d * d, 0.0))
    s1 = np.clip((tc - a) / np.where(b - a > 0, b - a, 1.0), 0.0, 1.0)
    x, w = np.polynomial.legendre.leggauss(4)
    h = 0.5 * s1 * (b - a)
    t = (a + h)[:, None] + h[:, None] * x[None, :]
    return 0.5 * s1 * np.sum(w[None, :] * np.exp(-0.5 * (d[:, None] ** 2 + t * t)), axis=1)


BASE_MIN = 1e-6  # targets are 0 below this baseline (the labels' tolerance is 1e-14 absolute)


def targets(feats, labels):
    """Training targets y = (B / base - 1) * YSCALE, clipped to [-8, 8]; 0 where the
    baseline is below BASE_MIN."""
    bs = base(feats)
    y = (np.asarray(labels) / np.where(bs > BASE_MIN, bs, 1.0) - 1.0) * YSCALE
    return np.where(bs > BASE_MIN, np.clip(y, -8.0, 8.0), 0.0)


def value(feats, y):
    """B from the network's output y: base (1 + y / YSCALE)."""
    return base(feats) * (1.0 + np.asarray(y, dtype=np.float64) / YSCALE)


def forward_bf16(p, feats):
    """y of the deployed network: BF16 weights; the first layer split three ways
    (x_hi W_hi + x_lo W_hi + x_hi W_lo); hidden-layer biases as the BF16 pair
    hi + lo that the tensor cores add; BF16 activations; FP64 accumulation; tanh-form
    SiLU."""
    W1, b1, W2, b2, W3, b3, w4, b4 = split(p)
    silu = lambda z: 0.5 * z + 0.5 * z * np.tanh(0.5 * z)
    bpair = lambda b: bf16(b) + bf16(b - bf16(b))
    x = inputs(feats)
    xh, W1h = bf16(x), bf16(W1)
    xl, W1l = bf16(x - xh), bf16(W1 - W1h)
    z1 = xh @ W1h.T + xl @ W1h.T + xh @ W1l.T + bpair(b1)
    h = bf16(silu(z1))
    h = bf16(silu(h @ bf16(W2).T + bpair(b2)))
    h = silu(h @ bf16(W3).T + bpair(b3))
    return h @ bf16(w4) + b4
