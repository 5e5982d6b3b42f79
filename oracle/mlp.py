"""NumPy restatement of the learned proposal's MLP (forward pass and the
gradient of the mean squared error) with the same BF16 rounding of the
products' operands.  TEST INFRASTRUCTURE ONLY: the checker for the device
forward / backward kernels."""
from __future__ import annotations

import numpy as np


def bf16(x):
    """Round float32 to the nearest bfloat16 (ties to even), as float32."""
    x = np.ascontiguousarray(x, np.float32)
    u = x.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000).astype(np.uint32)
    return r.view(np.float32)


def unpack(p, nIn, nH):
    o = 0
    W1 = p[o:o + nH * nIn].reshape(nH, nIn); o += nH * nIn
    b1 = p[o:o + nH]; o += nH
    W2 = p[o:o + nH * nH].reshape(nH, nH); o += nH * nH
    b2 = p[o:o + nH]; o += nH
    W3 = p[o:o + nH]; o += nH
    b3 = p[o:o + 1]
    return W1, b1, W2, b2, W3, b3


def exact(x):
    """No rounding: the float64 network the BF16 one approximates."""
    return np.asarray(x, np.float64)


def _mm(a, b, rnd):
    out = rnd(a).astype(np.float64) @ rnd(b).astype(np.float64)
    return out if rnd is exact else out.astype(np.float32)


def forward(p, X, nIn, nH, rnd=bf16):
    """Layer activations H1, H2 (after ReLU) and the output y.  With rnd=bf16
    every product's operands are rounded to BF16 and the products and biases
    accumulate in FP32, as on the device; rnd=exact is the float64 network."""
    W1, b1, W2, b2, W3, b3 = unpack(rnd(p), nIn, nH)
    H1 = np.maximum(_mm(X, W1.T, rnd) + b1, 0)
    H2 = np.maximum(_mm(H1, W2.T, rnd) + b2, 0)
    y = _mm(H2, W3[:, None], rnd)[:, 0] + b3[0]
    return H1, H2, y


def loss(p, X, t, nIn, nH, rnd=bf16):
    y = forward(p, X, nIn, nH, rnd)[2]
    return float(np.mean((np.asarray(y, np.float64) - t) ** 2))


def gradient(p, X, t, nIn, nH, rnd=bf16):
    """Gradient of the mean squared error over the rows of X in the device's
    parameter order (W1, b1, W2, b2, W3, b3) and the loss."""
    W1, b1, W2, b2, W3, b3 = unpack(rnd(p), nIn, nH)
    H1, H2, y = forward(p, X, nIn, nH, rnd)
    n = len(X)
    dy = 2.0 * (y - t) / n
    if rnd is not exact:
        dy = dy.astype(np.float32)
    gW3 = _mm(dy[None, :], H2, rnd)[0]
    gb3 = np.array([dy.sum()])
    dH2 = _mm(dy[:, None], W3[None, :], rnd) * (H2 > 0)
    gW2 = _mm(dH2.T, H1, rnd)
    gb2 = dH2.sum(0)
    dH1 = _mm(dH2, W2, rnd) * (H1 > 0)
    gW1 = _mm(dH1.T, X, rnd)
    gb1 = dH1.sum(0)
    g = np.concatenate([gW1.ravel(), gb1, gW2.ravel(), gb2, gW3, gb3])
    return g, float(np.mean((np.asarray(y, np.float64) - t) ** 2))
