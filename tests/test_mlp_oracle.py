"""The learned proposal's MLP oracle (oracle/mlp.py): its backward pass
against central finite differences of its own float64 forward pass, and its
BF16 rounding against the definition (round to nearest, ties to even)."""
import numpy as np

from oracle import mlp as ref


def test_bf16_rounding():
    x = np.array([1.0, 1.0 + 2.0 ** -8, 1.0 + 3 * 2.0 ** -8, 1.0 + 2.0 ** -9, -2.5, 0.0, 3.0e38], np.float32)
    r = ref.bf16(x)
    # 1 + 2^-8 is a tie between 1 and 1 + 2^-7: ties go to the even mantissa (1)
    assert r[0] == 1.0 and r[1] == 1.0 and r[2] == 1.0 + 2.0 ** -6 and r[3] == 1.0
    assert r[4] == -2.5 and r[5] == 0.0
    assert np.all(np.abs(ref.bf16(np.linspace(-7, 7, 1001, dtype=np.float32)) - np.linspace(-7, 7, 1001))
                  <= 2.0 ** -8 * 8)


def test_gradient_matches_finite_differences():
    rng = np.random.default_rng(3)
    nIn, nH, n = 6, 9, 17
    P = nH * nIn + nH + nH * nH + nH + nH + 1
    p = rng.normal(scale=0.4, size=P)
    X = rng.normal(size=(n, nIn))
    t = rng.normal(size=n)
    g, _ = ref.gradient(p, X, t, nIn, nH, rnd=ref.exact)
    h = 1e-6
    fd = np.zeros(P)
    for i in range(P):
        e = np.zeros(P)
        e[i] = h
        fd[i] = (ref.loss(p + e, X, t, nIn, nH, ref.exact) - ref.loss(p - e, X, t, nIn, nH, ref.exact)) / (2 * h)
    np.testing.assert_allclose(g, fd, rtol=1e-5, atol=1e-8)


def test_bf16_forward_close_to_exact():
    rng = np.random.default_rng(4)
    nIn, nH = 32, 128
    P = nH * nIn + nH + nH * nH + nH + nH + 1
    p = rng.normal(scale=0.1, size=P).astype(np.float32)
    X = rng.normal(size=(64, nIn)).astype(np.float32)
    y16 = ref.forward(p, X, nIn, nH)[2]
    y64 = ref.forward(p, X, nIn, nH, rnd=ref.exact)[2]
    assert np.abs(y16 - y64).max() <= 2e-2 * (np.abs(y64).max() + 1e-3)
