"""The learned proposal's MLP on the device (BF16 operands, FP32
accumulation) against the NumPy oracle with the same rounding, and its
training loop."""
import numpy as np
import pytest

import optcuts_gb300 as oc
from oracle import mlp as ref

pytestmark = pytest.mark.gpu


def data(n, nIn=32, seed=0):
    rng = np.random.default_rng(seed)
    X = rng.normal(size=(n, nIn)).astype(np.float32)
    t = np.tanh(X[:, 0] - 0.5 * X[:, 1] * X[:, 2] + 0.25 * X[:, 3] ** 2).astype(np.float32)
    return X, t


def test_params_round_trip():
    m = oc.MLP(32, 128, seed=1)
    p = m.params()
    assert p.size == m.num_params() == 128 * 32 + 128 + 128 * 128 + 128 + 128 + 1
    q = np.random.default_rng(2).normal(scale=0.05, size=p.size).astype(np.float32)
    m.set_params(q)
    np.testing.assert_array_equal(m.params(), q)


@pytest.mark.parametrize("n", [1, 37, 1000])
def test_forward_matches_oracle(n):
    m = oc.MLP(32, 128, seed=5)
    X, _ = data(n, seed=n)
    y = m.predict(X)
    yr = ref.forward(m.params(), X, 32, 128)[2]
    # same BF16 operands; FP32 accumulation order differs (and may flip a
    # BF16 rounding of a hidden activation): 1e-3 of the output scale
    assert np.abs(y - yr).max() <= 1e-3 * (np.abs(yr).max() + 1e-3)


@pytest.mark.parametrize("n", [3, 256, 3000])
def test_gradient_matches_oracle(n):
    m = oc.MLP(32, 128, seed=7)
    X, t = data(n, seed=n + 1)
    g, loss = m.gradient(X, t)
    gr, lr = ref.gradient(m.params(), X, t, 32, 128)
    assert loss == pytest.approx(lr, rel=1e-4)
    # per block, relative to the block's norm
    nH, nIn = 128, 32
    offs = np.cumsum([0, nH * nIn, nH, nH * nH, nH, nH, 1])
    for a, b in zip(offs[:-1], offs[1:]):
        err = np.linalg.norm(g[a:b] - gr[a:b])
        assert err <= 2e-3 * (np.linalg.norm(gr[a:b]) + 1e-12), (a, b)


def test_gradient_step_decreases_loss():
    """The device gradient is a descent direction of the exact loss."""
    m = oc.MLP(32, 128, seed=11)
    X, t = data(512, seed=12)
    p = m.params()
    g, l0 = m.gradient(X, t)
    m.set_params(p - 1e-2 * g / (np.linalg.norm(g) + 1e-30))
    _, l1 = m.gradient(X, t)
    assert l1 < l0


def test_training_fits():
    m = oc.MLP(32, 128, seed=13)
    X, t = data(8192, seed=14)
    _, l0 = m.gradient(X, t)
    lf = m.train(X, t, epochs=40, batch=256, lr=2e-3, seed=1)
    Xv, tv = data(2048, seed=15)
    yv = m.predict(Xv)
    assert lf < 0.2 * l0
    assert np.mean((yv - tv) ** 2) < 0.3 * np.var(tv)


def test_invalid_arguments():
    m = oc.MLP(32, 128)
    with pytest.raises(oc.OCError):
        m.train(np.zeros((0, 32), np.float32), np.zeros(0, np.float32))


@pytest.mark.parametrize("M,N,K,ta,tb", [
    (128, 128, 64, False, False),   # one tile, one stage
    (1000, 128, 32, False, True),   # X W1^T: the first layer (K = 32, half a stage)
    (300, 128, 128, False, True),   # H1 W2^T: ragged rows, two stages
    (128, 128, 777, True, False),   # dH2^T H1: reduction over rows, ragged K
    (128, 32, 513, True, False),    # dH1^T X: N = 32
    (77, 200, 48, False, False),    # two tiles along N, ragged everything
])
def test_tensor_core_gemm_matches_cuda_cores(M, N, K, ta, tb):
    """tcgen05.mma (BF16 from shared memory, FP32 in tensor memory) against
    the CUDA-core kernel with the same BF16 operands, and both against the
    BF16-rounded float64 product."""
    rng = np.random.default_rng(M + N + K)
    A = rng.normal(size=(K, M) if ta else (M, K)).astype(np.float32)
    B = rng.normal(size=(N, K) if tb else (K, N)).astype(np.float32)
    tc = oc.bf16_gemm(A, B, True, ta, tb)
    cc = oc.bf16_gemm(A, B, False, ta, tb)
    a64 = ref.bf16(A).astype(np.float64)
    b64 = ref.bf16(B).astype(np.float64)
    exact = (a64.T if ta else a64) @ (b64.T if tb else b64)
    scale = np.sqrt(K) * 4.0
    assert np.abs(tc - exact).max() <= 1e-5 * scale
    assert np.abs(cc - exact).max() <= 1e-5 * scale
    np.testing.assert_allclose(tc, cc, rtol=0, atol=2e-5 * scale)


def test_tensor_core_wait_timeout_is_reported():
    """The bounded mbarrier wait of the tensor-core GEMM, made to run out
    (a bound of 0 polls: the first stage's MMAs are in flight): the product
    ends with OC_ERR_TIMEOUT after the kernel drained its MMAs and released
    its tensor memory, and the next product on the same context, with the
    default bound, is correct."""
    rng = np.random.default_rng(5)
    A = rng.normal(size=(1000, 128)).astype(np.float32)
    B = rng.normal(size=(128, 128)).astype(np.float32)
    assert oc.lib().oc_tc_set_wait_polls(0) == oc.OC_OK
    try:
        with pytest.raises(oc.OCError) as e:
            oc.bf16_gemm(A, B, True)
        assert e.value.status == oc.OC_ERR_TIMEOUT
    finally:
        assert oc.lib().oc_tc_set_wait_polls(-1) == oc.OC_OK
    assert oc.lib().oc_tc_set_wait_polls(-2) == oc.OC_ERR_INVALID
    tc = oc.bf16_gemm(A, B, True)
    exact = ref.bf16(A).astype(np.float64) @ ref.bf16(B).astype(np.float64)
    assert np.abs(tc - exact).max() <= 1e-5 * np.sqrt(128) * 4.0


def test_network_on_tensor_cores_matches_cuda_cores():
    """The two product kernels accumulate in a different order, so a hidden
    activation can round to the neighbouring BF16 value (2^-8 relative) on
    one of them: agreement to that scale."""
    X, t = data(700, seed=21)
    a = oc.MLP(32, 128, seed=22)
    b = oc.MLP(32, 128, seed=22)
    b.set_tensor_cores(False)
    ya, yb = a.predict(X), b.predict(X)
    assert np.abs(ya - yb).max() <= 4e-3 * np.abs(yb).max()
    assert np.median(np.abs(ya - yb)) <= 1e-5 * np.abs(yb).max()
    ga, la = a.gradient(X, t)
    gb, lb = b.gradient(X, t)
    assert la == pytest.approx(lb, rel=1e-3)
    assert np.linalg.norm(ga - gb) <= 2e-3 * np.linalg.norm(gb)
