"""The warm-start network: CPU oracle (oracle/mlp.py) pinned by finite
differences, and the GPU kernels (BF16 tensor-core GEMM, forward, backward,
Adam) checked against it.

Tolerances: the GEMM within 1e-5 of sum_k |a_k b_k| per output (FP32
accumulation of exact BF16 products); loss within 1e-5 relative, outputs
within 2e-3 and gradients within 5e-3 relative (2-norm per tensor) of the
oracle that rounds the same
operands to BF16 (the rest is FP32 accumulation order and the occasional
one-ulp BF16 flip of an intermediate gradient); within 5e-2 of the plain
float64 network (the BF16 error itself).
"""
import numpy as np
import pytest

from oracle import mlp as OM


def _params(dims, rng):
    return [(rng.standard_normal((dims[l + 1], dims[l])) * np.sqrt(2.0 / dims[l]),
             0.1 * rng.standard_normal(dims[l + 1])) for l in range(len(dims) - 1)]


def test_oracle_gradients_match_finite_differences():
    rng = np.random.default_rng(0)
    dims = [5, 7, 6, 4]
    params = _params(dims, rng)
    X = rng.standard_normal((9, 5))
    T = rng.standard_normal((9, 4))
    _, dW, db = OM.loss_and_gradients(params, X, T, bf16_ops=False)
    h = 1e-6
    for l, (W, b) in enumerate(params):
        for (i, j) in [(0, 0), (dims[l + 1] - 1, dims[l] - 1), (1, 2)]:
            Wp = [(w.copy(), bb.copy()) for w, bb in params]
            Wm = [(w.copy(), bb.copy()) for w, bb in params]
            Wp[l][0][i, j] += h
            Wm[l][0][i, j] -= h
            fd = (OM.loss_and_gradients(Wp, X, T, False)[0] - OM.loss_and_gradients(Wm, X, T, False)[0]) / (2 * h)
            assert abs(fd - dW[l][i, j]) < 1e-7 + 1e-6 * abs(fd)
        k = dims[l + 1] // 2
        bp = [(w.copy(), bb.copy()) for w, bb in params]
        bm = [(w.copy(), bb.copy()) for w, bb in params]
        bp[l][1][k] += h
        bm[l][1][k] -= h
        fd = (OM.loss_and_gradients(bp, X, T, False)[0] - OM.loss_and_gradients(bm, X, T, False)[0]) / (2 * h)
        assert abs(fd - db[l][k]) < 1e-7 + 1e-6 * abs(fd)


def test_bf16_rounding():
    x = np.array([1.0, 1.00390625, 1.005859375, -3.14159, 0.0, 65504.0], dtype=np.float32)
    r = OM.bf16(x)
    # bf16 keeps 8 significant bits; ties go to even
    assert r[0] == 1.0 and r[1] == 1.0 and r[2] == 1.0078125
    assert abs(r[3] + 3.140625) < 1e-12 and r[4] == 0.0
    bits = OM.bf16_bits(x)
    assert bits[0] == 0x3F80 and bits[4] == 0


def rel(a, b):
    return np.linalg.norm(np.asarray(a, np.float64) - b) / max(np.linalg.norm(b), 1e-300)


@pytest.mark.gpu
@pytest.mark.parametrize("M,N,K", [(1, 1, 8), (130, 70, 40), (256, 512, 512), (64, 96, 4096), (300, 257, 30752)])
def test_gemm_bf16(cuda_ok, M, N, K):
    from shell_gb300 import lib as L
    rng = np.random.default_rng(M + N + K)
    A = rng.standard_normal((M, K)).astype(np.float32)
    B = rng.standard_normal((N, K)).astype(np.float32)
    C = L.gemm_bf16(OM.bf16_bits(A), OM.bf16_bits(B))
    Ab, Bb = OM.bf16(A), OM.bf16(B)
    ref = Ab @ Bb.T
    bound = np.abs(Ab) @ np.abs(Bb).T
    assert np.all(np.abs(C - ref) <= 1e-5 * bound + 1e-30)


@pytest.mark.gpu
@pytest.mark.parametrize("dims,n", [([8, 64, 64, 40], 17), ([8, 512, 512, 512, 512, 30726], 32)])
def test_mlp_gradients_match_oracle(cuda_ok, dims, n):
    from shell_gb300 import lib as L
    rng = np.random.default_rng(1)
    net = L.MLP(dims, max_batch=64, seed=3)
    params = [(W.astype(np.float64), b.astype(np.float64)) for W, b in net.get_params()]
    params = [(W, 0.05 * rng.standard_normal(b.shape)) for W, b in params]
    net.set_params(params)
    params = [(W.astype(np.float32).astype(np.float64), b.astype(np.float32).astype(np.float64)) for W, b in params]
    X = rng.standard_normal((n, dims[0])).astype(np.float32)
    T = rng.standard_normal((n, dims[-1])).astype(np.float32)
    loss, dW, db = net.gradients(X, T)
    lo, dWo, dbo = OM.loss_and_gradients(params, X, T, bf16_ops=True)
    assert abs(loss - lo) <= 1e-5 * lo
    for l in range(len(dims) - 1):
        assert rel(dW[l], dWo[l]) < 5e-3, l
        assert rel(db[l], dbo[l]) < 5e-3, l
    lp, dWp, dbp = OM.loss_and_gradients(params, X, T, bf16_ops=False)
    assert abs(loss - lp) <= 5e-2 * lp
    for l in range(len(dims) - 1):
        assert rel(dW[l], dWp[l]) < 5e-2, l
    Y = net.predict(X)
    Yo, _ = OM.forward(params, X, bf16_ops=True)
    # a one-ulp BF16 flip of a hidden activation (2^-8 relative) propagates through the deeper layers
    assert rel(Y, Yo) < 2e-3


@pytest.mark.gpu
def test_mlp_training_fits_smooth_map(cuda_ok):
    """Adam on shuffled mini-batches drives the loss of a smooth 8 -> 300 map down."""
    from shell_gb300 import lib as L
    rng = np.random.default_rng(2)
    X = rng.uniform(-1, 1, (2048, 8)).astype(np.float32)
    basis = rng.standard_normal((8, 300))
    T = np.tanh(X @ basis * 0.5).astype(np.float32)
    net = L.MLP([8, 128, 128, 300], max_batch=256, seed=0)
    net.set_dataset(X, T)
    curve = net.train(1500, 256, lr0=2e-3, lr_final=1e-5, seed=0, curve_every=100)
    assert curve[-1] < 0.05 * curve[0], curve
    Y = net.predict(X[:100])
    assert np.mean((Y - T[:100]) ** 2) < 0.1 * np.mean(T[:100] ** 2)
