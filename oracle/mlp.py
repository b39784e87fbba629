"""CPU oracle of the warm-start surrogate network (numpy, float64 arithmetic).

Test infrastructure only: the GPU network (shl_mlp_*) is checked against this
restatement.  It mirrors the GPU's rounding points so that the comparison can
be tight: the GEMM operands (weights, activations, output gradients) are
rounded to bfloat16 (round to nearest even), products are accumulated exactly
enough in float64, GELU is the erf form, the loss is the mean squared error
over the real outputs and its gradient 2 (y - t) / (n n_out).  With
``bf16=False`` it is the plain float64 network (no rounding), the reference for
the size of the BF16 error itself.
"""
import math

import numpy as np

try:
    from scipy.special import erf as _erf
except ImportError:  # pragma: no cover
    _erf = np.vectorize(math.erf)


def bf16(x):
    """Round float32 values to bfloat16 (nearest even); returned as float64."""
    a = np.ascontiguousarray(x, dtype=np.float32)
    b = a.view(np.uint32).astype(np.uint64)
    b = (b + 0x7FFF + ((b >> 16) & 1)) & 0xFFFF0000
    return b.astype(np.uint32).view(np.float32).astype(np.float64)


def bf16_bits(x):
    """bfloat16 bit patterns (uint16) of float values, round to nearest even."""
    a = np.ascontiguousarray(x, dtype=np.float32)
    b = a.view(np.uint32).astype(np.uint64)
    return (((b + 0x7FFF + ((b >> 16) & 1)) >> 16) & 0xFFFF).astype(np.uint16)


def gelu(x):
    return 0.5 * x * (1.0 + _erf(x / math.sqrt(2.0)))


def gelu_grad(x):
    return 0.5 * (1.0 + _erf(x / math.sqrt(2.0))) + x * np.exp(-0.5 * x * x) / math.sqrt(2.0 * math.pi)


def forward(params, X, bf16_ops=True):
    """Returns (Y, cache).  params: [(W (out x in), b)], GELU after all but the last layer."""
    r = bf16 if bf16_ops else (lambda a: np.asarray(a, np.float64))
    H = r(X)
    cache = []
    L = len(params)
    for l, (W, b) in enumerate(params):
        Z = H @ r(W).T + np.asarray(b, np.float64)
        cache.append((H, Z))
        if l < L - 1:
            H = r(gelu(Z))
    return Z, cache


def loss_and_gradients(params, X, T, bf16_ops=True):
    """Mean squared error and its gradients (dW, db per layer), mirroring the GPU."""
    r = bf16 if bf16_ops else (lambda a: np.asarray(a, np.float64))
    Y, cache = forward(params, X, bf16_ops)
    n, m = Y.shape
    d = Y - np.asarray(T, np.float64)
    loss = float(np.mean(d * d))
    dZ = r(2.0 * d / (n * m))
    dWs, dbs = [None] * len(params), [None] * len(params)
    for l in range(len(params) - 1, -1, -1):
        H, _ = cache[l]
        dWs[l] = dZ.T @ H
        dbs[l] = dZ.sum(axis=0)
        if l == 0:
            break
        dH = dZ @ r(params[l][0])
        dZ = r(dH * gelu_grad(cache[l - 1][1]))
    return loss, dWs, dbs
