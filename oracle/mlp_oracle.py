"""TEST INFRASTRUCTURE: float64 NumPy restatement of the learned-seed encoder's
forward and backward pass, the checker of kcna_encoder_grads.

Encoder: x -> Z1 = W1 x + b1 -> G = GELU(Z1) -> Z2 = W2 G + b2 -> Y = Z2/|Z2|,
loss = mean over triplets of max(0, |Ya-Yp|^2 - |Ya-Yn|^2 + margin).
The CUDA path rounds the inputs of every product to BF16 (round to nearest
even) and accumulates in FP32; the oracle rounds the same operands to BF16 and
multiplies in float64, so the remaining differences are accumulation order and
single- vs double-precision elementwise arithmetic.
"""
from __future__ import annotations

import math

import numpy as np


def bf16(x) -> np.ndarray:
    """Round to the nearest BF16 (ties to even), returned as float64."""
    u = np.ascontiguousarray(x, dtype=np.float32).view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


_erf = np.vectorize(math.erf)


def gelu(x):
    return 0.5 * x * (1.0 + _erf(x / math.sqrt(2.0)))


def gelu_grad(x):
    return 0.5 * (1.0 + _erf(x / math.sqrt(2.0))) + x * np.exp(-0.5 * x * x) / math.sqrt(2.0 * math.pi)


def encoder_grads(X, W1, b1, W2, b2, margin):
    X = np.asarray(X, np.float64)
    R = X.shape[0]
    B = R // 3
    Z1 = bf16(X) @ bf16(W1).T + b1
    G = gelu(Z1)
    Z2 = bf16(G) @ bf16(W2).T + b2
    n = np.maximum(np.linalg.norm(Z2, axis=1, keepdims=True), 1e-12)
    Y = Z2 / n
    ya, yp, yn = Y[:B], Y[B:2 * B], Y[2 * B:]
    l = ((ya - yp) ** 2).sum(1) - ((ya - yn) ** 2).sum(1) + margin
    act = (l > 0).astype(np.float64)[:, None]
    loss = float((l * act[:, 0]).sum() / B)
    s = 2.0 / B * act
    dY = np.concatenate([s * (yn - yp), s * (yp - ya), s * (ya - yn)])
    dZ2 = (dY - Y * (Y * dY).sum(1, keepdims=True)) / n
    db2 = dZ2.sum(0)
    dW2 = bf16(dZ2).T @ bf16(G)
    dG = bf16(dZ2) @ bf16(W2)
    dZ1 = dG * gelu_grad(Z1)
    db1 = dZ1.sum(0)
    dW1 = bf16(dZ1).T @ bf16(X)
    return loss, dW1, db1, dW2, db2
