"""CPU FP64 restatement of the indicator network (TEST INFRASTRUCTURE ONLY):
forward, max-pooled BCE loss and its gradient, with the BF16-rounded weights
the GPU kernels use.  Used to check the GPU inference (tensor-core) and backward
kernels."""
from __future__ import annotations

import numpy as np

NIN, NH = 25, 32
NPARAM = NH * NIN + NH + NH * NH + NH + NH + 1


def bf16_round(p: np.ndarray) -> np.ndarray:
    """round-to-nearest-even float32 -> bfloat16, returned as float64"""
    u = np.ascontiguousarray(p, dtype=np.float32).view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def unpack(p):
    o = 0
    W1 = p[o:o + NH * NIN].reshape(NH, NIN); o += NH * NIN
    b1 = p[o:o + NH]; o += NH
    W2 = p[o:o + NH * NH].reshape(NH, NH); o += NH * NH
    b2 = p[o:o + NH]; o += NH
    W3 = p[o:o + NH]; o += NH
    b3 = p[o]
    return W1, b1, W2, b2, W3, b3


def logits(X, params, act_bf16=False):
    """[n][3] logits of every direction; act_bf16 rounds the inputs and the first
    hidden layer to BF16 as the tensor-core inference path does (its operand type)"""
    W1, b1, W2, b2, W3, b3 = unpack(bf16_round(params))
    X = bf16_round(X).reshape(X.shape) if act_bf16 else X.astype(np.float64)
    a1 = X @ W1.T + b1
    h1 = np.maximum(a1, 0.0)
    if act_bf16:
        h1 = bf16_round(h1).reshape(h1.shape)
    a2 = h1 @ W2.T + b2
    return np.maximum(a2, 0.0) @ W3 + b3


def loss_and_grad(X, y, params, pos_weight=1.0):
    W1, b1, W2, b2, W3, b3 = unpack(bf16_round(params))
    X = X.astype(np.float64)
    z_all = logits(X, params)
    d = np.argmax(z_all, axis=1)
    x = X[np.arange(X.shape[0]), d]
    a1 = x @ W1.T + b1
    h1 = np.maximum(a1, 0.0)
    a2 = h1 @ W2.T + b2
    h2 = np.maximum(a2, 0.0)
    z = h2 @ W3 + b3
    sp = lambda t: np.logaddexp(0.0, t)  # noqa: E731
    loss = float(np.sum(pos_weight * y * sp(-z) + (1 - y) * sp(z)))
    s = 1.0 / (1.0 + np.exp(-z))
    dz = pos_weight * y * (s - 1.0) + (1.0 - y) * s
    gW3 = dz @ h2
    gb3 = dz.sum()
    ga2 = (dz[:, None] * W3[None, :]) * (a2 > 0)
    gW2 = ga2.T @ h1
    gb2 = ga2.sum(0)
    ga1 = (ga2 @ W2) * (a1 > 0)
    gW1 = ga1.T @ x
    gb1 = ga1.sum(0)
    g = np.concatenate([gW1.ravel(), gb1, gW2.ravel(), gb2, gW3, [gb3]])
    return loss, g
