"""FP64 numpy restatement of the sign-risk network's forward and backward passes --
TEST INFRASTRUCTURE ONLY (the gradient check of the GPU kernels in
rhizome_v24.15_gb300/csrc/k_learn.cu). The network has no counterpart in the reference.

Arithmetic contract mirrored from the kernels: inputs, weights and hidden activations
are rounded to BF16 (round to nearest even) before each product, biases stay FP32, and
the gradient is taken with respect to the rounded weights (the FP32 master copy is what
Adam updates). Loss: weighted binary cross-entropy with logits, summed over rows.
"""
from __future__ import annotations

import numpy as np

F, H = 32, 64
oW1, ob1 = 0, H * F
oW2, ob2 = ob1 + H, ob1 + H + H * H
ow3 = ob2 + H
ob3 = ow3 + H
N_PARAMS = ob3 + 1


def bf16(x):
    """Round float32 values to bfloat16 (nearest even), returned as float64."""
    a = np.ascontiguousarray(np.asarray(x, np.float32))
    u = a.view(np.uint32).astype(np.uint64)
    rounding = ((u >> 16) & 1) + 0x7FFF
    r = ((u + rounding) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def _identity(x):
    return np.asarray(x, np.float64)


def unpack(P, rounding=True):
    r = bf16 if rounding else _identity
    P = np.asarray(P, np.float32 if rounding else np.float64)
    return (r(P[oW1:ob1]).reshape(H, F), P[ob1:oW2].astype(np.float64), r(P[oW2:ob2]).reshape(H, H),
            P[ob2:ow3].astype(np.float64), r(P[ow3:ob3]), float(P[ob3]))


def forward(P, X, rounding=True):
    """Logits of the rows of X. ``rounding=False`` drops every BF16 rounding (a smooth
    FP64 function, used to check the backward formulas by finite differences)."""
    r = bf16 if rounding else _identity
    W1, b1, W2, b2, w3, b3 = unpack(P, rounding)
    x = r(X)
    z1 = x @ W1.T + b1
    a1 = r(np.maximum(z1, 0.0).astype(np.float32 if rounding else np.float64))
    z2 = a1 @ W2.T + b2
    a2 = r(np.maximum(z2, 0.0).astype(np.float32 if rounding else np.float64))
    z = a2 @ w3 + b3
    return z, (x, z1, a1, z2, a2)


def loss(P, X, y, w=None, rounding=True):
    z, _ = forward(P, X, rounding)
    y = np.asarray(y, np.float64)
    w = np.ones_like(y) if w is None else np.asarray(w, np.float64)
    return float(np.sum(w * (np.maximum(z, 0) - z * y + np.log1p(np.exp(-np.abs(z))))))


def adam(P, g, m, v, step, lr, b1=0.9, b2=0.999, eps=1e-8, scale=1.0):
    """One Adam step (Kingma and Ba 2015) in FP64; returns new (P, m, v)."""
    g = np.asarray(g, np.float64) * scale
    m = b1 * m + (1 - b1) * g
    v = b2 * v + (1 - b2) * g * g
    P = P - lr * (m / (1 - b1 ** step)) / (np.sqrt(v / (1 - b2 ** step)) + eps)
    return P, m, v


def loss_and_grad(P, X, y, w=None, rounding=True):
    W1, b1, W2, b2, w3, b3 = unpack(P, rounding)
    z, (x, z1, a1, z2, a2) = forward(P, X, rounding)
    y = np.asarray(y, np.float64)
    w = np.ones_like(y) if w is None else np.asarray(w, np.float64)
    loss = float(np.sum(w * (np.maximum(z, 0) - z * y + np.log1p(np.exp(-np.abs(z))))))
    dz = w * (1.0 / (1.0 + np.exp(-z)) - y)
    g = np.zeros(N_PARAMS, np.float64)
    g[ob3] = dz.sum()
    g[ow3:ob3] = dz @ a2
    d2 = (dz[:, None] * w3[None, :]) * (z2 > 0)
    g[ob2:ow3] = d2.sum(0)
    g[oW2:ob2] = (d2.T @ a1).ravel()
    d1 = (d2 @ W2) * (z1 > 0)
    g[ob1:oW2] = d1.sum(0)
    g[oW1:ob1] = (d1.T @ x).ravel()
    return loss, g
