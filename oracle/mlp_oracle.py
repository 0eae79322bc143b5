"""float64 numpy restatement of the scoring MLP -- TEST INFRASTRUCTURE.

The GPU kernels (sgfim_mlp_forward / sgfim_mlp_backward) are checked against
this: the same bf16-rounded weights, fp32/fp64 arithmetic, ReLU, sigmoid
output and the weighted mean binary cross-entropy.  The reference project
has no learned component, so this oracle is pinned by finite differences
(see tests), not by reference outputs.
"""
from __future__ import annotations

import numpy as np


def bf16_round(a):
    """Round float32 values to bfloat16 (round to nearest, ties to even) and
    return them as float64."""
    u = np.ascontiguousarray(a, dtype=np.float32).view(np.uint32).astype(np.uint64)
    r = ((u >> 16) & 1) + 0x7FFF
    b = ((u + r) >> 16).astype(np.uint32) << 16
    return b.view(np.float32).astype(np.float64)


def forward(X, W1, b1, W2, b2, w3, b3):
    X = np.asarray(X, np.float64)
    z1 = X @ W1.T + b1
    h1 = np.maximum(z1, 0)
    z2 = h1 @ W2.T + b2
    h2 = np.maximum(z2, 0)
    s = h2 @ w3 + b3
    p = 1.0 / (1.0 + np.exp(-s))
    return z1, z2, p


def loss_and_grads(X, Y, WT, W1, b1, W2, b2, w3, b3):
    """Mean over rows of WT * BCE(p, Y) and its gradients (all float64)."""
    X = np.asarray(X, np.float64)
    n = len(X)
    WT = np.ones(n) if WT is None else np.asarray(WT, np.float64)
    z1, z2, p = forward(X, W1, b1, W2, b2, w3, b3)
    pc = np.clip(p, 1e-7, 1 - 1e-7)
    loss = float(np.sum(-WT * (Y * np.log(pc) + (1 - Y) * np.log(1 - pc))) / n)
    dz3 = WT * (p - Y) / n
    h1 = np.maximum(z1, 0)
    h2 = np.maximum(z2, 0)
    dw3 = h2.T @ dz3
    db3 = np.array([dz3.sum()])
    dz2 = np.outer(dz3, w3) * (z2 > 0)
    dW2 = dz2.T @ h1
    db2 = dz2.sum(0)
    dz1 = (dz2 @ W2) * (z1 > 0)
    dW1 = dz1.T @ X
    db1 = dz1.sum(0)
    return loss, dict(W1=dW1, b1=db1, W2=dW2, b2=db2, w3=dw3, b3=db3)
