"""TEST INFRASTRUCTURE ONLY: FP64 numpy restatement of the plan tuner's cost model.

The engine trains its cost model (a 3-layer MLP, in -> 64 -> 64 -> 1 with
ReLU, mean squared error, Adam) with its own CUDA kernels
(``kfft_gb300/csrc/mlp.cu``).  This module is the CPU check for those kernels:
the same forward pass, the analytic gradient by back-propagation, and Adam, in
FP64, on the same packed parameter layout

    W1[64][in] b1[64] W2[64][64] b2[64] W3[64] b3[1]   (row-major)

The reference has no learned planner (its factorisation rule is fixed,
kfft_generic.c:129-151), so there is nothing of the reference to pin here;
the gradient is pinned instead by central finite differences in the tests.
Only the tests import this module.
"""
from __future__ import annotations

import numpy as np

H = 64


def n_params(d_in: int) -> int:
    return H * d_in + H + H * H + H + H + 1


def unpack(p: np.ndarray, d_in: int):
    p = np.asarray(p, dtype=np.float64)
    o = 0
    W1 = p[o:o + H * d_in].reshape(H, d_in)
    o += H * d_in
    b1 = p[o:o + H]
    o += H
    W2 = p[o:o + H * H].reshape(H, H)
    o += H * H
    b2 = p[o:o + H]
    o += H
    W3 = p[o:o + H]
    o += H
    b3 = p[o]
    return W1, b1, W2, b2, W3, b3


def forward(p: np.ndarray, X: np.ndarray) -> np.ndarray:
    X = np.asarray(X, dtype=np.float64)
    W1, b1, W2, b2, W3, b3 = unpack(p, X.shape[1])
    h1 = np.maximum(X @ W1.T + b1, 0.0)
    h2 = np.maximum(h1 @ W2.T + b2, 0.0)
    return h2 @ W3 + b3


def loss_grad(p: np.ndarray, X: np.ndarray, y: np.ndarray):
    """Mean squared error over the rows and its gradient, packed like p."""
    X = np.asarray(X, dtype=np.float64)
    y = np.asarray(y, dtype=np.float64)
    n, d_in = X.shape
    W1, b1, W2, b2, W3, b3 = unpack(p, d_in)
    a1 = X @ W1.T + b1
    h1 = np.maximum(a1, 0.0)
    a2 = h1 @ W2.T + b2
    h2 = np.maximum(a2, 0.0)
    f = h2 @ W3 + b3
    e = f - y
    loss = float(np.mean(e * e))
    dout = 2.0 * e / n
    gW3 = h2.T @ dout
    gb3 = dout.sum()
    d2 = np.outer(dout, W3) * (a2 > 0)
    gW2 = d2.T @ h1
    gb2 = d2.sum(0)
    d1 = (d2 @ W2) * (a1 > 0)
    gW1 = d1.T @ X
    gb1 = d1.sum(0)
    g = np.concatenate([gW1.ravel(), gb1, gW2.ravel(), gb2, gW3, [gb3]])
    return loss, g


def adam_step(p, g, m, v, step, lr, b1=0.9, b2=0.999, eps=1e-8):
    """One Adam update (Kingma & Ba 2015, bias-corrected); returns p, m, v."""
    m = b1 * m + (1 - b1) * g
    v = b2 * v + (1 - b2) * g * g
    c1 = 1 - b1 ** step
    c2 = 1 - b2 ** step
    return p - lr * (m / c1) / (np.sqrt(v / c2) + eps), m, v
