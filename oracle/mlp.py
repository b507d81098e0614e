"""ORACLE — TEST INFRASTRUCTURE ONLY.

CPU reference of the warm-start network (24 -> 64 -> 64 -> 2, ReLU) and of its per-vertex
features, in FP64 numpy: the checker for the device's forward, gradients (backpropagation
written out by hand) and features.  The forward uses the BF16 rounding of the weights, as the
device does; `bf16` rounds FP32 values to the nearest BF16 (ties to even) by bit arithmetic.
The reference code base has no network; these restate the definitions in include/svm.h.
"""
from __future__ import annotations

import numpy as np

N_IN, N_H, N_OUT = 24, 64, 2
O_W1 = 0
O_B1 = O_W1 + N_H * N_IN
O_W2 = O_B1 + N_H
O_B2 = O_W2 + N_H * N_H
O_W3 = O_B2 + N_H
O_B3 = O_W3 + N_OUT * N_H
N_PARAMS = O_B3 + N_OUT


def bf16(w: np.ndarray) -> np.ndarray:
    """FP32 -> nearest BF16 (ties to even), returned as float64 values."""
    b = np.asarray(w, dtype=np.float32).view(np.uint32).astype(np.uint64)
    rounding = ((b >> 16) & 1) + 0x7FFF
    r = ((b + rounding) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def unpack(w):
    w = np.asarray(w, dtype=np.float64)
    W1 = w[O_W1:O_B1].reshape(N_H, N_IN)
    b1 = w[O_B1:O_W2]
    W2 = w[O_W2:O_B2].reshape(N_H, N_H)
    b2 = w[O_B2:O_W3]
    W3 = w[O_W3:O_B3].reshape(N_OUT, N_H)
    b3 = w[O_B3:N_PARAMS]
    return W1, b1, W2, b2, W3, b3


def forward(w, X):
    W1, b1, W2, b2, W3, b3 = unpack(w)
    a1 = X @ W1.T + b1
    h1 = np.maximum(a1, 0.0)
    a2 = h1 @ W2.T + b2
    h2 = np.maximum(a2, 0.0)
    return h2 @ W3.T + b3, (a1, h1, a2, h2)


def loss_and_grad(w, X, T):
    """mean_i |y_i - t_i|^2 and its gradient with respect to w (the parameters as given)."""
    X = np.asarray(X, dtype=np.float64)
    T = np.asarray(T, dtype=np.float64)
    n = X.shape[0]
    W1, b1, W2, b2, W3, b3 = unpack(w)
    y, (a1, h1, a2, h2) = forward(w, X)
    r = y - T
    loss = float(np.sum(r * r) / n)
    dy = 2.0 * r / n
    g = np.zeros(N_PARAMS)
    g[O_W3:O_B3] = (dy.T @ h2).reshape(-1)
    g[O_B3:N_PARAMS] = dy.sum(0)
    d2 = (dy @ W3) * (a2 > 0)
    g[O_W2:O_B2] = (d2.T @ h1).reshape(-1)
    g[O_B2:O_W3] = d2.sum(0)
    d1 = (d2 @ W2) * (a1 > 0)
    g[O_W1:O_B1] = (d1.T @ X).reshape(-1)
    g[O_B1:O_W2] = d1.sum(0)
    return loss, g


def features(pos, vnbr, vcell, cellpos, ap, pref, ring_counts, force):
    """The 24 features and (e1, e2) frames of every vertex (definition in include/svm.h)."""
    p = np.asarray(pos, dtype=np.float64)
    n = p / np.linalg.norm(p, axis=1, keepdims=True)
    d0 = p[vnbr[:, 0]] - p
    d0 = d0 - np.sum(d0 * n, axis=1, keepdims=True) * n
    e1 = d0 / np.linalg.norm(d0, axis=1, keepdims=True)
    e2 = np.cross(n, e1)
    X = np.zeros((p.shape[0], N_IN))
    for s in range(3):
        d = p[vnbr[:, s]] - p
        X[:, 2 * s] = np.sum(d * e1, 1)
        X[:, 2 * s + 1] = np.sum(d * e2, 1)
        c = vcell[:, s]
        dc = cellpos[c] - p
        X[:, 6 + 2 * s] = np.sum(dc * e1, 1)
        X[:, 7 + 2 * s] = np.sum(dc * e2, 1)
        X[:, 12 + 2 * s] = ap[c, 0] - pref[c, 0]
        X[:, 13 + 2 * s] = ap[c, 1] - pref[c, 1]
        X[:, 18 + s] = ring_counts[c].astype(np.float64) - 6.0
    X[:, 21] = np.sum(force * e1, 1)
    X[:, 22] = np.sum(force * e2, 1)
    X[:, 23] = np.linalg.norm(force, axis=1)
    return X, e1, e2
