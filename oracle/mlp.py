"""FP64 CPU restatement of the photon-chi MLP -- TEST INFRASTRUCTURE ONLY.

Same network and parameter layout as smilei_gb300/csrc/radiation.cu:
    h1 = tanh(W1 u + b1)      W1[H, 2]
    h2 = tanh(W2 h1 + b2)     W2[H, H]
    y  = W3 . h2 + b3         W3[H]
flat layout W1, b1, W2, b2, W3, b3; loss = mean (y - t)^2.  ``gradients``
is the analytic back-propagation; ``fd_gradients`` the central finite
differences used to check it.
"""
from __future__ import annotations

import numpy as np


def nparams(H: int) -> int:
    return H * H + 5 * H + 1


def unpack(p, H):
    p = np.asarray(p, dtype=np.float64)
    o = 0
    W1 = p[o:o + 2 * H].reshape(H, 2); o += 2 * H
    b1 = p[o:o + H]; o += H
    W2 = p[o:o + H * H].reshape(H, H); o += H * H
    b2 = p[o:o + H]; o += H
    W3 = p[o:o + H]; o += H
    b3 = p[o]
    return W1, b1, W2, b2, W3, b3


def forward(p, H, X):
    W1, b1, W2, b2, W3, b3 = unpack(p, H)
    h1 = np.tanh(X @ W1.T + b1)
    h2 = np.tanh(h1 @ W2.T + b2)
    return h2 @ W3 + b3, h1, h2


def loss(p, H, X, T):
    y, _, _ = forward(p, H, X)
    return float(np.mean((y - T) ** 2))


def gradients(p, H, X, T):
    W1, b1, W2, b2, W3, b3 = unpack(p, H)
    y, h1, h2 = forward(p, H, X)
    B = X.shape[0]
    d3 = 2.0 * (y - T) / B
    d2 = np.outer(d3, W3) * (1 - h2 ** 2)
    d1 = (d2 @ W2) * (1 - h1 ** 2)
    g = np.concatenate([(d1.T @ X).ravel(), d1.sum(0), (d2.T @ h1).ravel(), d2.sum(0), h2.T @ d3, [d3.sum()]])
    return g, float(np.mean((y - T) ** 2))


def fd_gradients(p, H, X, T, eps=1e-6, idx=None):
    p = np.asarray(p, dtype=np.float64).copy()
    idx = range(len(p)) if idx is None else idx
    out = {}
    for k in idx:
        old = p[k]
        p[k] = old + eps
        lp = loss(p, H, X, T)
        p[k] = old - eps
        lm = loss(p, H, X, T)
        p[k] = old
        out[k] = (lp - lm) / (2 * eps)
    return out
