"""TEST INFRASTRUCTURE: FP64 numpy restatement of the learned troubled-cell sensor (an MLP
64 -> 64 -> 64 -> 1 with GELU hidden layers and a sigmoid output scaled to [0, alpha_max]) and of
its mean-squared-error gradient, the checker for the CUDA forward / backward / Adam kernels.
Parameter layout: W1[64][64], b1[64], W2[64][64], b2[64], w3[64], b3 (row-major, out x in).
The learned sensor has no counterpart in the reference; nothing here is a restatement of it.
"""
from __future__ import annotations

import math

import numpy as np

N_IN = 64
N_HID = 64
N_PARAMS = N_HID * N_IN + N_HID + N_HID * N_HID + N_HID + N_HID + 1

_erf = np.vectorize(math.erf, otypes=[np.float64])


def unpack(p):
    p = np.asarray(p, dtype=np.float64)
    o = 0
    W1 = p[o:o + N_HID * N_IN].reshape(N_HID, N_IN); o += N_HID * N_IN
    b1 = p[o:o + N_HID]; o += N_HID
    W2 = p[o:o + N_HID * N_HID].reshape(N_HID, N_HID); o += N_HID * N_HID
    b2 = p[o:o + N_HID]; o += N_HID
    w3 = p[o:o + N_HID]; o += N_HID
    b3 = p[o]
    return W1, b1, W2, b2, w3, b3


def gelu(x):
    return 0.5 * x * (1.0 + _erf(x / math.sqrt(2.0)))


def gelu_d(x):
    return 0.5 * (1.0 + _erf(x / math.sqrt(2.0))) + x * np.exp(-0.5 * x * x) / math.sqrt(2.0 * math.pi)


def init_params(seed: int = 0) -> np.ndarray:
    """He-style initialisation, output bias set so the initial alpha is small."""
    rng = np.random.default_rng(seed)
    W1 = rng.normal(0, math.sqrt(2.0 / N_IN), (N_HID, N_IN))
    W2 = rng.normal(0, math.sqrt(2.0 / N_HID), (N_HID, N_HID))
    w3 = rng.normal(0, math.sqrt(1.0 / N_HID), N_HID)
    p = np.concatenate([W1.ravel(), np.zeros(N_HID), W2.ravel(), np.zeros(N_HID), w3, [-4.0]])
    return p.astype(np.float32)


def forward(p, x, alpha_max=0.5):
    W1, b1, W2, b2, w3, b3 = unpack(p)
    x = np.asarray(x, dtype=np.float64)
    a1 = x @ W1.T + b1
    h1 = gelu(a1)
    a2 = h1 @ W2.T + b2
    h2 = gelu(a2)
    z = h2 @ w3 + b3
    s = 1.0 / (1.0 + np.exp(-z))
    return alpha_max * s, (a1, h1, a2, h2, s)


def loss_grad(p, x, y, alpha_max=0.5):
    """Mean squared error of alpha against y and its gradient (same layout as p)."""
    W1, b1, W2, b2, w3, b3 = unpack(p)
    x = np.asarray(x, dtype=np.float64)
    y = np.asarray(y, dtype=np.float64)
    B = x.shape[0]
    alpha, (a1, h1, a2, h2, s) = forward(p, x, alpha_max)
    d = alpha - y
    loss = float(np.mean(d * d))
    dz = (2.0 / B) * d * alpha_max * s * (1 - s)
    gw3 = h2.T @ dz
    gb3 = dz.sum()
    da2 = np.outer(dz, w3) * gelu_d(a2)
    gW2 = da2.T @ h1
    gb2 = da2.sum(0)
    da1 = (da2 @ W2) * gelu_d(a1)
    gW1 = da1.T @ x
    gb1 = da1.sum(0)
    g = np.concatenate([gW1.ravel(), gb1, gW2.ravel(), gb2, gw3, [gb3]])
    return loss, g
