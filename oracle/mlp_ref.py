"""TEST INFRASTRUCTURE ONLY — FP64 reference of the surrogate network
(48 -> 64 -> 64 -> 2, ReLU) used to check the tensor-core kernels.

`bf16=True` rounds to BF16 exactly where the GPU path does (inputs, weights,
hidden activations, and the backward operands dY, dZ2, dZ1 of the tensor-core
GEMMs) and accumulates in FP64, so only summation order separates it from the
GPU.  `bf16=False` is the plain FP64 network.

Parameter layout: W1[64][48], b1[64], W2[64][64], b2[64], W3[2][64], b3[2].
Loss: L = 1/(2n) sum_points sum_outputs (y - t)^2.
"""
from __future__ import annotations

import numpy as np

N_PARAMS = 64 * 48 + 64 + 64 * 64 + 64 + 2 * 64 + 2


def bf16(a):
    """Round float values to BF16 (nearest even), returned as float64."""
    f = np.asarray(a, np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def unpack(p):
    p = np.asarray(p, np.float64)
    o = 0
    W1 = p[o:o + 64 * 48].reshape(64, 48); o += 64 * 48
    b1 = p[o:o + 64]; o += 64
    W2 = p[o:o + 64 * 64].reshape(64, 64); o += 64 * 64
    b2 = p[o:o + 64]; o += 64
    W3 = p[o:o + 128].reshape(2, 64); o += 128
    b3 = p[o:o + 2]
    return W1, b1, W2, b2, W3, b3


def pack(W1, b1, W2, b2, W3, b3):
    return np.concatenate([W1.ravel(), b1, W2.ravel(), b2, W3.ravel(), b3])


def forward(p, X, bf=True):
    r = bf16 if bf else (lambda a: np.asarray(a, np.float64))
    W1, b1, W2, b2, W3, b3 = unpack(p)
    Xb = r(X)
    Z1 = Xb @ r(W1).T + b1
    H1 = r(np.maximum(Z1, 0.0))
    Z2 = H1 @ r(W2).T + b2
    H2 = r(np.maximum(Z2, 0.0))
    Y = H2 @ r(W3).T + b3
    return Y, (Xb, Z1, H1, Z2, H2)


def gradients(p, X, T, bf=True):
    r = bf16 if bf else (lambda a: np.asarray(a, np.float64))
    W1, b1, W2, b2, W3, b3 = unpack(p)
    n = len(X)
    Y, (Xb, Z1, H1, Z2, H2) = forward(p, X, bf)
    E = Y - np.asarray(T, np.float64)
    loss = 0.5 * float((E * E).sum()) / n
    dY = E / n
    dYb = r(dY)
    dZ2 = (dYb @ r(W3)) * (Z2 > 0)
    dZ2b = r(dZ2)
    dZ1 = (dZ2b @ r(W2)) * (Z1 > 0)
    dZ1b = r(dZ1)
    dW3 = dY.T @ H2            # CUDA-core reduction: FP32 dY against BF16 H2
    dW2 = dZ2b.T @ H1
    dW1 = dZ1b.T @ Xb
    return pack(dW1, dZ1b.sum(0), dW2, dZ2b.sum(0), dW3, dY.sum(0)), loss
