"""FP64 restatement of the surrogate MLP (forward, MSE loss, backward) with
bf16 rounding at the points where the GPU stores bf16 (inputs, weights,
hidden activations, activation gradients). There is no reference
counterpart; this is the oracle the GPU gradients are checked against.

TEST INFRASTRUCTURE ONLY.
"""
from __future__ import annotations

import math

import numpy as np
from scipy.special import erf


def bf16(a: np.ndarray) -> np.ndarray:
    """Round to the nearest bfloat16 (ties to even), returned as float64."""
    f = np.ascontiguousarray(a, dtype=np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    lsb = (u >> 16) & 1
    u = ((u + 0x7FFF + lsb) >> 16) << 16
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def gelu(z):
    return 0.5 * z * (1.0 + erf(z / math.sqrt(2.0)))


def gelu_d(z):
    return 0.5 * (1.0 + erf(z / math.sqrt(2.0))) + z * np.exp(-0.5 * z * z) / math.sqrt(2 * math.pi)


def forward(x, ws, bs):
    """x [B][n_in]; ws[l] [out][in] fp32 masters; returns (y, Z list, H list)."""
    h = bf16(x)
    H, Z = [h], [None]
    L = len(ws)
    for l in range(L - 1):
        z = h @ bf16(ws[l]).T + bs[l]
        Z.append(z)
        h = bf16(gelu(z))
        H.append(h)
    y = h @ bf16(ws[-1]).T[:, 0] + bs[-1][0]
    return y, Z, H


def loss_and_grads(x, t, ws, bs):
    """MSE loss and the gradients of every weight and bias."""
    y, Z, H = forward(x, ws, bs)
    B = x.shape[0]
    dy = 2.0 * (y - t) / B
    L = len(ws)
    gw, gb = [None] * L, [None] * L
    gw[L - 1] = (dy[:, None] * H[L - 1]).sum(0)[None, :]
    gb[L - 1] = np.array([dy.sum()])
    dz = bf16(dy[:, None] * bf16(ws[L - 1])[0][None, :] * gelu_d(Z[L - 1]))
    for l in range(L - 2, -1, -1):
        gw[l] = dz.T @ H[l]
        gb[l] = dz.sum(0)
        if l > 0:
            dz = bf16((dz @ bf16(ws[l])) * gelu_d(Z[l]))
    return float(np.mean((y - t) ** 2)), gw, gb
