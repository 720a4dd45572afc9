"""NumPy float64 reference of the pair-surrogate network — TEST INFRASTRUCTURE ONLY.

Forward, loss and gradients of the 1 -> 64 -> 64 -> 2 tanh network that the GPU
trains (parameter layout as ``dompap_gb300.mlp``): w1[64], b1[64], W2[64][64]
(row = output unit), b2[64], W3[2][64], b3[2]. The forward rounds W2 to
bf16 as the GPU does (``round_bf16``; w1 and W3 too when ``scalar_bf16``,
the library's DP_MLP_SCALAR_BF16 build); loss per sample is
``(y0 - t0)^2 + wf (y1 - t1)^2``, averaged over the batch. Used to check the
GPU gradients.
"""
from __future__ import annotations

import numpy as np

H = 64
NPARAM = 64 + 64 + 64 * 64 + 64 + 2 * 64 + 2


def round_bf16(a: np.ndarray) -> np.ndarray:
    """Round-to-nearest-even to bfloat16, returned as float64."""
    f = np.asarray(a, dtype=np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    lsb = (u >> 16) & 1
    u = (u + 0x7FFF + lsb) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def unpack(p: np.ndarray):
    p = np.asarray(p, dtype=np.float64)
    w1, b1 = p[0:64], p[64:128]
    w2 = p[128:128 + 4096].reshape(64, 64)
    b2 = p[4224:4288]
    w3 = p[4288:4416].reshape(2, 64)
    b3 = p[4416:4418]
    return w1, b1, w2, b2, w3, b3


def forward(p, x, scalar_bf16=False):
    """x: normalised inputs (B,). Returns y (B, 2) and the activations."""
    w1, b1, w2, b2, w3, b3 = unpack(p)
    w2q = round_bf16(w2)
    w1q, w3q = (round_bf16(w1), round_bf16(w3)) if scalar_bf16 else (w1, w3)
    h1 = np.tanh(np.outer(x, w1q) + b1)
    z2 = h1 @ w2q.T + b2
    h2 = np.tanh(z2)
    y = h2 @ w3q.T + b3
    return y, (h1, z2, h2, w2q, w3q)


def loss_and_grad(p, x, t, wf=1.0, scalar_bf16=False):
    """Mean loss and its gradient with respect to the fp32 masters (straight-through bf16 rounding)."""
    y, (h1, z2, h2, w2q, w3q) = forward(p, x, scalar_bf16)
    b = x.shape[0]
    e = y - t
    loss = float(np.mean(e[:, 0] ** 2 + wf * e[:, 1] ** 2))
    dy = np.stack([2 * e[:, 0], 2 * wf * e[:, 1]], axis=1) / b
    gw3 = dy.T @ h2
    gb3 = dy.sum(axis=0)
    dz2 = (dy @ w3q) * (1 - h2 ** 2)
    gw2 = dz2.T @ h1
    gb2 = dz2.sum(axis=0)
    dh1 = dz2 @ w2q
    dz1 = dh1 * (1 - h1 ** 2)
    gw1 = (dz1 * x[:, None]).sum(axis=0)
    gb1 = dz1.sum(axis=0)
    grad = np.concatenate([gw1, gb1, gw2.reshape(-1), gb2, gw3.reshape(-1), gb3])
    return loss, grad
