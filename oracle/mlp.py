"""CPU restatement of the accelerator MLP (TEST INFRASTRUCTURE ONLY).

FP64 forward and backward of the 8 -> 128 -> 128 -> 128 -> 1 ReLU network in
the flat parameter layout of include/bte_cuda.h, with BF16 rounding applied
where the GPU kernels round (inputs, weights, post-ReLU activations and the
back-propagated pre-activation gradients), so that the GPU's gradient can be
checked element by element.  Used by tests only.
"""
from __future__ import annotations

import numpy as np

IN, H = 8, 128
OFF_W1 = 0
OFF_B1 = OFF_W1 + IN * H
OFF_W2 = OFF_B1 + H
OFF_B2 = OFF_W2 + H * H
OFF_W3 = OFF_B2 + H
OFF_B3 = OFF_W3 + H * H
OFF_W4 = OFF_B3 + H
OFF_B4 = OFF_W4 + H
NPARAM = OFF_B4 + 1


def bf16(x):
    """Round to bfloat16 (round to nearest even), returned as float64."""
    u = np.ascontiguousarray(x, dtype=np.float32).view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def unpack(p):
    p = np.asarray(p, np.float64)
    return (p[OFF_W1:OFF_B1].reshape(IN, H), p[OFF_B1:OFF_W2], p[OFF_W2:OFF_B2].reshape(H, H), p[OFF_B2:OFF_W3],
            p[OFF_W3:OFF_B3].reshape(H, H), p[OFF_B3:OFF_W4], p[OFF_W4:OFF_B4], p[OFF_B4])


def forward(p, X):
    W1, b1, W2, b2, W3, b3, W4, b4 = unpack(p)
    x = bf16(X)
    h1 = bf16(np.maximum(x @ bf16(W1) + b1, 0))
    h2 = bf16(np.maximum(h1 @ bf16(W2) + b2, 0))
    h3 = bf16(np.maximum(h2 @ bf16(W3) + b3, 0))
    y = h3 @ bf16(W4) + b4
    return y, (x, h1, h2, h3)


def loss_grad(p, X, Y):
    """0.5 mean (y - Y)^2 and its gradient (flat layout)."""
    W1, b1, W2, b2, W3, b3, W4, b4 = unpack(p)
    y, (x, h1, h2, h3) = forward(p, X)
    M = len(Y)
    d = y - np.asarray(Y, np.float64)
    loss = 0.5 * np.mean(d * d)
    dy = (d / M).astype(np.float32).astype(np.float64)
    dz3 = bf16(np.outer(dy, W4) * (h3 > 0))
    dz2 = bf16((dz3 @ bf16(W3).T) * (h2 > 0))
    dz1 = bf16((dz2 @ bf16(W2).T) * (h1 > 0))
    g = np.zeros(NPARAM)
    g[OFF_W1:OFF_B1] = (x.T @ dz1).ravel()
    g[OFF_B1:OFF_W2] = dz1.sum(0)
    g[OFF_W2:OFF_B2] = (h1.T @ dz2).ravel()
    g[OFF_B2:OFF_W3] = dz2.sum(0)
    g[OFF_W3:OFF_B3] = (h2.T @ dz3).ravel()
    g[OFF_B3:OFF_W4] = dz3.sum(0)
    g[OFF_W4:OFF_B4] = h3.T @ dy
    g[OFF_B4] = dy.sum()
    return loss, g
