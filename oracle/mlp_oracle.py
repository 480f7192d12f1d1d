"""CPU restatement (numpy, float64) of the learned endpoint proposal's forward and backward pass,
for gradient checks of the tensor-core kernels. TEST INFRASTRUCTURE ONLY.

The GPU computes GEMMs from BF16 operands with FP32 accumulation; this oracle rounds operands to
BF16 at the same points (inputs, weights, hidden activations, the backward operands) and
accumulates in float64, so the comparison isolates accumulation order and transcendental ulps.
Architecture: y = W3 g(W2 g(W1 x + b1) + b2) + b3, g = tanh-form GELU; loss = mean over samples
of the sum over outputs 0..5 of (y - t)^2 plus, for output 6, (y - t)^2 or (tau > 0) the pinball
loss bw * max(tau (t - y), (1 - tau) (y - t)).
"""
from __future__ import annotations

import numpy as np


def bf16(a):
    """Round-to-nearest-even to bfloat16, returned as float64."""
    a = np.asarray(a, np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


C = 0.7978845608


def gelu(x):
    return 0.5 * x * (1 + np.tanh(C * (x + 0.044715 * x ** 3)))


def gelu_grad(x):
    t = np.tanh(C * (x + 0.044715 * x ** 3))
    return 0.5 * (1 + t) + 0.5 * x * (1 - t * t) * C * (1 + 3 * 0.044715 * x * x)


def inputs(blocks: np.ndarray) -> np.ndarray:
    """(n, 64) RGBA8 -> (n, 48) RGB in [0, 1] (float32 division as on the device)."""
    px = blocks.reshape(-1, 16, 4)[:, :, :3].reshape(-1, 48).astype(np.float32)
    return (px * np.float32(1.0 / 255.0)).astype(np.float64)


def forward(p: dict, blocks: np.ndarray):
    x = bf16(inputs(blocks))
    pre1 = x @ bf16(p["W1"]).T + p["b1"]
    h1 = bf16(gelu(pre1))
    pre2 = h1 @ bf16(p["W2"]).T + p["b2"]
    h2 = bf16(gelu(pre2))
    y = h2 @ bf16(p["W3"]).T + p["b3"]
    return y, (x, pre1, h1, pre2, h2)


def gradients(p: dict, blocks: np.ndarray, targets: np.ndarray, tau: float = 0.0, bw: float = 1.0):
    y, (x, pre1, h1, pre2, h2) = forward(p, blocks)
    B = y.shape[0]
    d = np.zeros_like(y)
    d[:, :7] = y[:, :7] - targets[:, :7]
    dy = 2 * d / B
    if tau > 0:
        r = d[:, 6]
        loss = float(((d[:, :6] ** 2).sum() + (bw * np.where(r > 0, (1 - tau) * r, -tau * r)).sum()) / B)
        dy[:, 6] = bw * np.where(r > 0, 1 - tau, -tau) / B
    else:
        loss = float((d[:, :7] ** 2).sum() / B)
    g = {}
    g["W3"] = bf16(dy).T @ h2
    g["b3"] = dy.sum(0)
    dpre2 = (bf16(dy) @ bf16(p["W3"])) * gelu_grad(pre2)
    g["W2"] = bf16(dpre2).T @ h1
    g["b2"] = dpre2.sum(0)
    dpre1 = (bf16(dpre2) @ bf16(p["W2"])) * gelu_grad(pre1)
    g["W1"] = bf16(dpre1).T @ x
    g["b1"] = dpre1.sum(0)
    return loss, g
