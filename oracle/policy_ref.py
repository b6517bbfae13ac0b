"""FP64 CPU restatement of the round-policy MLP (test infrastructure only).

The learned policy has no counterpart in the reference, so this oracle is the
mathematics of the model itself: x = (clamp(f, lo, hi) - mean) * scale, h1 = relu(W1 x + b1),
h2 = relu(W2 h1 + b2), out = W3 h2 + b3, masked mean squared error against
log2 round times, and its exact gradient by backpropagation.  It checks the
GPU forward/backward kernels (grd_policy_grad, grd_policy_predict) and the
fused per-round inference.  Only tests may import it.
"""
from __future__ import annotations

import numpy as np


def forward(p: dict, x: np.ndarray):
    """p: float64 arrays (mean, scale, w1 [64,8], b1, w2 [64,64], b2, w3 [4,64],
    b3).  Returns (out [n,4], cache)."""
    f = np.asarray(x, dtype=np.float64)
    if "lo" in p:
        f = np.clip(f, p["lo"], p["hi"])
    xs = (f - p["mean"]) * p["scale"]
    a1 = xs @ p["w1"].T + p["b1"]
    h1 = np.maximum(a1, 0.0)
    a2 = h1 @ p["w2"].T + p["b2"]
    h2 = np.maximum(a2, 0.0)
    out = h2 @ p["w3"].T + p["b3"]
    return out, (xs, a1, h1, a2, h2)


def loss_and_grad(p: dict, x: np.ndarray, y: np.ndarray, mask: np.ndarray):
    """Masked MSE over measured targets and the gradient, flattened in the
    order w1, b1, w2, b2, w3, b3."""
    out, (xs, a1, h1, a2, h2) = forward(p, x)
    m = np.asarray(mask, dtype=np.float64)
    cnt = m.sum()
    e = (out - np.asarray(y, dtype=np.float64)) * m
    loss = float((e * e).sum() / cnt)
    d_out = 2.0 * e / cnt
    g_w3 = d_out.T @ h2
    g_b3 = d_out.sum(axis=0)
    d_h2 = (d_out @ p["w3"]) * (a2 > 0)
    g_w2 = d_h2.T @ h1
    g_b2 = d_h2.sum(axis=0)
    d_h1 = (d_h2 @ p["w2"]) * (a1 > 0)
    g_w1 = d_h1.T @ xs
    g_b1 = d_h1.sum(axis=0)
    flat = np.concatenate([g_w1.ravel(), g_b1, g_w2.ravel(), g_b2, g_w3.ravel(), g_b3])
    return loss, flat


def choose(out: np.ndarray, allowed: int = 0xF) -> np.ndarray:
    """argmin over the allowed modes (bit m = mode m)."""
    o = np.where([(allowed >> m) & 1 for m in range(out.shape[1])], out, np.inf)
    return np.argmin(o, axis=1).astype(np.int32)
