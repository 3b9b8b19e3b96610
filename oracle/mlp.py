"""FP64 oracle of the warm-start MLP — test infrastructure only.

Forward / backward of the 2-layer network the engine trains on the GPU
(f_in -> 128 ReLU -> 1, loss sum_e (y_e - t_e)^2 / 2), in float64 numpy,
with the BF16 weight rounding applied to W1 and w2 exactly as the device
copies hold them.  Used to check the device gradients.
"""
from __future__ import annotations

import numpy as np


def bf16_round(w: np.ndarray) -> np.ndarray:
    """Round FP32 values to BF16 (nearest even) and widen back to FP32."""
    u = np.asarray(w, dtype=np.float32).view(np.uint32).astype(np.uint64)
    lsb = (u >> 16) & 1
    r = ((u + 0x7FFF + lsb) >> 16) << 16
    return r.astype(np.uint32).view(np.float32)


def bf16_bits(w: np.ndarray) -> np.ndarray:
    return (bf16_round(w).view(np.uint32) >> 16).astype(np.uint16)


def forward(X, W1, b1, w2, b2):
    H = np.maximum(X.astype(np.float64) @ W1.astype(np.float64).T + b1.astype(np.float64), 0.0)
    return H @ w2.astype(np.float64) + float(b2), H


def backward(X, target, W1, b1, w2, b2):
    """Returns (grad [W1 | b1 | w2 | b2], loss)."""
    X64 = X.astype(np.float64)
    y, H = forward(X, W1, b1, w2, b2)
    dy = y - target.astype(np.float64)
    loss = 0.5 * float(dy @ dy)
    g = (H > 0) * (dy[:, None] * w2.astype(np.float64)[None, :])
    dW1 = g.T @ X64
    db1 = g.sum(axis=0)
    dw2 = H.T @ dy
    db2 = dy.sum()
    return np.concatenate([dW1.ravel(), db1, dw2, [db2]]), loss
