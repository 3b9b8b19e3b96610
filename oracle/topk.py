"""Top-k of matrix columns — test infrastructure only.

Restates the selection ``gl_topk_columns`` promises, which the reference
leaves to its frontend (it returns all N ranks, ``Backend/server/app.py:146-158``):
per column the k largest values by the order of their bit patterns mapped
to unsigned keys (negative floats: all bits flipped; non-negative: sign bit
set — IEEE order, with +0.0 above -0.0), ties to the lowest row.
"""
from __future__ import annotations

import numpy as np


def order_keys(x: np.ndarray) -> np.ndarray:
    u = np.ascontiguousarray(x, dtype=np.float32).view(np.uint32)
    return np.where(u >> 31, ~u, u | np.uint32(0x80000000)).astype(np.uint32)


def topk_columns(X: np.ndarray, k: int, columns=None):
    """(values [C, k] float32, rows [C, k] int32); -inf / -1 past the rows."""
    X = np.asarray(X, dtype=np.float32)
    cols = np.arange(X.shape[1]) if columns is None else np.asarray(columns)
    n = X.shape[0]
    vals = np.full((len(cols), k), -np.inf, dtype=np.float32)
    rows = np.full((len(cols), k), -1, dtype=np.int32)
    for i, c in enumerate(cols):
        key = order_keys(X[:, c])
        order = np.lexsort((np.arange(n), ~key))[:k]    # key descending, row ascending
        vals[i, :order.size] = X[order, c]
        rows[i, :order.size] = order
    return vals, rows
