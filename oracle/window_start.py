"""FP64 restatement of the window-solve warm start — test infrastructure only.

The reference has no warm start (its iterate starts from the seed indicators,
``Backend/graph_link/kernels/ppr_kernel.cu:199-209``); this oracle states the
start's mathematics directly so the device kernels
(``page_rank_gb300/csrc/window_start.cu``) can be checked entry by entry:

* :func:`window_blocks` — the dense diagonal window blocks ``I - alpha A_w``;
* :func:`near_field` — ``(1 - alpha) (y_0 + ... + y_L)`` with
  ``y_0 = B^-1 v`` and ``y_k = B^-1 (alpha M y_{k-1})`` (``B`` the block
  diagonal of the window blocks, ``M`` the edges that leave their window),
  the inverses taken with ``numpy.linalg.inv``;
* :func:`window_start` — the near field plus its missing mass along a shape;
* :func:`cold_residual` — ``||P(v) - v||_1`` of one power step from the
  teleport vector, with dangling mass returned through ``v``.

As ``L`` grows the near field converges to the exact PPR vector of a graph
without dangling nodes (the series is a block-Jacobi splitting of
``(I - alpha A) x = (1 - alpha) v``); the CPU tests pin the oracle on that.
"""
from __future__ import annotations

import numpy as np
import scipy.sparse as sp

WINDOW = 64


def window_blocks(A: sp.csr_matrix, alpha: float) -> np.ndarray:
    """[ceil(n / 64), 64, 64] FP64 blocks I - alpha A_w (identity past n)."""
    A = sp.csr_matrix(A)
    n = A.shape[0]
    W = -(-n // WINDOW)
    B = np.tile(np.eye(WINDOW), (W, 1, 1))
    rows = np.repeat(np.arange(n), np.diff(A.indptr))
    cols = A.indices
    keep = (rows // WINDOW) == (cols // WINDOW)
    np.add.at(B, (rows[keep] // WINDOW, rows[keep] % WINDOW, cols[keep] % WINDOW),
              -alpha * A.data[keep].astype(np.float64))
    return B


def off_window(A: sp.csr_matrix) -> sp.csr_matrix:
    """The entries of A whose row and column lie in different windows."""
    A = sp.csr_matrix(A)
    n = A.shape[0]
    rows = np.repeat(np.arange(n), np.diff(A.indptr))
    keep = (rows // WINDOW) != (A.indices // WINDOW)
    return sp.csr_matrix((A.data[keep].astype(np.float64), (rows[keep], A.indices[keep])), shape=A.shape)


def apply_inverse(inv: np.ndarray, T: np.ndarray) -> np.ndarray:
    """B^-1 T window by window (T [n, K])."""
    n, K = T.shape
    W = inv.shape[0]
    pad = np.zeros((W * WINDOW, K))
    pad[:n] = T
    out = np.einsum("wrq,wqk->wrk", inv, pad.reshape(W, WINDOW, K)).reshape(W * WINDOW, K)
    return out[:n]


def near_field(A: sp.csr_matrix, V: np.ndarray, alpha: float, leaves: int, inv: np.ndarray | None = None):
    if inv is None:
        inv = np.linalg.inv(window_blocks(A, alpha))
    M = off_window(A)
    y = apply_inverse(inv, np.asarray(V, np.float64))
    nf = (1.0 - alpha) * y
    for _ in range(leaves):
        y = apply_inverse(inv, alpha * (M @ y))
        nf += (1.0 - alpha) * y
    return nf


def window_start(A: sp.csr_matrix, V: np.ndarray, alpha: float, leaves: int, shape: np.ndarray) -> np.ndarray:
    nf = near_field(A, V, alpha, leaves)
    missing = np.maximum(0.0, 1.0 - nf.sum(axis=0))
    return nf + np.asarray(shape, np.float64)[:, None] * missing[None, :]


def cold_residual(A: sp.csr_matrix, V: np.ndarray, alpha: float, dangling: np.ndarray | None = None) -> np.ndarray:
    """||P(v) - v||_1 per column, P(x) = alpha A x + ((1 - alpha) + alpha d(x)) v."""
    V = np.asarray(V, np.float64)
    d = V[np.asarray(dangling, bool)].sum(axis=0) if dangling is not None else np.zeros(V.shape[1])
    P = alpha * (A.astype(np.float64) @ V) + ((1.0 - alpha) + alpha * d)[None, :] * V
    return np.abs(P - V).sum(axis=0)
