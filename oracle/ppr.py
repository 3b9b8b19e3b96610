"""FP64 Personalized-PageRank oracles — test infrastructure only.

* :func:`power_iteration_fp64` restates the reference power iteration
  (``Backend/graph_link/graph_link/__init__.py:242-271``) with the update of
  ``ppr_update_normalized_kernel`` (``kernels/ppr_kernel.cu:130-168``):
  ``X <- alpha * A X + (1 - alpha) * V`` and the stop rule "largest per-column
  L1 change < tol", or, with ``dangling`` set, the missing-mass update of
  ``batched_ppr_update_kernel`` (``kernels/ppr_kernel.cu:57-97``) generalised to
  a teleport matrix V: the mass of dangling columns returns through V.
* :func:`direct_solve_fp64` solves the fixed point exactly for small n:
  ``(I - alpha * (A + V d^T)) x = (1 - alpha) v`` per column.
* :func:`teleport_matrix` builds V from per-column seed sets (uniform weights).
"""
from __future__ import annotations

import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla


def teleport_matrix(n: int, seed_sets) -> np.ndarray:
    V = np.zeros((n, len(seed_sets)), dtype=np.float64)
    for k, seeds in enumerate(seed_sets):
        seeds = np.asarray(seeds, dtype=np.int64)
        np.add.at(V[:, k], seeds, 1.0 / len(seeds))
    return V


def dangling_mask(A: sp.csr_matrix) -> np.ndarray:
    """Columns without any stored entry."""
    present = np.zeros(A.shape[1], dtype=bool)
    present[A.indices] = True
    return ~present


def power_iteration_fp64(A: sp.csr_matrix, V: np.ndarray, alpha: float, max_iterations: int,
                         tol: float, dangling: np.ndarray | None = None, x0: np.ndarray | None = None):
    """Returns (X, iterations, converged, history)."""
    A64 = A.astype(np.float64).tocsr()
    X = V.copy() if x0 is None else np.asarray(x0, dtype=np.float64).copy()
    history = []
    for t in range(max_iterations):
        Y = A64 @ X
        Xn = alpha * Y + (1.0 - alpha) * V
        if dangling is not None:
            d = X[dangling].sum(axis=0)
            Xn += alpha * d[None, :] * V
        err = np.abs(Xn - X).sum(axis=0)
        X = Xn
        history.append(float(err.max()))
        if err.max() < tol:
            return X, t + 1, True, history
    return X, max_iterations, False, history


def direct_solve_fp64(A: sp.csr_matrix, V: np.ndarray, alpha: float,
                      dangling: np.ndarray | None = None) -> np.ndarray:
    """Fixed point of x = alpha (A + v d^T) x + (1 - alpha) v for every column
    v of V (d = dangling indicator): one sparse LU of I - alpha A, and the
    rank-one dangling term per column by Sherman-Morrison."""
    n = A.shape[0]
    M = (sp.identity(n, format="csc") - alpha * A.astype(np.float64).tocsc()).tocsc()
    lu = spla.splu(M)
    V = np.asarray(V, dtype=np.float64)
    Y = lu.solve((1.0 - alpha) * V)
    if dangling is None or not np.any(dangling):
        return Y
    d = np.asarray(dangling, dtype=bool)
    Z = lu.solve(alpha * V)
    dy = Y[d].sum(axis=0)
    dz = Z[d].sum(axis=0)
    return Y + Z * (dy / (1.0 - dz))[None, :]
