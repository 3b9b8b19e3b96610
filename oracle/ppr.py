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
* :func:`refine_fp64` continues the FP64 power iteration from a given start
  until every column carries a certified bound on its L1 distance to the
  exact fixed point; the large-graph parity tests compare the GPU's columns
  with these references.  Row-split over host threads (scipy's sparse
  products release the GIL).
"""
from __future__ import annotations

import os
from concurrent.futures import ThreadPoolExecutor

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


class RowSplitMatrix:
    """A CSR matrix cut into row ranges so ``A @ X`` runs on several host
    threads (test infrastructure for graphs of millions of nodes)."""

    def __init__(self, A: sp.csr_matrix, threads: int | None = None):
        A = A.tocsr()
        self.shape = A.shape
        self.threads = max(1, int(threads or os.cpu_count() or 1))
        bounds = np.searchsorted(A.indptr, np.linspace(0, A.nnz, self.threads + 1)).clip(0, A.shape[0])
        bounds[0], bounds[-1] = 0, A.shape[0]
        self.bounds = np.maximum.accumulate(bounds)
        self.parts = [A[self.bounds[i]:self.bounds[i + 1]] for i in range(self.threads)]
        self.pool = ThreadPoolExecutor(self.threads)

    def __matmul__(self, X: np.ndarray) -> np.ndarray:
        out = np.empty((self.shape[0],) + X.shape[1:], dtype=np.result_type(self.parts[0].dtype, X.dtype))

        def part(i):
            out[self.bounds[i]:self.bounds[i + 1]] = self.parts[i] @ X

        list(self.pool.map(part, range(self.threads)))
        return out

    def close(self):
        self.pool.shutdown()


def ppr_apply_fp64(A64, X: np.ndarray, V: np.ndarray, alpha: float, dangling: np.ndarray | None = None,
                   dangling_uniform: bool = False) -> np.ndarray:
    """One FP64 application of the PPR map T(X) = alpha (A X + dangling
    term) + (1 - alpha) V: the dangling mass of each column returns through
    its teleport vector (``kernels/ppr_kernel.cu:57-97``) or, with
    ``dangling_uniform``, spreads as 1/n over all nodes (the fixed point of
    the reference's dense ``normalize_transition_matrix``,
    ``graph_link/__init__.py:200-206``)."""
    Y = alpha * (A64 @ X) + (1.0 - alpha) * V
    if dangling is not None and np.any(dangling):
        d = X[dangling].sum(axis=0)
        if dangling_uniform:
            Y += (alpha * d / X.shape[0])[None, :]
        else:
            Y += alpha * d[None, :] * V
    return Y


def refine_fp64(A: sp.csr_matrix, X0: np.ndarray, V: np.ndarray, alpha: float,
                dangling: np.ndarray | None = None, bound: float = 1e-10, max_iterations: int = 2000,
                threads: int | None = None, dangling_uniform: bool = False):
    """FP64 power iteration from X0 until every column's distance to the exact
    fixed point is certified below ``bound``.

    T is an alpha-contraction in L1 (A plus the dangling term is column
    stochastic), so after an update x_t = T x_{t-1} the distance obeys
    ||x_t - x*||_1 <= alpha / (1 - alpha) * ||x_t - x_{t-1}||_1.  Returns
    (X, per-column certified bounds, iterations)."""
    M = RowSplitMatrix(A.astype(np.float64), threads)
    try:
        X = np.asarray(X0, dtype=np.float64).copy()
        V = np.asarray(V, dtype=np.float64)
        cert = np.full(X.shape[1], np.inf)
        for t in range(max_iterations):
            Xn = ppr_apply_fp64(M, X, V, alpha, dangling, dangling_uniform)
            cert = alpha / (1.0 - alpha) * np.abs(Xn - X).sum(axis=0)
            X = Xn
            if cert.max() < bound:
                return X, cert, t + 1
        return X, cert, max_iterations
    finally:
        M.close()
