"""FP64 SpMM oracle — test infrastructure only.

Two independent statements of Y = A X:
* :func:`spmm_csr_fp64` — scipy CSR product in float64 (what the reference's
  accuracy test compares against, ``Tests/test_spmm.py:46``);
* :func:`spmm_pbr_fp64` — the reference's CPU SpMM semantics over PBR arrays
  (``Backend/graph_link/pbr_matrix/pbr_matrix.cpp:17-68``): block values pair
  with set bits in row-major bit order, then the CSR remainder is added.
"""
from __future__ import annotations

import numpy as np
import scipy.sparse as sp

from . import expand_pbr_coo


def spmm_csr_fp64(A: sp.csr_matrix, X: np.ndarray) -> np.ndarray:
    """A @ X in float64; X is [cols, F] or [batch, cols, F]."""
    A64 = A.astype(np.float64)
    X = np.asarray(X, dtype=np.float64)
    if X.ndim == 2:
        return np.asarray(A64 @ X)
    return np.stack([np.asarray(A64 @ X[b]) for b in range(X.shape[0])])


def spmm_pbr_fp64(pbr: dict, X: np.ndarray) -> np.ndarray:
    """Reference CPU SpMM semantics on PBR arrays, in float64."""
    r, c, v = expand_pbr_coo(pbr)
    A = sp.csr_matrix((v.astype(np.float64), (r, c)), shape=(pbr["rows"], pbr["cols"]))
    return spmm_csr_fp64(A, X)


def spmm_csr_fp32(A: sp.csr_matrix, X: np.ndarray) -> np.ndarray:
    """A @ X in float32 with scipy — the CPU SpMM the reference's own tests
    run (``Tests/test_spmm.py:46``); used as the timed CPU baseline."""
    return np.asarray(A @ X)
