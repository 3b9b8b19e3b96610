"""Transition matrices and the edge-list request path of the HTTP service.

:func:`normalize_columns` is the reference's ``normalize_transition_matrix``
(``graph_link/__init__.py:184-207``) without its dense step: columns are
divided by their sum in the same FP32 arithmetic, but a dangling column
(sum 0) stays empty and is reported in a mask instead of being filled with
N values of 1/N.  The fused PPR step then redistributes the dangling mass in
its epilogue (uniformly — the reference's semantics — or to the teleport
vector), which reaches the same fixed point with O(nnz) instead of
O(nnz + N * #dangling) storage.
"""
from __future__ import annotations

import numpy as np
import scipy.sparse as sp
import torch

from . import native


def normalize_columns(A_csr: sp.csr_matrix) -> tuple[sp.csr_matrix, np.ndarray]:
    """(column-normalized FP32 CSR, dangling mask)."""
    A = A_csr.tocsc().astype(np.float32)
    col_sums = np.asarray(A.sum(axis=0), dtype=np.float32).ravel()
    inv = np.zeros_like(col_sums)
    np.divide(1.0, col_sums, out=inv, where=col_sums > 0)
    A_norm = sp.csr_matrix(A.multiply(inv).tocsr())
    A_norm.sum_duplicates()
    return A_norm, col_sums == 0


def edge_list_csr(n: int, src_idx: np.ndarray, dst_idx: np.ndarray, weight: np.ndarray) -> sp.csr_matrix:
    """A[target, source] = weight, duplicate edges summed (``app.py:111-131``)."""
    return sp.csr_matrix((weight.astype(np.float32), (dst_idx.astype(np.int64), src_idx.astype(np.int64))),
                         shape=(n, n))


def solve_edge_list_request(ids, index_of, src, dst, weight, seed_idx, alpha, max_iter, tol,
                            block_size: int = 2, min_nnz: int = 2) -> dict:
    """The body of ``POST /api/ppr`` after validation (``app.py:102-152``)."""
    from .graph_link import csr_to_pbr, get_pbr_gpu_meta
    from .ppr import PprRun, teleport_from_seed_sets

    n = len(ids)
    in_deg = {nid: 0.0 for nid in ids}
    out_deg = {nid: 0.0 for nid in ids}
    for s, t in zip(src, dst):
        if s in out_deg:
            out_deg[s] += 1.0
        if t in in_deg:
            in_deg[t] += 1.0
    si = np.fromiter((index_of.get(s, -1) for s in src), dtype=np.int64, count=len(src))
    ti = np.fromiter((index_of.get(t, -1) for t in dst), dtype=np.int64, count=len(dst))
    w = np.asarray(weight, dtype=np.float64)
    ok = (si >= 0) & (ti >= 0) & np.isfinite(w) & (w > 0)
    A = edge_list_csr(n, si[ok], ti[ok], w[ok])
    A_norm, dangling = normalize_columns(A)

    dev = torch.device("cuda", torch.cuda.current_device())
    pbr = csr_to_pbr(A_norm, block_size, block_size, min_nnz).to(dev)
    meta = get_pbr_gpu_meta(pbr)
    K = len(seed_idx)
    seeds = torch.tensor(seed_idx, dtype=torch.int32, device=dev)
    tp = teleport_from_seed_sets(torch.arange(K + 1, dtype=torch.int32, device=dev), seeds, n, block_size)
    from .engine import _bitmap_from_mask
    dbits = _bitmap_from_mask(dangling, dev)
    run = PprRun(meta, n, n, block_size, block_size, tp, alpha, max_iter, tol, native.GL_PPR_STOP_ALL,
                 dbits, native.GL_DANGLING_UNIFORM)
    res = run.run(chunk=8)
    r = res.X.to(torch.float64).mean(dim=1)
    total = float(r.sum().item())
    if total > 0:
        r = r / total
    return {"ranks": r.cpu().numpy(), "iterations": res.iterations, "converged": res.converged,
            "history": res.history, "in_deg": in_deg, "out_deg": out_deg}
