"""Transition matrices and the edge-list request path of the HTTP service.

:func:`normalize_columns` is the reference's ``normalize_transition_matrix``
(``graph_link/__init__.py:184-207``) without its dense step: columns are
divided by their sum in the same FP32 arithmetic, but a dangling column
(sum 0) stays empty and is reported in a mask instead of being filled with
N values of 1/N.  The fused PPR step then redistributes the dangling mass in
its epilogue (uniformly — the reference's semantics — or to the teleport
vector), which reaches the same fixed point with O(nnz) instead of
O(nnz + N * #dangling) storage.

:func:`device_transition` does the same from an edge list on the GPU
(``gl_edges_to_transition``), and :func:`solve_edge_list_request` serves
``POST /api/ppr`` with it, keeping recently used request graphs resident.
"""
from __future__ import annotations

import hashlib
import threading
from collections import OrderedDict

import numpy as np
import scipy.sparse as sp
import torch

from . import native
from .trace import nvtx_range


def normalize_columns(A_csr: sp.csr_matrix) -> tuple[sp.csr_matrix, np.ndarray]:
    """(column-normalized FP32 CSR, dangling mask)."""
    A = A_csr.tocsc().astype(np.float32)
    col_sums = np.asarray(A.sum(axis=0), dtype=np.float32).ravel()
    inv = np.zeros_like(col_sums)
    np.divide(1.0, col_sums, out=inv, where=col_sums > 0)
    A_norm = sp.csr_matrix(A.multiply(inv).tocsr())
    A_norm.sum_duplicates()
    return A_norm, col_sums == 0


def device_transition(n: int, source, target, weight, device=None, normalize: bool = True):
    """Edge list -> transition matrix on the GPU (``gl_edges_to_transition``).

    ``source`` / ``target``: node indices (int, -1 or anything outside
    [0, n) for an unknown node), ``weight``: float64; numpy arrays or
    tensors.  Returns ``(indptr int32 [n + 1], indices int32 [nnz], data
    float32 [nnz], dangling bool [n])`` on ``device`` — the reference's
    ``A[target, source] = weight`` with duplicates summed
    (``app.py:111-131``), column-normalized as ``normalize_transition_matrix``
    does (``__init__.py:184-207``) but with dangling columns left empty and
    flagged.  One host synchronization (the stored count)."""
    dev = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
    if dev.type != "cuda":
        raise RuntimeError("device_transition needs a CUDA device")

    def host(x, dtype):
        t = x if isinstance(x, torch.Tensor) else torch.from_numpy(np.ascontiguousarray(np.asarray(x)))
        return t.reshape(-1).to(dtype)

    src64, dst64, w64 = host(source, torch.int64), host(target, torch.int64), host(weight, torch.float64)
    m = int(src64.numel())
    if int(dst64.numel()) != m or int(w64.numel()) != m:
        raise ValueError("source, target and weight must have one entry per edge")
    # an index outside [0, n) names no node: -1 before narrowing to int32
    src = torch.where((src64 < 0) | (src64 >= n), -1, src64).to(device=dev, dtype=torch.int32)
    dst = torch.where((dst64 < 0) | (dst64 >= n), -1, dst64).to(device=dev, dtype=torch.int32)
    w = w64.to(device=dev)
    with nvtx_range(f"edges.transition m={m}"):
        return _device_transition(n, m, src, dst, w, dev, normalize)


def _device_transition(n, m, src, dst, w, dev, normalize):
    L = native.lib()
    ws_bytes = int(L.gl_edges_workspace_bytes(n, m))
    if ws_bytes < 0:
        raise ValueError("too many nodes or edges for gl_edges_to_transition")
    ws = torch.empty(ws_bytes, dtype=torch.uint8, device=dev)
    indptr = torch.empty(n + 1, dtype=torch.int32, device=dev)
    indices = torch.empty(max(m, 1), dtype=torch.int32, device=dev)
    data = torch.empty(max(m, 1), dtype=torch.float32, device=dev)
    dangling = torch.empty(max(n, 1), dtype=torch.uint8, device=dev)
    nnz = torch.empty(1, dtype=torch.int64, device=dev)
    stream = torch.cuda.current_stream(dev).cuda_stream
    native.check(L.gl_edges_to_transition(n, m, src.data_ptr(), dst.data_ptr(), w.data_ptr(), int(bool(normalize)),
                                          indptr.data_ptr(), indices.data_ptr(), data.data_ptr(),
                                          dangling.data_ptr(), nnz.data_ptr(), ws.data_ptr(), ws_bytes, stream))
    k = int(nnz.item())
    return indptr, indices[:k], data[:k], dangling[:n].bool()


def edge_list_csr(n: int, src_idx: np.ndarray, dst_idx: np.ndarray, weight: np.ndarray) -> sp.csr_matrix:
    """A[target, source] = weight, duplicate edges summed (``app.py:111-131``)."""
    return sp.csr_matrix((weight.astype(np.float32), (dst_idx.astype(np.int64), src_idx.astype(np.int64))),
                         shape=(n, n))


# Resident graphs of the request path: a request whose edge list, node count
# and block parameters match a recent one reuses its device PBR matrix
# instead of rebuilding it (the reference rebuilds on every request,
# app.py:134).  Keyed by a digest of the indexed edge arrays; least recently
# used graphs are dropped past RESIDENT_GRAPHS.
RESIDENT_GRAPHS = 8
_resident: "OrderedDict[str, tuple]" = OrderedDict()
_resident_lock = threading.Lock()


def dangling_bitmap(mask: torch.Tensor) -> torch.Tensor:
    """Bit j % 32 of word j // 32 = mask[j] (the PPR step's dangling bitmap),
    computed on mask's device."""
    n = int(mask.numel())
    words = max(1, -(-n // 32))
    bits = torch.zeros(words * 32, dtype=torch.int64, device=mask.device)
    bits[:n] = mask.to(torch.int64)
    shifts = torch.arange(32, dtype=torch.int64, device=mask.device)
    packed = (bits.view(words, 32) << shifts).sum(dim=1)            # in [0, 2^32)
    return torch.where(packed >= 2 ** 31, packed - 2 ** 32, packed).to(torch.int32)


def resident_graph(n: int, si: np.ndarray, ti: np.ndarray, w: np.ndarray, block_size: int, min_nnz: int,
                   device) -> tuple:
    """(pbr, meta, dangling bitmap) of the request graph, built on the device
    (edge list -> transition matrix -> PBR) or taken from the resident set."""
    from .graph_link import get_pbr_gpu_meta
    from .pbr import pbr_from_device_csr

    dev = torch.device(device)
    h = hashlib.blake2b(digest_size=20)
    h.update(np.array([n, block_size, min_nnz, dev.index or 0, si.size], dtype=np.int64).tobytes())
    for a in (si, ti, w):
        h.update(np.ascontiguousarray(a).tobytes())
    key = h.hexdigest()
    with _resident_lock:
        hit = _resident.get(key)
        if hit is not None:
            _resident.move_to_end(key)
            return hit
    indptr, indices, data, dangling = device_transition(n, si, ti, w, dev)
    pbr = pbr_from_device_csr(indptr, indices, data, n, n, block_size, block_size, min_nnz).to(dev)
    entry = (pbr, get_pbr_gpu_meta(pbr), dangling_bitmap(dangling))
    with _resident_lock:
        _resident[key] = entry
        _resident.move_to_end(key)
        while len(_resident) > RESIDENT_GRAPHS:
            _resident.popitem(last=False)
    return entry


def clear_resident_graphs() -> None:
    with _resident_lock:
        _resident.clear()


def solve_edge_list_request(ids, index_of, src, dst, weight, seed_idx, alpha, max_iter, tol,
                            block_size: int = 2, min_nnz: int = 2) -> dict:
    """The body of ``POST /api/ppr`` after validation (``app.py:102-152``):
    degrees as plain edge counts, the transition matrix and its PBR built on
    the device (or reused), the fused power iteration with one column per
    seed, then the renormalized mean over the columns."""
    from .ppr import PprRun, teleport_from_seed_sets

    n = len(ids)
    si = np.fromiter((index_of.get(s, -1) for s in src), dtype=np.int64, count=len(src))
    ti = np.fromiter((index_of.get(t, -1) for t in dst), dtype=np.int64, count=len(dst))
    w = np.asarray(weight, dtype=np.float64).reshape(-1)
    # degrees count every edge whose endpoint is a node, valid weight or not
    out_c = np.bincount(si[si >= 0], minlength=n).astype(np.float64)
    in_c = np.bincount(ti[ti >= 0], minlength=n).astype(np.float64)
    out_deg = {nid: float(out_c[index_of[nid]]) for nid in ids}
    in_deg = {nid: float(in_c[index_of[nid]]) for nid in ids}

    dev = torch.device("cuda", torch.cuda.current_device())
    _, meta, dbits = resident_graph(n, si, ti, w, block_size, min_nnz, dev)
    K = len(seed_idx)
    seeds = torch.tensor(seed_idx, dtype=torch.int32, device=dev)
    tp = teleport_from_seed_sets(torch.arange(K + 1, dtype=torch.int32, device=dev), seeds, n, block_size)
    run = PprRun(meta, n, n, block_size, block_size, tp, alpha, max_iter, tol, native.GL_PPR_STOP_ALL,
                 dbits, native.GL_DANGLING_UNIFORM)
    res = run.run(chunk=8)
    r = res.X.to(torch.float64).mean(dim=1)
    total = float(r.sum().item())
    if total > 0:
        r = r / total
    return {"ranks": r.cpu().numpy(), "iterations": res.iterations, "converged": res.converged,
            "history": res.history, "in_deg": in_deg, "out_deg": out_deg}
