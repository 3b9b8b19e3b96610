"""Drop-in mirror of the reference Python API ``graph_link``.

Same names, signatures, defaults, return values and error types as the
reference package (``Backend/graph_link/graph_link/__init__.py:274-285``),
with the work done by this repository's sm_103a kernels:

* ``csr_to_pbr`` builds the PBR arrays on the GPU (bit-identical to the
  reference builder for canonical CSR input);
* ``pbr_matmul`` / ``pbr_batched_matmul_cuda`` run one fused, atomic-free
  PBR + CSR-remainder SpMM launch;
* ``run_personalized_pagerank`` runs the fused power-iteration step (SpMM,
  alpha scaling, teleport and L1 residual in one pass per iteration).

Use it as ``from page_rank_gb300 import graph_link`` (or alias it to the
module name ``graph_link``).
"""
from __future__ import annotations

import numpy as np
import scipy.sparse as sp
import torch

from .. import native
from ..pbr import (DataOrder, PBRMatrix, PBRMatrixInt32Double, PBRMatrixInt32Float,
                   PBRMatrixInt64Double, PBRMatrixInt64Float, matrix_desc, pbr_from_device_csr,
                   spmm_workspace)
from ..pbr_io import load_pbr, save_pbr
from ..ppr import PprRun, dangling_bitmap, teleport_from_seed_sets
from ..trace import nvtx_range
from .pbr_registry import clear_pbr_gpu_meta, get_pbr_gpu_meta, set_pbr_gpu_meta


def _require_cuda(what: str) -> torch.device:
    if not torch.cuda.is_available():
        raise RuntimeError(f"{what} runs on the GPU and no CUDA device is available")
    return torch.device("cuda", torch.cuda.current_device())


# ---------------------------------------------------------------------------
# SpMM
# ---------------------------------------------------------------------------
def pbr_batched_matmul_cuda(pbr_mat, x: torch.Tensor) -> torch.Tensor:
    """Y = A @ x with shape [batch, rows, features] (``__init__.py:66-101``).

    One launch of the fused stripe kernel on the current stream; Y is
    allocated uninitialized because the kernel writes every element."""
    meta = get_pbr_gpu_meta(pbr_mat)
    if meta is None:
        raise RuntimeError("PBRMatrix is not on GPU. Call .to('cuda') first.")
    index_dtype = meta["coords"].dtype
    data_dtype = meta["data"].dtype
    if index_dtype != torch.int32 or data_dtype not in (torch.float32, torch.float64):
        raise TypeError(f"Unsupported dtype combination: index={index_dtype}, data={data_dtype}")
    if x.dtype != data_dtype:
        raise RuntimeError(f"expected x of dtype {data_dtype}, got {x.dtype}")
    if not x.is_cuda:
        raise RuntimeError("x must be a CUDA tensor")
    x3 = x.unsqueeze(0) if x.dim() == 2 else x
    if x3.dim() != 3:
        raise ValueError(f"Expected 2D or 3D input, got {x.dim()}D")
    if x3.shape[1] != pbr_mat.cols:
        raise ValueError(f"x has {x3.shape[1]} rows, the matrix has {pbr_mat.cols} columns")
    x3 = x3.contiguous()
    batch, _, width = x3.shape
    y = torch.empty((batch, pbr_mat.rows, width), dtype=x.dtype, device=x.device)
    with torch.cuda.device(x.device), nvtx_range(f"pbr.spmm F={width}"):
        desc = matrix_desc(meta, pbr_mat.rows, pbr_mat.cols, pbr_mat.block_rows, pbr_mat.block_cols)
        ws = spmm_workspace(meta, desc, batch, width, x.device)
        native.check(native.lib().gl_pbr_spmm(desc, x3.data_ptr() if x3.numel() else None,
                                              y.data_ptr() if y.numel() else None, batch, width,
                                              ws.data_ptr() if ws is not None else None,
                                              ws.numel() if ws is not None else 0,
                                              torch.cuda.current_stream(x.device).cuda_stream))
    return y


def pbr_matmul(pbr_mat, x: torch.Tensor):
    """Unified entry point (``__init__.py:104-134``): GPU for CUDA ``x``."""
    if x.dim() == 2:
        pass
    elif x.dim() == 3:
        pass
    else:
        raise ValueError(f"Expected 2D or 3D input, got {x.dim()}D")
    if x.is_cuda:
        if get_pbr_gpu_meta(pbr_mat) is None:
            pbr_mat = pbr_mat.to(x.device)
        y = pbr_batched_matmul_cuda(pbr_mat, x)
        return y.squeeze(0) if x.dim() == 2 else y
    return pbr_batched_matmul_cpu(pbr_mat, x)


def pbr_batched_matmul_cpu(pbr_mat, x):
    """The reference binds a CPU SpMM under this name, but it cannot be called
    with tensors (``bindings.cpp:65-68`` lacks the tensor caster, so it raises
    ``TypeError``).  This engine has no CPU path either; it raises the same
    error type."""
    raise TypeError("pbr_batched_matmul_cpu(): CPU SpMM is not provided; move x to a CUDA device")


def pbr_batched_matmul_triton_gpu(pbr_mat, x: torch.Tensor, y: torch.Tensor, batch_size: int,
                                  width: int):
    """Name kept from the reference's experimental Triton kernel
    (``pbr_matrix_triton.py:77-110``), which accumulated into ``y``.  Here it
    adds this engine's SpMM result into ``y`` (no Triton involved)."""
    out = pbr_batched_matmul_cuda(pbr_mat, x)
    y += out.view_as(y) if y.dim() == out.dim() else out.squeeze(0).view_as(y)
    return y


# ---------------------------------------------------------------------------
# Builder and format helpers
# ---------------------------------------------------------------------------
def _csr_parts(mat):
    if isinstance(mat, torch.Tensor):
        if mat.device.type != "cpu":
            raise ValueError("Input tensor must be on CPU")
        indptr = mat.crow_indices().numpy()
        indices = mat.col_indices().numpy()
        data = mat.values().cpu().numpy()
        shape = tuple(mat.shape)
        canonical = None
    elif isinstance(mat, sp.csr_matrix):
        indptr, indices, data, shape = mat.indptr, mat.indices, mat.data, mat.shape
        canonical = mat.has_canonical_format
    else:
        raise TypeError(f"Unsupported type {type(mat)}")
    return indptr, indices, data, shape, canonical


def _dtypes(indptr, indices, data):
    """The reference's pybind overload order picks int64/float first, then
    int32/float, int64/double, int32/double (``bindings.cpp:70-73``)."""
    idx64 = indptr.dtype == np.int64 or indices.dtype == np.int64
    itype = np.int64 if idx64 else np.int32
    vtype = np.float64 if data.dtype == np.float64 else np.float32
    return itype, vtype


def csr_to_pbr(mat, block_rows: int = 2, block_cols: int = 2, min_nnz_per_block: int = 2):
    """CSR -> PBR on the GPU (``__init__.py:137-156``, ``pbr_matrix.cpp:340-477``).

    The result is a host-side handle like the reference's (call ``.to('cuda')``
    before the GPU routines); its arrays already live in device memory.

    Input that is not in canonical CSR form (unsorted or duplicate column
    indices) is canonicalized first (duplicates summed, indices sorted).  The
    reference does not do this and, for such input, pairs values with the
    wrong bits; canonical input gives the reference's exact output.
    """
    if not isinstance(min_nnz_per_block, (int, np.integer)) or not 0 <= int(min_nnz_per_block) <= 255:
        raise TypeError("min_nnz_per_block must be an integer in 0..255 (uint8_t)")
    indptr, indices, data, shape, canonical = _csr_parts(mat)
    itype, vtype = _dtypes(indptr, indices, data)
    if canonical is not True:
        m = sp.csr_matrix((np.asarray(data), np.asarray(indices), np.asarray(indptr)), shape=shape)
        if not m.has_canonical_format:
            m = m.copy()
            m.sum_duplicates()
        indptr, indices, data = m.indptr, m.indices, m.data
    dev = _require_cuda("csr_to_pbr")
    rows, cols = int(shape[0]), int(shape[1])
    t_indptr = torch.from_numpy(np.ascontiguousarray(indptr, dtype=itype)).to(dev)
    t_indices = torch.from_numpy(np.ascontiguousarray(indices, dtype=itype)).to(dev)
    t_data = torch.from_numpy(np.ascontiguousarray(data, dtype=vtype)).to(dev)
    return pbr_from_device_csr(t_indptr, t_indices, t_data, rows, cols, int(block_rows),
                               int(block_cols), int(min_nnz_per_block))


def pbr_to_csr(pbr_mat, indptr, indices, data):
    """Fill caller-provided CSR arrays from a PBR matrix (``pbr_matrix.cpp:289-338``),
    computed on the device (``gl_pbr_to_csr``) and copied into the arrays
    (numpy arrays or torch tensors, any index / value dtype).

    Unlike the reference, matrices whose row count is not a multiple of the
    block height are handled (the reference throws ``RuntimeError`` there)."""
    from ..pbr import device_to_csr
    dev = _require_cuda("pbr_to_csr")
    src = pbr_mat._build.codes.device if pbr_mat._build.codes.is_cuda else dev
    ip, ix, dv = device_to_csr(pbr_mat, src)
    nnz = ix.numel()
    for dst, t, n in ((indptr, ip, pbr_mat.rows + 1), (indices, ix, nnz), (data, dv, nnz)):
        if isinstance(dst, torch.Tensor):
            dst[:n].copy_(t.to(dst.device, dst.dtype))
        else:
            dst[:n] = t.cpu().numpy()


def pbr_analyze_csr(mat, block_rows: int = 8, block_cols: int = 8, min_nnz_coverage=1000):
    """Block-pattern statistics (``__init__.py:163-181``; the reference's
    ``pbr_analyze_csr``, ``pbr_matrix.cpp:71-156``, returns an unbound type and
    never records block coordinates, so it is unusable there).  Returns a dict:
    pattern occurrences and the nnz they would cover under the coverage rule."""
    from ..analyze import analyze_csr
    return analyze_csr(mat, block_rows, block_cols, min_nnz_coverage)


def normalize_transition_matrix(A_csr: sp.csr_matrix) -> sp.csr_matrix:
    """Column-stochastic transition matrix (``__init__.py:184-207``).

    Same FP32 arithmetic, in the same order, as the reference: columns are
    divided by their sum, and every dangling column (sum 0) becomes a dense
    uniform 1/N column.  (``page_rank_gb300.transition`` offers the variant
    that keeps dangling columns empty and redistributes their mass in the
    kernel instead.)"""
    N = A_csr.shape[0]
    A = A_csr.tocsc().astype(np.float32)
    col_sums = np.asarray(A.sum(axis=0), dtype=np.float32).ravel()
    inv = np.zeros_like(col_sums)
    np.divide(1.0, col_sums, out=inv, where=col_sums > 0)
    A_norm = A.multiply(inv).tocsr()
    dangling = np.where(col_sums == 0)[0]
    if dangling.size > 0:
        r = np.tile(np.arange(N, dtype=np.int32), dangling.size)
        c = np.repeat(dangling.astype(np.int32), N)
        v = np.full(N * dangling.size, 1.0 / N, dtype=np.float32)
        A_norm = A_norm + sp.csr_matrix((v, (r, c)), shape=(N, N))
    return A_norm


# ---------------------------------------------------------------------------
# Personalized PageRank
# ---------------------------------------------------------------------------
def run_personalized_pagerank(pbr_mat, source_nodes: torch.Tensor, alpha: float = 0.85,
                              max_iterations: int = 100, tolerance: float = 1e-6,
                              return_history: bool = False, warm_start: torch.Tensor | None = None):
    """Batched PPR by power iteration (``__init__.py:210-271``):

        X_{t+1} = alpha * A @ X_t + (1 - alpha) * e_s

    one column per source node.  Stops when the largest per-column L1 update
    falls below ``tolerance``.  Returns ``(X, iterations, converged)`` or, with
    ``return_history``, ``(X, iterations, converged, history)``.

    ``warm_start`` (an addition; the reference always starts from the
    one-hot sources): start columns [rows, K] on the matrix's device, e.g.
    ``window_start.WindowStart(...).start(...)``; the fixed point and the
    stop rule are unchanged."""
    meta = get_pbr_gpu_meta(pbr_mat)
    if meta is None:
        raise RuntimeError("PBRMatrix is not on GPU. Call .to('cuda') first.")
    if source_nodes.dtype != torch.int32:
        source_nodes = source_nodes.to(torch.int32)
    device = meta["data"].device
    K = int(source_nodes.shape[0])
    if K == 0:
        raise RuntimeError("run_personalized_pagerank: source_nodes is empty")
    N = pbr_mat.rows
    with torch.cuda.device(device):
        seeds = source_nodes.to(device).contiguous()
        seed_ptr = torch.arange(K + 1, dtype=torch.int32, device=device)
        tp = teleport_from_seed_sets(seed_ptr, seeds, N, pbr_mat.block_rows)
        run = PprRun(meta, N, pbr_mat.cols, pbr_mat.block_rows, pbr_mat.block_cols, tp, alpha,
                     max_iterations, tolerance, native.GL_PPR_STOP_ALL, None)
        if warm_start is not None:
            if tuple(warm_start.shape) != (N, K):
                raise ValueError(f"warm_start must be [{N}, {K}]")
            warm_start = warm_start.to(device=device, dtype=run.bufs[0].dtype)
        res = run.run(chunk=8, x0=warm_start)
    if return_history:
        return res.X, res.iterations, res.converged, res.history
    return res.X, res.iterations, res.converged


__all__ = [
    "csr_to_pbr",
    "pbr_to_csr",
    "pbr_analyze_csr",
    "pbr_matmul",
    "pbr_batched_matmul_cpu",
    "pbr_batched_matmul_triton_gpu",
    "pbr_batched_matmul_cuda",
    "get_pbr_gpu_meta",
    "normalize_transition_matrix",
    "run_personalized_pagerank",
    "clear_pbr_gpu_meta",
    "DataOrder",
    "save_pbr",
    "load_pbr",
    "PBRMatrixInt32Float",
    "PBRMatrixInt64Float",
    "PBRMatrixInt32Double",
    "PBRMatrixInt64Double",
]
