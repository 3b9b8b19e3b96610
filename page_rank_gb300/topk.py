"""Top-k of PPR columns on the device (``gl_topk_columns``).

The reference returns all N ranks of a query and leaves the top-X cut to its
frontend (``Backend/server/app.py:146-158``); a serving caller that wants
the X best nodes of each of many columns copies k (value, row) pairs per
column back instead of N values.
"""
from __future__ import annotations

import torch

from . import native
from .trace import nvtx_range


def topk_columns(X: torch.Tensor, k: int, columns=None) -> tuple[torch.Tensor, torch.Tensor]:
    """``(values [C, k] float32, rows [C, k] int32)`` of the k largest entries
    of each selected column of the row-major FP32 matrix ``X [rows, ld]``
    (``columns``: int sequence / tensor of column numbers, default all),
    sorted by value descending, equal values by row ascending.  With fewer
    than k rows the trailing slots hold ``-inf`` and ``-1``.  Asynchronous on
    the current stream (no host synchronization)."""
    if X.device.type != "cuda" or X.dtype != torch.float32 or X.dim() != 2:
        raise TypeError("X must be a 2-D float32 CUDA tensor")
    if X.stride(1) != 1 or (X.shape[0] > 1 and X.stride(0) < X.shape[1]):
        X = X.contiguous()
    k = int(k)
    if not 0 <= k <= native.GL_TOPK_MAX:
        raise ValueError(f"k must be in [0, {native.GL_TOPK_MAX}]")
    rows, ld = int(X.shape[0]), int(X.stride(0)) if X.shape[0] > 1 else int(X.shape[1])
    dev = X.device
    if columns is None:
        cols = None
        C = int(X.shape[1])
    else:
        cols = torch.as_tensor(columns).reshape(-1)
        C = int(cols.numel())
        if C and (int(cols.min()) < 0 or int(cols.max()) >= X.shape[1]):   # host check for host input
            raise ValueError("column number out of range")
        cols = cols.to(device=dev, dtype=torch.int32)
    values = torch.empty((C, k), dtype=torch.float32, device=dev)
    rows_out = torch.empty((C, k), dtype=torch.int32, device=dev)
    if C == 0 or k == 0:
        return values, rows_out
    L = native.lib()
    with nvtx_range(f"topk k={k} C={C}"):
        return _topk(L, X, rows, ld, cols, C, k, values, rows_out, dev)


def _topk(L, X, rows, ld, cols, C, k, values, rows_out, dev):
    ws_bytes = int(L.gl_topk_workspace_bytes(rows, C, k))
    ws = torch.empty(max(ws_bytes, 1), dtype=torch.uint8, device=dev)
    native.check(L.gl_topk_columns(X.data_ptr() if X.numel() else None, rows, ld,
                                   cols.data_ptr() if cols is not None else None, C, k, values.data_ptr(),
                                   rows_out.data_ptr(), ws.data_ptr(), ws_bytes,
                                   torch.cuda.current_stream(dev).cuda_stream))
    return values, rows_out
