"""SpMM over batches that live in host memory, with copies overlapped.

``spmm_host_batches(pbr, xs, ys)`` computes ``ys[i] = A @ xs[i]`` for a list
of pinned host arrays.  Three CUDA streams and two device buffer pairs form a
pipeline: the host-to-device copy of batch i+1, the fused SpMM of batch i and
the device-to-host copy of batch i-1 run at the same time, so a long
sequence costs about max(copy in, SpMM, copy out) per batch instead of their
sum.  The SpMM needs all of X before it starts (its gathers touch every
row), so the overlap is across batches, not inside one.
"""
from __future__ import annotations

import torch

from . import native
from .graph_link.pbr_registry import get_pbr_gpu_meta
from .pbr import matrix_desc, spmm_workspace


def spmm_host_batches(pbr_mat, xs: list[torch.Tensor], ys: list[torch.Tensor], device=None) -> None:
    """ys[i][:] = A @ xs[i] for pinned host tensors xs[i] [cols, F], ys[i] [rows, F]."""
    meta = get_pbr_gpu_meta(pbr_mat)
    if meta is None:
        raise RuntimeError("PBRMatrix is not on GPU. Call .to('cuda') first.")
    if len(xs) != len(ys):
        raise ValueError("xs and ys must have the same length")
    if not xs:
        return
    dev = meta["data"].device if device is None else torch.device(device)
    F = xs[0].shape[1]
    dtype = meta["data"].dtype
    for x, y in zip(xs, ys):
        if x.shape != (pbr_mat.cols, F) or y.shape != (pbr_mat.rows, F):
            raise ValueError("every batch must be [cols, F] in and [rows, F] out with the same F")
        if x.dtype != dtype or y.dtype != dtype:
            raise TypeError(f"batches must be {dtype}")
    L = native.lib()
    with torch.cuda.device(dev):
        desc = matrix_desc(meta, pbr_mat.rows, pbr_mat.cols, pbr_mat.block_rows, pbr_mat.block_cols)
        s_in, s_mm, s_out = torch.cuda.Stream(dev), torch.cuda.Stream(dev), torch.cuda.Stream(dev)
        with torch.cuda.stream(s_mm):
            ws = spmm_workspace(meta, desc, 1, F, dev)
        xb = [torch.empty((pbr_mat.cols, F), dtype=dtype, device=dev) for _ in range(2)]
        yb = [torch.empty((pbr_mat.rows, F), dtype=dtype, device=dev) for _ in range(2)]
        ev_in = [torch.cuda.Event() for _ in range(2)]      # X copy done
        ev_mm = [torch.cuda.Event() for _ in range(2)]      # SpMM done (X free, Y ready)
        ev_out = [torch.cuda.Event() for _ in range(2)]     # Y copy done (Y free)
        cur = torch.cuda.current_stream(dev)
        s_in.wait_stream(cur)
        s_mm.wait_stream(cur)
        s_out.wait_stream(cur)
        for i, (x, y) in enumerate(zip(xs, ys)):
            k = i % 2
            if i >= 2:
                s_in.wait_event(ev_mm[k])         # the SpMM that read xb[k] is done
            with torch.cuda.stream(s_in):
                xb[k].copy_(x, non_blocking=True)
                ev_in[k].record(s_in)
            s_mm.wait_event(ev_in[k])
            if i >= 2:
                s_mm.wait_event(ev_out[k])        # yb[k] has been copied out
            native.check(L.gl_pbr_spmm(desc, xb[k].data_ptr(), yb[k].data_ptr(), 1, F,
                                       ws.data_ptr() if ws is not None else None,
                                       ws.numel() if ws is not None else 0, s_mm.cuda_stream))
            ev_mm[k].record(s_mm)
            s_out.wait_event(ev_mm[k])
            with torch.cuda.stream(s_out):
                y.copy_(yb[k], non_blocking=True)
                ev_out[k].record(s_out)
        cur.wait_stream(s_out)
        cur.wait_stream(s_mm)
        for t in xb + yb:
            t.record_stream(cur)
