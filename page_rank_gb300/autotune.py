"""Autotuner for the PBR layout and launch shape of a resident graph.

For a given transition matrix and working-set width K it builds the PBR
matrix for each candidate (block size 2 / 4 / 8, min_nnz_per_block, column
tile), times a few fused PPR steps with CUDA events, and returns the fastest
configuration.  Building is cheap on the device, so the whole sweep costs a
fraction of one batched solve.
"""
from __future__ import annotations

import itertools
from dataclasses import dataclass, field

import numpy as np
import scipy.sparse as sp
import torch

from . import native
from .pbr import pbr_from_device_csr
from .ppr import PprRun, dangling_bitmap, teleport_from_seed_sets


@dataclass
class TuneResult:
    block_size: int
    min_nnz: int
    column_tile: int
    ms_per_step: float
    table: list = field(default_factory=list)   # (block, min_nnz, tile, ms, packed fraction)


def default_candidates(K: int):
    blocks = {2: (1, 2), 4: (2, 4), 8: (4, 8, 12)}
    tiles = (0, 64) if K >= 128 else (0,)
    for bs, mins in blocks.items():
        for mn, tile in itertools.product(mins, tiles):
            yield bs, mn, tile


def autotune(A: sp.csr_matrix, K: int, device=None, candidates=None, steps: int = 4,
             alpha: float = 0.85, seed: int = 0) -> TuneResult:
    from .graph_link.pbr_registry import get_pbr_gpu_meta

    dev = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
    n = A.shape[0]
    with torch.cuda.device(dev):
        indptr = torch.from_numpy(A.indptr.astype(np.int32)).to(dev)
        indices = torch.from_numpy(A.indices.astype(np.int32)).to(dev)
        data = torch.from_numpy(A.data.astype(np.float32)).to(dev)
        dbits = dangling_bitmap(indices, n)
        rng = np.random.default_rng(seed)
        seeds = torch.from_numpy(rng.integers(0, n, K).astype(np.int32)).to(dev)
        sptr = torch.arange(K + 1, dtype=torch.int32, device=dev)
        gen = torch.Generator(device=dev).manual_seed(seed)
        x_dense = torch.rand((n, K), generator=gen, device=dev)
        x_dense /= x_dense.sum(dim=0, keepdim=True)
        table = []
        best = None
        for bs, mn, tile in (candidates or default_candidates(K)):
            pbr = pbr_from_device_csr(indptr, indices, data, n, n, bs, bs, mn).to(dev)
            meta = get_pbr_gpu_meta(pbr)
            meta["column_tile"] = tile
            tp = teleport_from_seed_sets(sptr, seeds, n, bs)
            run = PprRun(meta, n, n, bs, bs, tp, alpha, steps + 2, 0.0, native.GL_PPR_STOP_ALL, dbits)
            # a dense start: mid-solve iterates are dense, and a step over
            # them measured ~30 % slower than over the first, sparse ones
            run.init(x_dense)
            run.launch_chunk(2)                      # warm (occupancy query, caches)
            torch.cuda.synchronize(dev)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            run.launch_chunk(steps)
            e1.record()
            torch.cuda.synchronize(dev)
            ms = e0.elapsed_time(e1) / steps
            packed = pbr.compressed_nnz() / max(1, A.nnz)
            table.append((bs, mn, tile, round(ms, 4), round(packed, 3)))
            if best is None or ms < best[3]:
                best = (bs, mn, tile, ms)
            del run, pbr, meta
        torch.cuda.empty_cache()
    return TuneResult(block_size=best[0], min_nnz=best[1], column_tile=best[2], ms_per_step=best[3],
                      table=table)
