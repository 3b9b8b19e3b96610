"""Block-pattern statistics of a CSR matrix (the reference's ``pbr_analyze_csr``).

The reference defines this analysis (``pbr_matrix.cpp:71-156,275-287``) but it
cannot run there: the stripe walk never records block indices, so every
statistic stays zero, and the result type is not bound to Python.  Here the
blocks come from the device builder run with ``min_nnz_per_block = 0`` (every
block kept), the patterns are counted on the device, and the same coverage
rule and size formulas are applied: a pattern is "compressed" when
occurrences x popcount >= ``min_nnz_coverage``.
"""
from __future__ import annotations

import numpy as np
import torch


def analyze_csr(mat, block_rows: int = 8, block_cols: int = 8, min_nnz_coverage: int = 1000,
                index_bytes: int = 4, value_bytes: int = 4) -> dict:
    from .graph_link import csr_to_pbr

    pbr = csr_to_pbr(mat, block_rows, block_cols, 0)
    codes = pbr._build.codes
    if codes.numel():
        uniq, counts = torch.unique(codes, return_counts=True)
        uniq_np = uniq.cpu().numpy().view(np.uint64)
        counts_np = counts.cpu().numpy().astype(np.int64)
    else:
        uniq_np = np.zeros(0, np.uint64)
        counts_np = np.zeros(0, np.int64)
    pops = np.array([bin(int(c)).count("1") for c in uniq_np], dtype=np.int64)
    coverage = counts_np * pops
    compress = coverage >= min_nnz_coverage
    nnz = int(pbr.total_nnz)
    remainder_nnz = int(coverage[~compress].sum())
    accounted_blocks = int(counts_np[compress].sum())
    remainder_coo_overhead = float(remainder_nnz) * (2.0 * index_bytes + value_bytes)
    return {
        "rows": pbr.rows, "cols": pbr.cols, "nnz": nnz,
        "block_rows": block_rows, "block_cols": block_cols, "min_nnz_coverage": min_nnz_coverage,
        "accounted_nnz": nnz - remainder_nnz,
        "remainder_nnz": remainder_nnz,
        "accounted_patterns": int(compress.sum()),
        "accounted_blocks": accounted_blocks,
        "remainder_coo_overhead": remainder_coo_overhead,
        "csr_index_size": float(nnz + pbr.cols + 1) * index_bytes,
        "pbr_index_size": float(2.0 * accounted_blocks + remainder_coo_overhead) * index_bytes,
        "patterns": {int(c): int(n) for c, n in zip(uniq_np, counts_np)},
        "mean_block_density": float((pops * counts_np).sum() / max(1, counts_np.sum()))
        / float(block_rows * block_cols),
    }
