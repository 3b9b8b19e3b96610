"""Block-pattern statistics of a CSR matrix (the reference's ``pbr_analyze_csr``).

The reference defines this analysis (``pbr_matrix.cpp:71-156,275-287``) but it
cannot run there: the stripe walk never records block indices, so every
statistic stays zero, and the result type is not bound to Python.  Here the
blocks come from the device builder run with ``min_nnz_per_block = 0`` (every
block kept), and the distinct codes, their occurrences and the coverage-rule
totals are counted on the device (``gl_pbr_block_patterns``); the size
formulas are the reference's: a pattern is "compressed" when occurrences x
popcount >= ``min_nnz_coverage``.
"""
from __future__ import annotations


def analyze_csr(mat, block_rows: int = 8, block_cols: int = 8, min_nnz_coverage: int = 1000,
                index_bytes: int = 4, value_bytes: int = 4) -> dict:
    from .graph_link import csr_to_pbr
    from .pbr import block_patterns

    pbr = csr_to_pbr(mat, block_rows, block_cols, 0)
    uniq, counts, totals = block_patterns(pbr._build.codes, min_nnz_coverage)
    nnz = int(pbr.total_nnz)
    remainder_nnz = totals["remainder_nnz"]
    accounted_blocks = totals["accounted_blocks"]
    remainder_coo_overhead = float(remainder_nnz) * (2.0 * index_bytes + value_bytes)
    nblocks = int(counts.sum())
    return {
        "rows": pbr.rows, "cols": pbr.cols, "nnz": nnz,
        "block_rows": block_rows, "block_cols": block_cols, "min_nnz_coverage": min_nnz_coverage,
        "accounted_nnz": nnz - remainder_nnz,
        "remainder_nnz": remainder_nnz,
        "accounted_patterns": totals["accounted_patterns"],
        "accounted_blocks": accounted_blocks,
        "remainder_coo_overhead": remainder_coo_overhead,
        "csr_index_size": float(nnz + pbr.cols + 1) * index_bytes,
        "pbr_index_size": float(2.0 * accounted_blocks + remainder_coo_overhead) * index_bytes,
        "patterns": {int(c): int(n) for c, n in zip(uniq, counts)},
        # every stored value sits in a block when min_nnz_per_block = 0
        "mean_block_density": float(nnz) / max(1, nblocks) / float(block_rows * block_cols),
    }
