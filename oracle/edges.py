"""Edge list -> column-normalized transition CSR — test infrastructure only.

Restates what the reference service does between the request body and the
PBR build (``Backend/server/app.py:111-131`` then
``normalize_transition_matrix``, ``Backend/graph_link/graph_link/__init__.py:184-207``),
minus the dense dangling columns (a dangling column is reported in a mask
instead of being filled with N values of 1/N):

1. an edge is kept when both endpoints are nodes (index in [0, n)) and its
   weight is finite and > 0 (``app.py:114-122``); the weight is rounded to
   FP32 (``app.py:126``);
2. ``A[target, source]`` sums duplicate edges (scipy's COO -> CSR
   conversion).  This restatement sums them in input order, which is what
   scipy does whenever its per-row sort (``std::sort`` on column only) keeps
   equal columns in input order: rows of at most 16 entries (insertion sort),
   or at most two duplicates of a pair (FP32 addition commutes), or equal
   weights (exact sums);
3. column sums in FP32 exactly as ``csc.sum(axis=0)`` computes them: scipy's
   minor-axis reduction ``np.add.reduceat`` over each column's entries in
   increasing row order, i.e. the first entry plus numpy's pairwise sum of
   the rest (numpy ``loops_utils.h``: below 8 elements a sequential sum, up
   to 128 eight interleaved accumulators combined as a balanced tree, beyond
   that the halves split at a multiple of 8);
4. ``inv = 1 / colsum`` (0 for a zero sum) and ``A[i, j] * inv[j]`` in FP32;
   products that are exactly zero are not stored (scipy's sparse product
   keeps nonzeros only).
"""
from __future__ import annotations

import numpy as np


def pairwise_sum_f32(a: np.ndarray) -> np.float32:
    """numpy's pairwise summation of a float32 vector, in float32."""
    n = len(a)
    if n < 8:
        res = np.float32(0.0)
        for v in a:
            res = np.float32(res + v)
        return res
    if n <= 128:
        r = [np.float32(v) for v in a[:8]]
        i = 8
        stop = n - (n % 8)
        while i < stop:
            for j in range(8):
                r[j] = np.float32(r[j] + a[i + j])
            i += 8
        res = np.float32(np.float32(np.float32(r[0] + r[1]) + np.float32(r[2] + r[3]))
                         + np.float32(np.float32(r[4] + r[5]) + np.float32(r[6] + r[7])))
        while i < n:
            res = np.float32(res + a[i])
            i += 1
        return res
    n2 = n // 2
    n2 -= n2 % 8
    return np.float32(pairwise_sum_f32(a[:n2]) + pairwise_sum_f32(a[n2:]))


def column_sum_f32(a: np.ndarray) -> np.float32:
    """``np.add.reduceat`` of one non-empty segment: first + pairwise(rest)."""
    return np.float32(a[0] + pairwise_sum_f32(a[1:]))


def edges_to_csr(n: int, source: np.ndarray, target: np.ndarray, weight: np.ndarray):
    """(indptr int64, indices int32, data float32) of A[target, source] with
    duplicates summed in input order; no normalization."""
    s = np.asarray(source, dtype=np.int64)
    t = np.asarray(target, dtype=np.int64)
    w = np.asarray(weight, dtype=np.float64)
    ok = (s >= 0) & (s < n) & (t >= 0) & (t < n) & np.isfinite(w) & (w > 0)
    s, t, w32 = s[ok], t[ok], w[ok].astype(np.float32)
    order = np.lexsort((s, t))          # stable: input order among equal (t, s)
    s, t, w32 = s[order], t[order], w32[order]
    head = np.ones(len(s), dtype=bool)
    head[1:] = (s[1:] != s[:-1]) | (t[1:] != t[:-1])
    starts = np.flatnonzero(head)
    vals = np.empty(len(starts), dtype=np.float32)
    for k, b in enumerate(starts):
        e = starts[k + 1] if k + 1 < len(starts) else len(s)
        acc = w32[b]
        for q in range(b + 1, e):
            acc = np.float32(acc + w32[q])
        vals[k] = acc
    rows, cols = t[starts], s[starts]
    indptr = np.zeros(n + 1, dtype=np.int64)
    np.add.at(indptr, rows + 1, 1)
    return np.cumsum(indptr), cols.astype(np.int32), vals


def normalize_csr(n: int, indptr: np.ndarray, indices: np.ndarray, data: np.ndarray):
    """(indptr, indices, data, dangling mask) of the column-normalized matrix."""
    rows = np.repeat(np.arange(n, dtype=np.int64), np.diff(indptr))
    order = np.lexsort((rows, indices))     # column-major, rows increasing
    colsum = np.zeros(n, dtype=np.float32)
    cs = indices[order]
    vs = data[order]
    bounds = np.searchsorted(cs, np.arange(n + 1))
    for j in range(n):
        if bounds[j + 1] > bounds[j]:
            colsum[j] = column_sum_f32(vs[bounds[j]:bounds[j + 1]])
    inv = np.zeros(n, dtype=np.float32)
    with np.errstate(over="ignore"):   # a subnormal sum has no finite inverse (inf, as scipy)
        np.divide(np.float32(1.0), colsum, out=inv, where=colsum != 0)
    with np.errstate(invalid="ignore", over="ignore"):
        vals = (data * inv[indices]).astype(np.float32)
    keep = vals != 0
    kept_rows = rows[keep]
    out_ptr = np.zeros(n + 1, dtype=np.int64)
    np.add.at(out_ptr, kept_rows + 1, 1)
    return np.cumsum(out_ptr), indices[keep], vals[keep], colsum == 0


def transition_from_edges(n: int, source, target, weight):
    """Edge list -> (indptr, indices, data, dangling): steps 1-4 above."""
    indptr, indices, data = edges_to_csr(n, source, target, weight)
    return normalize_csr(n, indptr, indices, data)
