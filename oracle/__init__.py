"""Oracle package — TEST INFRASTRUCTURE, not product code.

Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` may import this package, and only as the checker (or the timed
CPU baseline).  The product package ``page_rank_gb300`` never imports it.

Contents
--------
* ``pbr_oracle.cpp`` — C++ restatement of the reference PBR builder
  (``Backend/graph_link/pbr_matrix/pbr_matrix.cpp:340-477``) and of
  ``pbr_to_csr`` (``pbr_matrix.cpp:289-338``), built here by
  :func:`build_oracle` with g++ and called through ctypes.
* ``spmm.py`` — FP64 SpMM oracle: the reference CPU SpMM semantics
  (``pbr_matrix.cpp:17-68``) and scipy's ``A @ X`` (the check used by
  ``Tests/test_spmm.py:46``).
* ``ppr.py`` — FP64 Personalized PageRank oracles: the reference power
  iteration and stop rule (``graph_link/__init__.py:258-267``,
  ``kernels/ppr_kernel.cu:130-168``), the dangling-mass-to-personalization
  update (``kernels/ppr_kernel.cu:57-97``), and a direct sparse solve.
* ``edges.py`` — the reference service's edge list -> normalized matrix step
  (``Backend/server/app.py:111-131`` + ``normalize_transition_matrix``),
  including numpy's pairwise column-sum order; pinned against golden
  fixtures written by the reference's own code path.
* ``topk.py`` — the top-k selection ``gl_topk_columns`` promises (numpy
  lexicographic sort on order-preserving keys).
* ``ref_build.py`` — recipe that compiles the reference's own CPU builder into
  ``oracle/_ref/`` where the reference checkout exists (this container), used
  to pin the restatement and to generate ``tests/golden/``.

Parity pin: the restated builder is checked bit for bit against the compiled
reference builder on randomized matrices (``tests/test_oracle_vs_reference.py``)
and against the golden fixtures that builder wrote
(``tests/test_oracle_golden.py``).
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from pathlib import Path

import numpy as np

_HERE = Path(__file__).resolve().parent
_BUILD_DIR = _HERE / "_build"
_LIB_PATH = _BUILD_DIR / "liboracle_pbr.so"
_lib = None

_SUFFIX = {
    (np.dtype(np.int32), np.dtype(np.float32)): "i32_f32",
    (np.dtype(np.int32), np.dtype(np.float64)): "i32_f64",
    (np.dtype(np.int64), np.dtype(np.float32)): "i64_f32",
    (np.dtype(np.int64), np.dtype(np.float64)): "i64_f64",
}


def build_oracle(force: bool = False) -> Path:
    """Compile ``pbr_oracle.cpp`` with g++ into ``oracle/_build``."""
    src = _HERE / "pbr_oracle.cpp"
    if (not force and _LIB_PATH.is_file()
            and _LIB_PATH.stat().st_mtime >= src.stat().st_mtime):
        return _LIB_PATH
    _BUILD_DIR.mkdir(exist_ok=True)
    tmp = _LIB_PATH.with_suffix(f".{os.getpid()}.tmp.so")
    subprocess.check_call(["g++", "-O2", "-std=c++17", "-shared", "-fPIC",
                           str(src), "-o", str(tmp)])
    os.replace(tmp, _LIB_PATH)
    return _LIB_PATH


def _load():
    global _lib
    if _lib is None:
        _lib = ctypes.CDLL(str(build_oracle()))
    return _lib


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(ctypes.c_void_p)


def csr_to_pbr(indptr, indices, data, rows: int, cols: int,
               block_rows: int, block_cols: int, min_nnz_per_block: int) -> dict:
    """Run the restated reference builder; returns the PBR arrays as numpy.

    Index dtype (int32/int64) and value dtype (float32/float64) select the
    same template instance the reference's pybind overloads would pick.
    """
    indptr = np.ascontiguousarray(indptr)
    itype = indptr.dtype
    indices = np.ascontiguousarray(indices, dtype=itype)
    data = np.ascontiguousarray(data)
    sfx = _SUFFIX[(itype, data.dtype)]
    lib = _load()
    f = getattr(lib, f"oracle_csr_to_pbr_{sfx}")
    f.restype = ctypes.c_void_p
    f.argtypes = [ctypes.c_void_p] * 3 + [ctypes.c_int64] * 4 + [ctypes.c_int]
    h = f(_ptr(indptr), _ptr(indices), _ptr(data), rows, cols, block_rows, block_cols,
          int(min_nnz_per_block))
    try:
        sizes = np.zeros(4, np.int64)
        g = getattr(lib, f"oracle_pbr_sizes_{sfx}")
        g.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
        g(h, _ptr(sizes))
        nb, nd, nr, tot = (int(x) for x in sizes)
        out = {
            "rows": rows, "cols": cols, "block_rows": block_rows, "block_cols": block_cols,
            "total_nnz": tot,
            "block_codes": np.zeros(nb, np.uint64),
            "block_coords": np.zeros(2 * nb, itype),
            "block_offsets": np.zeros(nb + 1, itype),
            "block_data": np.zeros(nd, data.dtype),
            "remainder_indptr": np.zeros(rows + 1, itype),
            "remainder_col_ind": np.zeros(nr, itype),
            "remainder_data": np.zeros(nr, data.dtype),
        }
        c = getattr(lib, f"oracle_pbr_copy_{sfx}")
        c.argtypes = [ctypes.c_void_p] * 8
        c(h, *(_ptr(out[k]) for k in ("block_codes", "block_coords", "block_offsets",
                                       "block_data", "remainder_indptr",
                                       "remainder_col_ind", "remainder_data")))
        return out
    finally:
        fr = getattr(lib, f"oracle_pbr_free_{sfx}")
        fr.argtypes = [ctypes.c_void_p]
        fr(h)


def pbr_to_csr(pbr: dict):
    """Expand PBR arrays (as returned by :func:`csr_to_pbr`) back to CSR."""
    itype = pbr["block_coords"].dtype
    stype = pbr["block_data"].dtype
    rows, cols = pbr["rows"], pbr["cols"]
    nnz = len(pbr["block_data"]) + len(pbr["remainder_data"])
    indptr = np.zeros(rows + 1, itype)
    indices = np.zeros(max(nnz, 1), itype)
    vals = np.zeros(max(nnz, 1), stype)
    # Rebuild the block/remainder arrays into the oracle's internal form via a
    # round trip through the reference semantics: expand in numpy directly.
    r_list, c_list, v_list = expand_pbr_coo(pbr)
    order = np.lexsort((v_list, c_list, r_list))
    r_list, c_list, v_list = r_list[order], c_list[order], v_list[order]
    counts = np.bincount(r_list, minlength=rows) if rows else np.zeros(0, np.int64)
    indptr[1:] = np.cumsum(counts)
    n = len(r_list)
    indices[:n] = c_list
    vals[:n] = v_list
    return indptr, indices[:n], vals[:n]


def expand_pbr_coo(pbr: dict):
    """PBR arrays -> COO triplets (row, col, value), blocks first then remainder.

    Block values pair with set bits in row-major bit order, the order the
    reference SpMM walks them (``pbr_matrix.cpp:38-57``).
    """
    br, bc = pbr["block_rows"], pbr["block_cols"]
    codes = pbr["block_codes"].astype(np.uint64)
    nb = len(codes)
    bits = np.arange(br * bc, dtype=np.uint64)
    setmask = ((codes[:, None] >> bits[None, :]) & np.uint64(1)).astype(bool) if nb else \
        np.zeros((0, br * bc), bool)
    blk, bit = np.nonzero(setmask)
    coords = pbr["block_coords"].astype(np.int64).reshape(-1, 2)
    r = coords[blk, 0] + bit // bc
    c = coords[blk, 1] + bit % bc
    # The k-th set bit overall takes block_data[k] (blocks are contiguous).
    v = pbr["block_data"][: len(blk)]
    ri = pbr["remainder_indptr"].astype(np.int64)
    rr = np.repeat(np.arange(pbr["rows"], dtype=np.int64), np.diff(ri))
    rc = pbr["remainder_col_ind"].astype(np.int64)
    rv = pbr["remainder_data"]
    return (np.concatenate([r, rr]).astype(np.int64), np.concatenate([c, rc]).astype(np.int64),
            np.concatenate([v, rv]))


def bucket_chain(hint: int, max_elems: int) -> np.ndarray:
    """(element count, bucket count) transitions of the standard library's
    unordered_map built with ``hint`` and filled one key at a time."""
    lib = _load()
    f = lib.oracle_bucket_chain
    f.restype = ctypes.c_int64
    f.argtypes = [ctypes.c_uint64, ctypes.c_int64, ctypes.c_void_p, ctypes.c_int64]
    buf = np.zeros(2 * 256, np.int64)
    n = f(hint, max_elems, _ptr(buf), 256)
    return buf[: 2 * n].reshape(-1, 2)
