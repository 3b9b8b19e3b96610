"""Shared input generators and comparison helpers for the tests."""
from __future__ import annotations

from pathlib import Path

import numpy as np
import scipy.sparse as sp

GOLDEN = Path(__file__).resolve().parent / "golden"
PBR_KEYS = ["block_codes", "block_coords", "block_offsets", "block_data",
            "remainder_indptr", "remainder_col_ind", "remainder_data"]


def random_csr(n, density, dtype=np.float32, seed=42, m=None):
    """The reference tests' generator (``Tests/test_spmm.py:13-15``)."""
    return sp.random(n, n if m is None else m, density=density, format="csr", dtype=dtype,
                     random_state=np.random.default_rng(seed).integers(2**31))


def random_x(n, f, seed=0):
    """``Tests/test_spmm.py:18-19``."""
    return np.random.default_rng(seed).random((n, f)).astype(np.float32)


def load_builder_cases():
    z = np.load(GOLDEN / "builder_cases.npz")
    out = []
    for name in z["names"]:
        name = str(name)
        rows, cols, br, bc, mn, tot = (int(x) for x in z[f"{name}/meta"])
        A = sp.csr_matrix((z[f"{name}/data"], z[f"{name}/indices"], z[f"{name}/indptr"]),
                          shape=(rows, cols))
        ref = {k: z[f"{name}/{k}"] for k in PBR_KEYS}
        ref["total_nnz"] = tot
        out.append((name, A, br, bc, mn, ref))
    return out


def assert_pbr_equal(got: dict, want: dict, ctx: str = ""):
    """Bit-exact comparison of PBR arrays (values compared as raw bytes)."""
    for k in PBR_KEYS:
        a = np.asarray(got[k])
        b = np.asarray(want[k])
        assert a.shape == b.shape, f"{ctx} {k}: shape {a.shape} != {b.shape}"
        if a.dtype != b.dtype:
            assert a.dtype.kind == b.dtype.kind and a.itemsize == b.itemsize or \
                np.array_equal(a.astype(np.int64), b.astype(np.int64)), f"{ctx} {k}: dtype {a.dtype} vs {b.dtype}"
        if a.dtype.kind == "f":
            assert a.dtype == b.dtype, f"{ctx} {k}: dtype {a.dtype} vs {b.dtype}"
            assert np.array_equal(a.view(np.uint8), b.view(np.uint8)), f"{ctx} {k}: values differ"
        else:
            assert np.array_equal(a.astype(np.uint64) if k == "block_codes" else a,
                                  b.astype(np.uint64) if k == "block_codes" else b), f"{ctx} {k}: differ"


def load_edge_cases():
    """(name, n, source, target, weight, A, An) from edges_cases.npz: the
    reference service's matrix A and its normalize_transition_matrix An."""
    z = np.load(GOLDEN / "edges_cases.npz")
    out = []
    for name in z["names"]:
        name = str(name)
        n = int(z[f"{name}/n"])
        A = sp.csr_matrix((z[f"{name}/A_data"], z[f"{name}/A_indices"], z[f"{name}/A_indptr"]), shape=(n, n))
        An = sp.csr_matrix((z[f"{name}/out_data"], z[f"{name}/out_indices"], z[f"{name}/out_indptr"]),
                           shape=(n, n))
        out.append((name, n, z[f"{name}/source"], z[f"{name}/target"], z[f"{name}/weight"], A, An))
    return out


def without_dense_columns(An: sp.csr_matrix, dangling: np.ndarray) -> sp.csr_matrix:
    """The reference's normalized matrix with its dense 1/N dangling columns
    removed (what the engine stores; it redistributes that mass in-kernel)."""
    A = sp.csr_matrix(An, copy=True)
    A.sort_indices()
    drop = dangling[A.indices]
    rows = np.repeat(np.arange(A.shape[0]), np.diff(A.indptr))
    keep = ~drop
    out = sp.csr_matrix((A.data[keep], (rows[keep], A.indices[keep])), shape=A.shape)
    out.sort_indices()
    return out
