"""Generate the golden fixtures in this directory from the reference itself.

Run in a checkout that has the reference sources (read-only) and its builder
compiled into ``oracle/_ref`` (``python oracle/ref_build.py``)::

    python tests/golden/make_golden.py

Writes:
* ``builder_cases.npz`` — CSR inputs and the reference ``csr_to_pbr`` output
  (``Backend/graph_link/pbr_matrix/pbr_matrix.cpp:340-477``) for small edge
  cases: ragged stripes, empty rows / matrices, int64 indices, float64 values,
  min_nnz 0 / above 64, and a stripe wide enough to rehash the builder's map;
* ``normalize_cases.npz`` — the reference ``normalize_transition_matrix``
  (``Backend/graph_link/graph_link/__init__.py:184-207``) on graphs with
  dangling nodes;
* ``ppr_nx_cases.npz`` — the NetworkX PPR values the reference's accuracy
  test compares against (``Tests/test_ppr_accuracy.py:14-40``), with the
  column-stochastic matrices they come from, so GPU machines without
  NetworkX can run that test.
"""
from __future__ import annotations

import importlib.util
import sys
from pathlib import Path

import numpy as np
import scipy.sparse as sp

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
sys.path.insert(0, str(ROOT))

from oracle import ref_build  # noqa: E402

KEYS = ["block_codes", "block_coords", "block_offsets", "block_data",
        "remainder_indptr", "remainder_col_ind", "remainder_data"]


def _reference_normalize():
    path = ref_build.REF_SRC / "graph_link" / "__init__.py"
    src = path.read_text()
    # Only the pure-scipy normalize function is needed; extract its source so
    # the reference package (which needs its CUDA module) is not imported.
    start = src.index("def normalize_transition_matrix")
    end = src.index("def run_personalized_pagerank")
    ns: dict = {"np": np, "sp": sp}
    exec(compile(src[start:end], str(path), "exec"), ns)
    return ns["normalize_transition_matrix"]


def builder_cases():
    rng = np.random.default_rng(20261203)
    cases = []

    def add(name, A, br, bc, mn):
        cases.append((name, A, br, bc, mn))

    for br in (2, 4, 8):
        for mn in (1, 4):
            A = sp.random(64, 64, density=0.15, format="csr", dtype=np.float32,
                          random_state=int(rng.integers(1 << 30)))
            add(f"rand64_b{br}_m{mn}", A, br, br, mn)
    add("ragged_rows_37x53_b4", sp.random(37, 53, density=0.2, format="csr", dtype=np.float32,
                                          random_state=3), 4, 4, 2)
    add("ragged_rows_101x101_b8", sp.random(101, 101, density=0.1, format="csr", dtype=np.float32,
                                            random_state=4), 8, 8, 3)
    add("rect_blocks_2x8", sp.random(96, 96, density=0.1, format="csr", dtype=np.float32,
                                     random_state=5), 2, 8, 2)
    add("empty_matrix", sp.csr_matrix((40, 40), dtype=np.float32), 4, 4, 1)
    E = sp.random(64, 64, density=0.2, format="lil", dtype=np.float32, random_state=6)
    E[10:30, :] = 0
    add("empty_rows", sp.csr_matrix(E), 4, 4, 2)
    A = sp.random(80, 80, density=0.1, format="csr", dtype=np.float32, random_state=7)
    A64 = sp.csr_matrix((A.data, A.indices.astype(np.int64), A.indptr.astype(np.int64)), shape=A.shape)
    add("int64_index", A64, 4, 4, 2)
    add("float64_values", sp.random(80, 80, density=0.1, format="csr", dtype=np.float64,
                                    random_state=8), 8, 8, 2)
    add("min_nnz_0", sp.random(64, 64, density=0.05, format="csr", dtype=np.float32,
                               random_state=9), 4, 4, 0)
    add("min_nnz_65", sp.random(64, 64, density=0.5, format="csr", dtype=np.float32,
                                random_state=10), 8, 8, 65)
    # one wide stripe with hundreds of blocks: the builder's map rehashes
    W = sp.random(16, 8192, density=0.08, format="csr", dtype=np.float32, random_state=11)
    add("wide_rehash", W, 8, 8, 1)
    return cases


def main():
    core = ref_build.load_reference_core()
    if core is None:
        raise SystemExit("build the reference first: python oracle/ref_build.py")
    out = {}
    names = []
    for name, A, br, bc, mn in builder_cases():
        p = core.csr_to_pbr(A.indptr, A.indices, A.data, A.shape[0], A.shape[1], br, bc, mn)
        names.append(name)
        out[f"{name}/indptr"] = A.indptr
        out[f"{name}/indices"] = A.indices
        out[f"{name}/data"] = A.data
        out[f"{name}/meta"] = np.array([A.shape[0], A.shape[1], br, bc, mn, p.total_nnz], np.int64)
        for k in KEYS:
            out[f"{name}/{k}"] = np.asarray(getattr(p, k))
    out["names"] = np.array(names)
    np.savez_compressed(HERE / "builder_cases.npz", **out)

    normalize = _reference_normalize()
    norm = {}
    rng = np.random.default_rng(7)
    for i, (n, p) in enumerate([(30, 0.08), (64, 0.03), (50, 0.1)]):
        M = (rng.random((n, n)) < p).astype(np.float32) * rng.random((n, n)).astype(np.float32)
        M[:, rng.integers(0, n, 3)] = 0.0   # force dangling columns
        A = sp.csr_matrix(M)
        An = normalize(A)
        norm[f"c{i}/indptr"], norm[f"c{i}/indices"], norm[f"c{i}/data"] = A.indptr, A.indices, A.data
        norm[f"c{i}/shape"] = np.array(A.shape)
        norm[f"c{i}/out_indptr"], norm[f"c{i}/out_indices"] = An.indptr, An.indices
        norm[f"c{i}/out_data"] = An.data
    norm["count"] = np.array(3)
    np.savez_compressed(HERE / "normalize_cases.npz", **norm)

    import networkx as nx
    ppr = {}
    for (N, p) in [(50, 0.10), (100, 0.05)]:
        G = nx.erdos_renyi_graph(N, p, directed=True, seed=42)
        A_nx = nx.to_scipy_sparse_array(G, nodelist=range(N), format="csr", dtype=np.float32)
        A_col = sp.csr_matrix(A_nx.T)
        An = normalize(A_col)
        key = f"N{N}"
        ppr[f"{key}/indptr"], ppr[f"{key}/indices"], ppr[f"{key}/data"] = An.indptr, An.indices, An.data
        for alpha in (0.85, 0.90):
            for src in (0, N // 4, N // 2, N - 1):
                pers = {n: (1.0 if n == src else 0.0) for n in range(N)}
                dang = {n: 1.0 / N for n in range(N)}
                sc = nx.pagerank(G, alpha=alpha, personalization=pers, dangling=dang, tol=1e-6, max_iter=500)
                ppr[f"{key}/a{alpha}/s{src}"] = np.array([sc[n] for n in range(N)], np.float32)
    np.savez_compressed(HERE / "ppr_nx_cases.npz", **ppr)
    print("wrote", sorted(p.name for p in HERE.glob("*.npz")))


if __name__ == "__main__":
    main()
