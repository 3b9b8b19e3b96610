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
* ``edges_cases.npz`` — the reference service's edge list -> matrix step
  (``Backend/server/app.py:111-131``: edges with unknown endpoints or a
  non-finite / non-positive weight skipped, ``A[target, source] = weight``
  in FP32 with duplicates summed by scipy) followed by the reference
  ``normalize_transition_matrix``, on edge lists with invalid edges,
  duplicates (equal weights, or at most two copies, or short rows), long
  columns and empty graphs;
* ``pbr_to_csr_cases.npz`` — the reference ``pbr_to_csr``
  (``Backend/graph_link/pbr_matrix/pbr_matrix.cpp:289-338``) applied to the
  reference builder's output for every builder case whose row count is a
  multiple of the block height (the reference throws on the others);
  ``python tests/golden/make_golden.py --only pbr_to_csr`` writes just this
  file;
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


def reference_edge_matrix(n, source, target, weight):
    """The reference service's step from indexed edges to ``A``
    (``app.py:111-131``), with -1 standing for an id that is not a node."""
    rows, cols, data = [], [], []
    for s, t, w in zip(source, target, weight):
        if s < 0 or t < 0 or not np.isfinite(w) or w <= 0:
            continue
        rows.append(int(t))
        cols.append(int(s))
        data.append(float(w))
    return sp.csr_matrix((np.asarray(data, dtype=np.float32),
                          (np.asarray(rows, dtype=np.int64), np.asarray(cols, dtype=np.int64))),
                         shape=(n, n))


def edge_cases():
    """(name, n, source, target, weight) lists whose duplicate sums do not
    depend on the order scipy's per-row sort leaves them in."""
    rng = np.random.default_rng(20261204)
    cases = []
    n = 60
    m = 700
    s, t = rng.integers(-1, n, m), rng.integers(-1, n, m)
    w = rng.choice([1.0, 1.0, 1.0, 2.0, 0.0, -3.0, np.inf, np.nan], m)
    cases.append(("invalid_and_equal_weight_dups", n, s, t, w))
    n = 80
    pairs = np.unique(rng.integers(0, n, (900, 2)), axis=0)
    rng.shuffle(pairs)
    twice = pairs[rng.random(len(pairs)) < 0.4]
    e = np.concatenate([pairs, twice])
    perm = rng.permutation(len(e))
    cases.append(("two_copies_distinct_weights", n, e[perm, 0], e[perm, 1], rng.random(len(e)) * 4 + 1e-3))
    n = 50
    s = rng.integers(0, n, 300)
    t = rng.integers(0, n, 300)
    t[:40] = 7
    s[:40] = rng.integers(0, 3, 40)    # row 7: 40 entries over 3 columns...
    keep = (t != 7) | (np.arange(300) < 12)  # ...cut to 12 so the row stays short
    cases.append(("short_rows_many_copies", n, s[keep], t[keep], rng.random(keep.sum()) * 3 + 0.5))
    n = 2000
    m = 6000
    s = np.concatenate([np.full(1500, 5), rng.integers(0, n, m)])   # column 5: ~1500 entries
    t = np.concatenate([rng.permutation(n)[:1500], rng.integers(0, n, m)])
    key = np.unique(np.stack([s, t], 1), axis=0, return_index=True)[1]
    key.sort()
    cases.append(("long_column_pairwise", n, s[key], t[key], rng.random(key.size) * 2 + 0.01))
    cases.append(("no_edges", 5, np.zeros(0, np.int64), np.zeros(0, np.int64), np.zeros(0)))
    cases.append(("single_self_loop", 1, np.array([0]), np.array([0]), np.array([2.5])))
    cases.append(("all_invalid", 4, np.array([0, -1, 2]), np.array([1, 1, -1]), np.array([-1.0, 1.0, 1.0])))
    cases.append(("tiny_weights", 6, np.array([0, 1, 2, 2]), np.array([1, 2, 3, 4]),
                  np.array([1e-300, 1e-44, 3.0, 1e-30])))
    return cases


def pbr_to_csr_cases(core):
    """The reference pbr_to_csr on the reference builder's PBR of each builder
    case (cases with a ragged last stripe are left out: it throws there)."""
    out = {}
    names = []
    for name, A, br, bc, mn in builder_cases():
        if A.shape[0] % br != 0:
            continue
        p = core.csr_to_pbr(A.indptr, A.indices, A.data, A.shape[0], A.shape[1], br, bc, mn)
        indptr = np.zeros(A.shape[0] + 1, A.indptr.dtype)
        indices = np.zeros(A.nnz, A.indices.dtype)
        data = np.zeros(A.nnz, A.data.dtype)
        core.pbr_to_csr(p, indptr, indices, data)
        names.append(name)
        out[f"{name}/out_indptr"], out[f"{name}/out_indices"], out[f"{name}/out_data"] = indptr, indices, data
    out["names"] = np.array(names)
    np.savez_compressed(HERE / "pbr_to_csr_cases.npz", **out)


def main():
    core = ref_build.load_reference_core()
    if core is None:
        raise SystemExit("build the reference first: python oracle/ref_build.py")
    if "--only" in sys.argv and sys.argv[sys.argv.index("--only") + 1] == "pbr_to_csr":
        pbr_to_csr_cases(core)
        print("wrote pbr_to_csr_cases.npz")
        return
    pbr_to_csr_cases(core)
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

    edges = {}
    names = []
    for name, n, src, dst, w in edge_cases():
        A = reference_edge_matrix(n, src, dst, w)
        An = normalize(A)
        names.append(name)
        edges[f"{name}/n"] = np.array(n)
        edges[f"{name}/source"] = np.asarray(src, np.int64)
        edges[f"{name}/target"] = np.asarray(dst, np.int64)
        edges[f"{name}/weight"] = np.asarray(w, np.float64)
        edges[f"{name}/A_indptr"], edges[f"{name}/A_indices"] = A.indptr, A.indices
        edges[f"{name}/A_data"] = A.data
        edges[f"{name}/out_indptr"], edges[f"{name}/out_indices"] = An.indptr, An.indices
        edges[f"{name}/out_data"] = An.data
    edges["names"] = np.array(names)
    np.savez_compressed(HERE / "edges_cases.npz", **edges)

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
