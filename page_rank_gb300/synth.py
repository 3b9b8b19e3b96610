"""Seeded synthetic graphs for the workloads the engine is measured on.

No dataset ships with the reference (its Wikipedia inputs are not part of the
checkout), so every workload is a seeded synthetic graph with the stated
shape.  Graphs are returned as column-stochastic CSR transition matrices
``A[target, source] = multiplicity / out_degree(source)`` (duplicate edges
summed), i.e. ``normalize_transition_matrix`` without the dense dangling
columns; dangling sources simply have empty columns.

* :func:`sbm_graph`      — stochastic block model (64 x 64, p_in 0.1, p_out 5e-4)
* :func:`cluster_rmat_graph` — 2**20 nodes in clusters of 64, mean out-degree
  16, 70% uniform in-cluster targets, 30% R-MAT (0.57, 0.19, 0.19, 0.05)
* :func:`cluster_zipf_graph` — Zipf(2.1) out-degrees scaled so the mean
  distinct out-degree is the stated one, 80% of a node's edges to distinct
  targets inside its 64-node cluster
* :func:`seed_sets`      — per-column uniform seed sets of random sizes
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np
import scipy.sparse as sp


@dataclass
class Graph:
    """Column-stochastic transition matrix plus bookkeeping."""

    A: sp.csr_matrix          # float32, canonical CSR
    n: int
    dangling: np.ndarray      # bool [n]: sources without out-edges
    description: str


def edges_to_transition(src: np.ndarray, dst: np.ndarray, n: int, description: str,
                        device=None) -> Graph:
    """Sum duplicate edges and normalize columns by out-degree.

    With ``device`` (a CUDA torch device) the sort / dedup runs there; the
    result is the same canonical CSR either way."""
    src = np.asarray(src, dtype=np.int64)
    dst = np.asarray(dst, dtype=np.int64)
    outdeg = np.bincount(src, minlength=n).astype(np.float64)
    if device is not None:
        import torch

        key = torch.from_numpy(dst * n + src).to(device)
        key, counts = torch.unique(key, sorted=True, return_counts=True)
        rows = (key // n)
        cols = (key % n)
        od = torch.from_numpy(outdeg).to(device)
        vals = (counts.to(torch.float64) / od[cols]).to(torch.float32)
        indptr = torch.zeros(n + 1, dtype=torch.int64, device=device)
        indptr[1:] = torch.cumsum(torch.bincount(rows, minlength=n), 0)
        A = sp.csr_matrix((vals.cpu().numpy(), cols.to(torch.int32).cpu().numpy(),
                           indptr.to(torch.int32).cpu().numpy()), shape=(n, n))
        A.has_sorted_indices = True
    else:
        key = dst * n + src
        key, counts = np.unique(key, return_counts=True)
        rows, cols = key // n, key % n
        vals = (counts / outdeg[cols]).astype(np.float32)
        indptr = np.zeros(n + 1, dtype=np.int64)
        indptr[1:] = np.cumsum(np.bincount(rows, minlength=n))
        A = sp.csr_matrix((vals, cols.astype(np.int32), indptr.astype(np.int32)), shape=(n, n))
    return Graph(A=A, n=n, dangling=outdeg == 0, description=description)


def sbm_graph(communities: int = 64, size: int = 64, p_in: float = 0.1, p_out: float = 0.0005,
              seed: int = 1) -> Graph:
    """Directed stochastic block model (every ordered pair drawn independently)."""
    rng = np.random.default_rng(seed)
    n = communities * size
    comm = np.arange(n) // size
    src_list, dst_list = [], []
    for s0 in range(0, n, 512):   # row blocks keep memory small
        s = np.arange(s0, min(n, s0 + 512))
        same = comm[s][:, None] == comm[None, :]
        p = np.where(same, p_in, p_out)
        hit = rng.random((len(s), n)) < p
        np.fill_diagonal(hit[:, s0:s0 + len(s)], False)
        ss, dd = np.nonzero(hit)
        src_list.append(s[ss])
        dst_list.append(dd)
    return edges_to_transition(np.concatenate(src_list), np.concatenate(dst_list), n,
                               f"SBM {communities}x{size} p_in={p_in} p_out={p_out} seed={seed}")


def rmat_targets(rng, m: int, levels: int, a: float, b: float, c: float) -> tuple[np.ndarray, np.ndarray]:
    """m R-MAT (source, target) pairs over 2**levels nodes."""
    src = np.zeros(m, dtype=np.int64)
    dst = np.zeros(m, dtype=np.int64)
    for lvl in range(levels):
        u = rng.random(m)
        right = (u >= a) & (u < a + b) | (u >= a + b + c)      # quadrants b, d: dst bit
        down = u >= a + b                                      # quadrants c, d: src bit
        bit = np.int64(1) << np.int64(levels - 1 - lvl)
        src |= np.where(down, bit, 0)
        dst |= np.where(right, bit, 0)
    return src, dst


def cluster_rmat_edges(log2n: int = 20, cluster: int = 64, mean_degree: int = 16, p_intra: float = 0.7,
                       rmat=(0.57, 0.19, 0.19, 0.05), seed: int = 2) -> tuple[np.ndarray, np.ndarray]:
    """(source, target) edge arrays of :func:`cluster_rmat_graph`, duplicates
    included, in generation order."""
    rng = np.random.default_rng(seed)
    n = 1 << log2n
    m = n * mean_degree
    m_intra = int(round(m * p_intra))
    src_i = rng.integers(0, n, m_intra)
    dst_i = (src_i // cluster) * cluster + rng.integers(0, cluster, m_intra)
    src_r, dst_r = rmat_targets(rng, m - m_intra, log2n, rmat[0], rmat[1], rmat[2])
    return np.concatenate([src_i, src_r]), np.concatenate([dst_i, dst_r])


def cluster_rmat_graph(log2n: int = 20, cluster: int = 64, mean_degree: int = 16, p_intra: float = 0.7,
                       rmat=(0.57, 0.19, 0.19, 0.05), seed: int = 2, device=None) -> Graph:
    src, dst = cluster_rmat_edges(log2n, cluster, mean_degree, p_intra, rmat, seed)
    return edges_to_transition(src, dst, 1 << log2n,
                               f"n=2^{log2n}, clusters of {cluster}, mean out-degree {mean_degree}, "
                               f"{int(p_intra * 100)}% intra-cluster, {100 - int(p_intra * 100)}% "
                               f"R-MAT{tuple(rmat)}, seed={seed}", device=device)


def _zipf_scale(z: np.ndarray, target: float, p_intra: float, cluster: int, n: int) -> float:
    """Scale s for degrees d_i = max(1, round(s z_i)) such that the expected
    number of distinct out-neighbours, min(round(p_intra d_i), cluster) +
    (d_i - round(p_intra d_i)), averages ``target`` (bisection)."""
    def mean_distinct(scale):
        d = np.minimum(np.maximum(1, np.round(z * scale)), n - 1)
        di = np.round(p_intra * d)
        return float((np.minimum(di, cluster) + (d - di)).mean())

    lo, hi = 0.0, target / max(z.mean(), 1e-12)
    while mean_distinct(hi) < target:
        hi *= 2.0
    for _ in range(60):
        mid = 0.5 * (lo + hi)
        if mean_distinct(mid) < target:
            lo = mid
        else:
            hi = mid
    return hi


def cluster_zipf_edges(log2n: int = 22, mean_degree: float = 20.0, zipf_a: float = 2.1, cluster: int = 64,
                       p_intra: float = 0.8, seed: int = 3) -> tuple[np.ndarray, np.ndarray]:
    """(source, target) edges of :func:`cluster_zipf_graph`.

    Out-degrees follow Zipf(zipf_a), scaled so that the mean number of
    *distinct* out-neighbours is ``mean_degree``.  A node's p_intra share of
    its edges goes to distinct targets inside its own ``cluster``-node cluster
    (a random arithmetic progression with an odd step modulo the cluster
    size, at most ``cluster`` of them); the rest go to uniform targets across
    the graph (repeats there are rare and summed)."""
    rng = np.random.default_rng(seed)
    n = 1 << log2n
    z = rng.zipf(zipf_a, n).astype(np.float64)
    z = np.minimum(z, n)           # a single draw can exceed n
    scale = _zipf_scale(z, mean_degree, p_intra, cluster, n)
    deg = np.minimum(np.maximum(1, np.round(z * scale)), n - 1).astype(np.int64)
    k_in = np.minimum(np.round(p_intra * deg).astype(np.int64), cluster)
    k_out = deg - np.round(p_intra * deg).astype(np.int64)
    # intra-cluster targets: base + (offset + j * step) mod cluster, j < k_in
    src_i = np.repeat(np.arange(n, dtype=np.int64), k_in)
    first = np.cumsum(k_in) - k_in
    j = np.arange(src_i.size, dtype=np.int64) - np.repeat(first, k_in)
    offset = rng.integers(0, cluster, n)
    step = 2 * rng.integers(0, cluster // 2, n) + 1
    dst_i = (src_i // cluster) * cluster + (np.repeat(offset, k_in) + j * np.repeat(step, k_in)) % cluster
    src_o = np.repeat(np.arange(n, dtype=np.int64), k_out)
    dst_o = rng.integers(0, n, src_o.size)
    return np.concatenate([src_i, src_o]), np.concatenate([dst_i, dst_o])


def cluster_zipf_graph(log2n: int = 22, mean_degree: float = 20.0, zipf_a: float = 2.1, cluster: int = 64,
                       p_intra: float = 0.8, seed: int = 3, device=None) -> Graph:
    src, dst = cluster_zipf_edges(log2n, mean_degree, zipf_a, cluster, p_intra, seed)
    n = 1 << log2n
    return edges_to_transition(src, dst, n,
                               f"n=2^{log2n}, Zipf({zipf_a}) out-degree, mean distinct out-degree "
                               f"{mean_degree:g}, {int(p_intra * 100)}% of each node's edges to distinct "
                               f"targets in its {cluster}-node cluster, seed={seed}",
                               device=device)


def seed_sets(n: int, k: int, min_size: int = 1, max_size: int = 32, seed: int = 4) -> list[np.ndarray]:
    """k seed sets, sizes uniform in [min_size, max_size], seeds uniform without replacement."""
    rng = np.random.default_rng(seed)
    sizes = rng.integers(min_size, max_size + 1, k)
    return [np.sort(rng.choice(n, size=int(s), replace=False)) for s in sizes]


def seed_csr(sets: list[np.ndarray]) -> tuple[np.ndarray, np.ndarray]:
    ptr = np.zeros(len(sets) + 1, dtype=np.int32)
    ptr[1:] = np.cumsum([len(s) for s in sets])
    idx = np.concatenate(sets).astype(np.int32) if sets else np.zeros(0, np.int32)
    return ptr, idx
