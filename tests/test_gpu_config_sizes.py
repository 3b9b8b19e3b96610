"""Parity at the sizes the engine is measured on.

* SpMM configuration (n = 2^20 clustered R-MAT, PBR 8x8 min 8): the device
  build bit-exact against the oracle's restatement of the reference builder
  (``pbr_matrix.cpp:340-477``), and Y against the FP64 product at relative
  error <= 1e-5 per element (64 FP32 columns).
* Batched PPR configuration (n = 2^22 cluster / Zipf graph, 256 seed sets of
  1-32 seeds, layout from the autotuner, retirement + CUDA graphs): sampled
  columns against FP64 references, L1 <= 1e-6.
* Warm-start configuration (n = 2^21): warm and cold solves against the same
  FP64 references, L1 <= 1e-6 each.
* Serving configuration (cluster / Zipf graphs of 2^16 - 2^20 nodes, 1-64
  seeds, alpha in {.8, .85, .9}, warm start on): a sample of served requests
  against FP64 references.

The FP64 references come from ``oracle.ppr.refine_fp64``: the FP64 power
iteration continued until each column's distance to the exact fixed point is
certified below 1e-9 (the map is an alpha-contraction in L1), so "L1 <= 1e-6"
below is the GPU column's distance to the exact fixed point up to that bound.
"""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

L1_TOL = 1e-6
REF_BOUND = 1e-9


def _fp64_distance(A, dangling, X_gpu: np.ndarray, seed_sets, alphas):
    """L1 distance of each GPU column to its FP64 reference, plus the
    reference's certified bound (columns grouped by alpha)."""
    from oracle.ppr import refine_fp64, teleport_matrix
    n = A.shape[0]
    out = np.zeros(X_gpu.shape[1])
    alphas = np.asarray(alphas, dtype=np.float64)
    for a in np.unique(alphas):
        idx = np.nonzero(alphas == a)[0]
        V = teleport_matrix(n, [seed_sets[i] for i in idx])
        X0 = X_gpu[:, idx].astype(np.float64)
        Xref, cert, _ = refine_fp64(A, X0, V, float(a), dangling, bound=REF_BOUND)
        assert (cert < REF_BOUND).all()
        out[idx] = np.abs(X0 - Xref).sum(axis=0) + cert
    return out


def test_spmm_configuration_full_size_build_and_product(device):
    import oracle
    from oracle.ppr import RowSplitMatrix
    from page_rank_gb300 import graph_link as gl
    from page_rank_gb300 import synth
    g = synth.cluster_rmat_graph(log2n=20, cluster=64, mean_degree=16, p_intra=0.7, seed=2, device=device)
    A = g.A
    n = A.shape[0]
    p = gl.csr_to_pbr(A, block_rows=8, block_cols=8, min_nnz_per_block=8)
    o = oracle.csr_to_pbr(A.indptr, A.indices, A.data, n, n, 8, 8, 8)
    for k in ("block_codes", "block_coords", "block_offsets", "block_data",
              "remainder_indptr", "remainder_col_ind", "remainder_data"):
        a, b = np.asarray(getattr(p, k)), np.asarray(o[k])
        assert a.shape == b.shape, k
        assert np.array_equal(a.view(np.uint8), b.view(np.uint8)), k
    assert p.accounted_blocks() == 873322 and p.compressed_nnz() == 9743813 and p.remainder_nnz() == 5974903

    pd = p.to(device)
    X = torch.rand((n, 64), device=device, generator=torch.Generator(device=device).manual_seed(1234))
    Y = gl.pbr_matmul(pd, X).double().cpu().numpy()
    M = RowSplitMatrix(A.astype(np.float64))
    try:
        Yref = M @ X.double().cpu().numpy()
    finally:
        M.close()
    rel = np.abs(Y - Yref) / np.maximum(np.abs(Yref), 1e-30)
    assert float(rel.max()) <= 1e-5, float(rel.max())


def test_batched_ppr_configuration_sampled_columns(device):
    from page_rank_gb300 import synth
    from page_rank_gb300.autotune import autotune
    from page_rank_gb300.engine import PPREngine
    g = synth.cluster_zipf_graph(log2n=22, mean_degree=20.0, seed=3, device=device)
    K = 256
    sets = synth.seed_sets(g.n, K, 1, 32, seed=11)
    tuned = autotune(g.A, K, device=device)
    eng = PPREngine(g.A, block_size=tuned.block_size, min_nnz_per_block=tuned.min_nnz, device=device,
                    dangling=g.dangling, column_tile=tuned.column_tile)
    r = eng.solve(sets, alpha=0.85, tol=L1_TOL, retire=True, use_graphs=True)
    assert r.converged.all()
    cols = np.sort(np.random.default_rng(0).choice(K, 8, replace=False))
    X = r.X[:, torch.from_numpy(cols).to(device)].double().cpu().numpy()
    d = _fp64_distance(g.A, g.dangling, X, [sets[c] for c in cols], [0.85] * len(cols))
    assert (d <= L1_TOL).all(), d


def test_warm_start_configuration_warm_and_cold_against_fp64(device):
    """The window-solve start (the product's warm start) and the cold start
    on the 2^21-node configuration: both within the certified L1 of the FP64
    fixed point, the start with at least 1.5x fewer power iterations."""
    from page_rank_gb300 import synth
    from page_rank_gb300.engine import PPREngine
    from page_rank_gb300.window_start import WindowStart
    g = synth.cluster_zipf_graph(log2n=21, mean_degree=20.0, seed=3, device=device)
    eng = PPREngine(g.A, block_size=4, min_nnz_per_block=4, device=device, dangling=g.dangling)
    ws = WindowStart(eng)
    sets = synth.seed_sets(g.n, 8, 1, 32, seed=424242)
    cold = eng.solve(sets, tol=L1_TOL)
    warm = ws.solve(sets, tol=L1_TOL)
    assert cold.converged.all() and warm.converged.all() and warm.warm_columns.all()
    assert cold.iterations.mean() >= 1.5 * warm.iterations.mean()
    for res in (cold, warm):
        d = _fp64_distance(g.A, g.dangling, res.X.double().cpu().numpy(), sets, [0.85] * len(sets))
        assert (d <= L1_TOL).all(), d


def test_serving_configuration_sampled_requests_against_fp64(device):
    from page_rank_gb300 import synth
    from page_rank_gb300.serving import PPRServer
    from page_rank_gb300.warmstart import WarmStartGate
    from page_rank_gb300.window_start import WindowStart
    graphs = {f"g{i}": synth.cluster_zipf_graph(log2n=lg, mean_degree=20.0, seed=200 + i, device=device)
              for i, lg in enumerate((16, 18, 20))}
    srv = PPRServer(device=device, chunk=8)
    for name, g in graphs.items():
        eng = srv.add_graph(name, g.A, dangling=g.dangling, block_size=8, min_nnz=4)
        srv.warm[name] = WindowStart(eng, gate=WarmStartGate())
    rng = np.random.default_rng(7)
    reqs = []
    for wave in range(4):                     # requests arrive while others are on the GPU
        for _ in range(6):
            name = f"g{rng.integers(0, len(graphs))}"
            seeds = rng.choice(graphs[name].n, size=int(rng.integers(1, 65)), replace=False)
            reqs.append(srv.submit(name, seeds, alpha=float(rng.choice([0.8, 0.85, 0.9])), tol=L1_TOL))
        srv.step()
    srv.run_until_idle()
    assert all(r.done.is_set() and r.converged for r in reqs)
    for r in reqs[::4]:
        g = graphs[r.graph]
        d = _fp64_distance(g.A, g.dangling, r.result.double().numpy()[:, None], [r.seeds], [r.alpha])
        assert d[0] <= L1_TOL, (r.rid, r.graph, d[0])
