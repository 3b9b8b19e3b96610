"""Batched engine: seed-set columns, dangling mass to the teleport vector,
per-column retirement, CUDA-graph chunks — against the FP64 oracle."""
import numpy as np
import pytest
import torch

from oracle import ppr as oppr

pytestmark = pytest.mark.gpu


def _small_graph(seed=3):
    from page_rank_gb300 import synth
    return synth.cluster_zipf_graph(log2n=12, mean_degree=6.0, seed=seed)


def test_config1_sbm_dangling_to_personalization(device):
    """n=4096 SBM (64 x 64, p_in .1, p_out 5e-4), one seed set of 5 nodes,
    alpha .85, 100 iterations, tol 1e-8, PBR 4x4 min 4; FP32 GPU vs the
    FP64 fixed point."""
    from page_rank_gb300 import synth
    from page_rank_gb300.engine import PPREngine
    g = synth.sbm_graph(64, 64, 0.1, 0.0005, seed=1)
    seeds = np.sort(np.random.default_rng(5).choice(g.n, 5, replace=False))
    eng = PPREngine(g.A, block_size=4, min_nnz_per_block=4, device=device, dangling=g.dangling)
    res = eng.solve([seeds], alpha=0.85, tol=1e-8, max_iterations=100, certified=False, retire=False)
    V = oppr.teleport_matrix(g.n, [seeds])
    X64 = oppr.direct_solve_fp64(g.A, V, 0.85, g.dangling)
    Xp, it, conv, _ = oppr.power_iteration_fp64(g.A, V, 0.85, 100, 1e-8, g.dangling)
    got = res.X.cpu().numpy().astype(np.float64)
    l1 = np.abs(got - X64).sum()
    assert l1 <= 1e-6, l1
    assert np.abs(got - Xp).sum() <= 1e-6
    assert abs(got.sum() - 1.0) < 1e-5


@pytest.mark.parametrize("retire", [False, True])
@pytest.mark.parametrize("graphs", [False, True])
def test_batched_seed_sets_certified(retire, graphs, device):
    from page_rank_gb300 import synth
    from page_rank_gb300.engine import PPREngine
    g = _small_graph()
    sets = synth.seed_sets(g.n, 37, 1, 32, seed=9)
    eng = PPREngine(g.A, block_size=8, min_nnz_per_block=4, device=device, dangling=g.dangling)
    res = eng.solve(sets, alpha=0.85, tol=1e-6, max_iterations=400, retire=retire, use_graphs=graphs)
    assert res.converged.all()
    V = oppr.teleport_matrix(g.n, sets)
    X64 = oppr.direct_solve_fp64(g.A, V, 0.85, g.dangling)
    l1 = np.abs(res.X.cpu().numpy().astype(np.float64) - X64).sum(axis=0)
    assert l1.max() <= 1e-6, l1.max()


def test_retirement_reduces_column_steps(device):
    from page_rank_gb300 import synth
    from page_rank_gb300.engine import PPREngine
    g = _small_graph(seed=4)
    sets = synth.seed_sets(g.n, 64, 1, 32, seed=2)
    eng = PPREngine(g.A, block_size=4, device=device, dangling=g.dangling)
    a = eng.solve(sets, alpha=0.9, tol=1e-6, retire=False)
    b = eng.solve(sets, alpha=0.9, tol=1e-6, retire=True)
    assert b.column_steps < a.column_steps
    d = np.abs(a.X.cpu().numpy().astype(np.float64) - b.X.cpu().numpy()).sum(axis=0)
    assert d.max() <= 2e-6


def test_plain_matches_batched(device):
    from page_rank_gb300 import synth
    from page_rank_gb300.engine import PPREngine
    g = _small_graph(seed=6)
    sets = synth.seed_sets(g.n, 5, 1, 8, seed=3)
    eng = PPREngine(g.A, block_size=8, device=device, dangling=g.dangling)
    a = eng.solve_plain(sets, tol=1e-6)
    b = eng.solve(sets, tol=1e-6)
    d = np.abs(a.X.cpu().numpy().astype(np.float64) - b.X.cpu().numpy()).sum(axis=0)
    assert d.max() <= 2e-6


def test_uniform_dangling_matches_dense_normalization(device):
    """The in-kernel uniform redistribution reaches the fixed point of the
    reference's dense normalize_transition_matrix."""
    import scipy.sparse as sp
    from page_rank_gb300 import graph_link as gl
    from page_rank_gb300 import native
    from page_rank_gb300.engine import _bitmap_from_mask
    from page_rank_gb300.ppr import PprRun, teleport_from_seed_sets
    from page_rank_gb300.transition import normalize_columns
    rng = np.random.default_rng(0)
    n = 300
    M = (rng.random((n, n)) < 0.02).astype(np.float32)
    M[:, rng.integers(0, n, 20)] = 0
    A = sp.csr_matrix(M)
    dense = gl.normalize_transition_matrix(A)
    sparse_norm, dmask = normalize_columns(A)
    V = oppr.teleport_matrix(n, [[3], [77]])
    want = oppr.direct_solve_fp64(dense, V, 0.85)
    pbr = gl.csr_to_pbr(sparse_norm, 4, 4, 2).to(device)
    meta = gl.get_pbr_gpu_meta(pbr)
    tp = teleport_from_seed_sets(torch.arange(3, dtype=torch.int32, device=device),
                                 torch.tensor([3, 77], dtype=torch.int32, device=device), n, 4)
    run = PprRun(meta, n, n, 4, 4, tp, 0.85, 500, 1e-9, native.GL_PPR_STOP_ALL,
                 _bitmap_from_mask(dmask, device), native.GL_DANGLING_UNIFORM)
    r = run.run()
    assert r.converged
    assert np.abs(r.X.cpu().numpy() - want).sum(axis=0).max() < 1e-6
