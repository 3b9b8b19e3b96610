"""Fused power-iteration PPR against NetworkX (golden values, the reference's
own accuracy test) and against the FP64 oracle."""
import numpy as np
import pytest
import scipy.sparse as sp
import torch

from oracle import ppr as oppr
from tests._cases import GOLDEN

pytestmark = pytest.mark.gpu

NX = np.load(GOLDEN / "ppr_nx_cases.npz")


def _gl():
    from page_rank_gb300 import graph_link
    return graph_link


def _nx_matrix(N):
    k = f"N{N}"
    return sp.csr_matrix((NX[f"{k}/data"], NX[f"{k}/indices"], NX[f"{k}/indptr"]), shape=(N, N))


@pytest.mark.parametrize("N", [50, 100])
@pytest.mark.parametrize("alpha", [0.85, 0.90])
@pytest.mark.parametrize("block_size", [2, 4, 8])
@pytest.mark.parametrize("min_nnz", [1, 4])
def test_ppr_accuracy_vs_networkx(N, alpha, block_size, min_nnz, device):
    """Tests/test_ppr_accuracy.py:58-96 with the NetworkX values as fixtures."""
    A = _nx_matrix(N)
    sources = [0, N // 4, N // 2, N - 1]
    pbr = _gl().csr_to_pbr(A, block_rows=block_size, block_cols=block_size,
                           min_nnz_per_block=min_nnz).to(device)
    X, _, converged = _gl().run_personalized_pagerank(
        pbr, torch.tensor(sources, dtype=torch.int32, device=device), alpha=alpha,
        max_iterations=500, tolerance=1e-6)
    assert converged
    X = X.cpu().numpy()
    for k, src in enumerate(sources):
        col = X[:, k]
        ref = NX[f"N{N}/a{alpha}/s{src}"]
        assert np.isclose(col.sum(), 1.0, atol=1e-4)
        assert np.allclose(col, ref, atol=1e-3)


@pytest.mark.parametrize("block_size", [2, 4, 8])
def test_ppr_matches_fp64_power_iteration(block_size, device):
    """Same update and stop rule as the reference loop: same iteration count,
    and the FP32 result within 1e-6 L1 per column of the FP64 iterate."""
    A = _nx_matrix(100)
    sources = [3, 17, 42, 99, 0]
    V = oppr.teleport_matrix(100, [[s] for s in sources])
    X64, it64, conv64, hist64 = oppr.power_iteration_fp64(A, V, 0.85, 200, 1e-6)
    pbr = _gl().csr_to_pbr(A, block_size, block_size, 2).to(device)
    X, it, conv, hist = _gl().run_personalized_pagerank(
        pbr, torch.tensor(sources, dtype=torch.int32, device=device), alpha=0.85,
        max_iterations=200, tolerance=1e-6, return_history=True)
    assert conv and conv64
    assert abs(it - it64) <= 1
    assert len(hist) == it
    l1 = np.abs(X.cpu().numpy().astype(np.float64) - X64).sum(axis=0)
    assert l1.max() <= 1e-6, l1


def test_ppr_not_converged_and_zero_iterations(device):
    gl = _gl()
    A = _nx_matrix(50)
    pbr = gl.csr_to_pbr(A, 4, 4, 1).to(device)
    src = torch.tensor([1, 2], dtype=torch.int32, device=device)
    X, it, conv, hist = gl.run_personalized_pagerank(pbr, src, max_iterations=3, tolerance=1e-12,
                                                     return_history=True)
    assert it == 3 and not conv and len(hist) == 3
    X0, it0, conv0 = gl.run_personalized_pagerank(pbr, src, max_iterations=0)
    assert it0 == 0 and not conv0
    e = np.zeros((50, 2), np.float32)
    e[1, 0] = e[2, 1] = 1.0
    assert np.array_equal(X0.cpu().numpy(), e)


def test_ppr_int64_sources_and_bad_source(device):
    gl = _gl()
    pbr = gl.csr_to_pbr(_nx_matrix(50), 2, 2, 1).to(device)
    X, it, conv = gl.run_personalized_pagerank(pbr, torch.tensor([0, 5], device=device))
    assert conv
    with pytest.raises(ValueError):
        gl.run_personalized_pagerank(pbr, torch.tensor([50], dtype=torch.int32, device=device))


def test_ppr_float64_matrix(device):
    gl = _gl()
    A = _nx_matrix(50).astype(np.float64)
    pbr = gl.csr_to_pbr(A, 4, 4, 1).to(device)
    X, it, conv = gl.run_personalized_pagerank(pbr, torch.tensor([7], dtype=torch.int32, device=device),
                                               tolerance=1e-10, max_iterations=500)
    assert X.dtype == torch.float64 and conv
    V = oppr.teleport_matrix(50, [[7]])
    X64 = oppr.direct_solve_fp64(A, V, 0.85)
    assert np.abs(X.cpu().numpy() - X64).sum() < 1e-8


@pytest.mark.parametrize("K", [4, 40, 200])
def test_ppr_per_column_alpha_matches_scalar_runs(K, device):
    """Columns with their own alpha / certified threshold in one fused run
    give bit for bit the vectors of runs where every column has that alpha,
    and each is within L1 1e-6 of its FP64 fixed point."""
    from page_rank_gb300 import native, synth
    from page_rank_gb300.engine import PPREngine, certified_tolerance
    from page_rank_gb300.ppr import PprRun, teleport_from_seed_sets
    g = synth.cluster_zipf_graph(log2n=12, mean_degree=8.0, seed=3)
    n = g.n
    eng = PPREngine(g.A, block_size=4, min_nnz_per_block=4, device=device, dangling=g.dangling)
    rng = np.random.default_rng(7)
    sets = [rng.choice(n, size=int(rng.integers(1, 6)), replace=False) for _ in range(K)]
    alphas = np.array([(0.8, 0.85, 0.9)[k % 3] for k in range(K)])
    thr = np.array([certified_tolerance(1e-6, a) for a in alphas])

    def run(alpha, tol):
        ptr, rows, w = eng.teleport(sets)
        tp = teleport_from_seed_sets(ptr, rows, n, 4, w)
        r = PprRun(eng.meta, n, n, 4, 4, tp, alpha, 1000, tol, native.GL_PPR_STOP_PER_COLUMN, eng.dbits)
        return r.run(chunk=8)

    mixed = run(alphas, thr)
    assert mixed.converged
    for a in (0.8, 0.85, 0.9):
        single = run(a, certified_tolerance(1e-6, a))
        cols = np.nonzero(alphas == a)[0]
        assert torch.equal(mixed.X[:, cols], single.X[:, cols])
    V = oppr.teleport_matrix(n, sets)
    X = mixed.X.cpu().numpy().astype(np.float64)
    for a in (0.8, 0.85, 0.9):
        cols = np.nonzero(alphas == a)[0]
        want, _, ok, _ = oppr.power_iteration_fp64(g.A, V[:, cols], a, 5000, 1e-14, g.dangling)
        assert ok
        assert np.abs(X[:, cols] - want).sum(axis=0).max() <= 1e-6


@pytest.mark.parametrize("stop_mode", ["all", "per_column"])
@pytest.mark.parametrize("warm", [False, True])
def test_library_run_loop_matches_the_host_loop(stop_mode, warm, device):
    """gl_ppr_run (the loop inside the library) against PprRun.run (the host
    loop over gl_ppr_step): same iterations, same vectors bit for bit."""
    from page_rank_gb300 import native, synth
    from page_rank_gb300.graph_link.pbr_registry import get_pbr_gpu_meta
    from page_rank_gb300.ppr import PprRun, dangling_bitmap, teleport_from_seed_sets
    g = synth.cluster_zipf_graph(log2n=13, mean_degree=12.0, seed=4)
    from page_rank_gb300 import graph_link as gl
    pbr = gl.csr_to_pbr(g.A, block_rows=4, block_cols=4, min_nnz_per_block=4).to(device)
    meta = get_pbr_gpu_meta(pbr)
    sets = synth.seed_sets(g.n, 11, 1, 9, seed=5)
    ptr = torch.tensor(np.concatenate([[0], np.cumsum([len(s) for s in sets])]), dtype=torch.int32, device=device)
    idx = torch.tensor(np.concatenate(sets), dtype=torch.int32, device=device)
    tp = teleport_from_seed_sets(ptr, idx, g.n, 4)
    dbits = dangling_bitmap(torch.from_numpy(g.A.indices.astype(np.int32)).to(device), g.n)
    mode = native.GL_PPR_STOP_ALL if stop_mode == "all" else native.GL_PPR_STOP_PER_COLUMN
    x0 = None
    if warm:
        x0 = torch.rand((g.n, len(sets)), device=device, generator=torch.Generator(device=device).manual_seed(1))
        x0 /= x0.sum(dim=0, keepdim=True)
    runs = [PprRun(meta, g.n, g.n, 4, 4, tp, 0.85, 300, 1e-7, mode, dbits) for _ in range(2)]
    a = runs[0].run(chunk=8, x0=x0)
    b = runs[1].run_native(chunk=8, x0=x0)
    assert a.converged and b.converged and a.iterations == b.iterations
    assert torch.equal(a.X, b.X)
    if mode == native.GL_PPR_STOP_PER_COLUMN:
        assert np.array_equal(a.column_iterations, b.column_iterations)
