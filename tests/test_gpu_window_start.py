"""The window-solve warm start on the device against its FP64 oracle:
window inverses, the fused window apply (every column count, ragged row
counts, both near-field modes and the per-window column sums), start
vectors, exact cold residuals, the per-column fallback, and warm-started
solves that reach the same fixed point in fewer iterations."""
import numpy as np
import pytest
import scipy.sparse as sp
import torch

from oracle import ppr as oppr
from oracle import window_start as ows

pytestmark = pytest.mark.gpu


def _csr_dev(A, device):
    A = sp.csr_matrix(A, dtype=np.float32)
    A.sort_indices()
    return (torch.from_numpy(A.indptr.astype(np.int32)).to(device),
            torch.from_numpy(A.indices.astype(np.int32)).to(device),
            torch.from_numpy(A.data.astype(np.float32)).to(device))


def _inverses(A, alpha, device):
    from page_rank_gb300 import native
    L = native.lib()
    n = A.shape[0]
    ip, ix, dv = _csr_dev(A, device)
    W = -(-n // 64)
    inv = torch.empty((W, 64, 64), dtype=torch.float32, device=device)
    st = torch.cuda.current_stream(device).cuda_stream
    native.check(L.gl_window_blocks(ip.data_ptr(), ix.data_ptr(), dv.data_ptr(), n, alpha, inv.data_ptr(), st))
    status = torch.zeros(1, dtype=torch.int32, device=device)
    native.check(L.gl_window_invert(inv.data_ptr(), n, status.data_ptr(), st))
    return inv, int(status.item())


def _graph(log2n, seed=3):
    from page_rank_gb300 import synth
    return synth.cluster_zipf_graph(log2n=log2n, mean_degree=20.0, seed=seed)


@pytest.mark.parametrize("n", [64, 1000, 4096])
@pytest.mark.parametrize("alpha", [0.5, 0.85, 0.99])
def test_window_inverses_match_numpy(n, alpha, device):
    from page_rank_gb300 import synth
    A = synth.cluster_zipf_graph(log2n=12, mean_degree=20.0, seed=5).A[:n, :n]
    A = sp.csr_matrix(A / np.maximum(np.asarray(A.sum(axis=0)).ravel(), 1.0)[None, :])   # columns sum <= 1
    inv, status = _inverses(A, alpha, device)
    assert status == 0
    ref = np.linalg.inv(ows.window_blocks(A, alpha))
    got = inv.cpu().numpy().astype(np.float64).transpose(0, 2, 1)     # stored transposed
    assert np.abs(got - ref).max() <= 1e-5 * max(1.0, np.abs(ref).max())


def test_window_invert_reports_a_bad_pivot(device):
    A = sp.identity(200, format="csr", dtype=np.float32) * 2.0     # column sums 2: 1 - 0.9 * 2 < 0
    _, status = _inverses(A, 0.9, device)
    assert status == 1


@pytest.mark.parametrize("K", [1, 3, 8, 16, 40, 64, 100, 128, 130, 200, 256])
@pytest.mark.parametrize("n", [130, 4096])
def test_window_apply_matches_oracle(K, n, device):
    from page_rank_gb300 import native
    A = _graph(12).A[:n, :n]
    inv, _ = _inverses(A, 0.85, device)
    inv_np = inv.cpu().numpy().astype(np.float64).transpose(0, 2, 1)
    rng = np.random.default_rng(K + n)
    T = rng.random((n, K)).astype(np.float32)
    N0 = rng.random((n, K)).astype(np.float32)
    Td = torch.from_numpy(T).to(device)
    Y = torch.full((n, K), float("nan"), device=device)
    nf = torch.from_numpy(N0).to(device)
    W = -(-n // 64)
    part = torch.from_numpy(rng.random((W, K)).astype(np.float32)).to(device)
    part0 = part.cpu().numpy().astype(np.float64)
    st = torch.cuda.current_stream(device).cuda_stream
    L = native.lib()
    # accumulate mode
    native.check(L.gl_window_apply(inv.data_ptr(), n, K, Td.data_ptr(), 0.7, Y.data_ptr(), nf.data_ptr(), 0.15, 0,
                                   part.data_ptr(), st))
    y_ref = 0.7 * ows.apply_inverse(inv_np, T.astype(np.float64))
    assert np.abs(Y.cpu().numpy() - y_ref).max() <= 1e-5 * max(1.0, np.abs(y_ref).max())
    assert np.abs(nf.cpu().numpy() - (N0 + 0.15 * y_ref)).max() <= 1e-5 * max(1.0, np.abs(y_ref).max())
    pad = np.zeros((W * 64, K))
    pad[:n] = 0.15 * y_ref
    p_ref = part0 + pad.reshape(W, 64, K).sum(axis=1)
    assert np.abs(part.cpu().numpy() - p_ref).max() <= 1e-4 * max(1.0, np.abs(p_ref).max())
    # init mode without Y
    native.check(L.gl_window_apply(inv.data_ptr(), n, K, Td.data_ptr(), 1.0, None, nf.data_ptr(), 0.5, 1,
                                   part.data_ptr(), st))
    ref = 0.5 * ows.apply_inverse(inv_np, T.astype(np.float64))
    assert np.abs(nf.cpu().numpy() - ref).max() <= 1e-5 * max(1.0, np.abs(ref).max())
    pad[:n] = ref
    assert np.abs(part.cpu().numpy() - pad.reshape(W, 64, K).sum(axis=1)).max() <= 1e-4 * max(1.0, np.abs(ref).max())


@pytest.mark.parametrize("leaves", [0, 1, 3])
@pytest.mark.parametrize("shape", ["expected", "pagerank"])
def test_start_vectors_match_oracle(leaves, shape, device):
    from page_rank_gb300.engine import PPREngine
    from page_rank_gb300.window_start import WindowStart
    from page_rank_gb300 import synth
    g = _graph(12)
    eng = PPREngine(g.A, block_size=4, device=device)
    ws = WindowStart(eng, leaves=leaves, shape=shape)
    sets = synth.seed_sets(g.n, 37, 1, 32, seed=2)
    x0 = ws.start(sets, 0.85).cpu().numpy().astype(np.float64)
    far = ws._prepare(0.85)["shape"].cpu().numpy().astype(np.float64)
    V = oppr.teleport_matrix(g.n, sets)
    ref = ows.window_start(g.A, V, 0.85, leaves, far)
    assert np.abs(x0 - ref).sum(axis=0).max() <= 1e-5
    assert np.allclose(x0.sum(axis=0), 1.0, atol=1e-5)


def test_cold_residuals_are_exact(device):
    from page_rank_gb300.engine import PPREngine
    from page_rank_gb300.window_start import WindowStart
    from page_rank_gb300 import synth
    g = synth.cluster_zipf_graph(log2n=11, mean_degree=8.0, seed=7)
    A = g.A.tolil()
    A[:, 11] = 0                                 # a dangling seed
    A = sp.csr_matrix(A, dtype=np.float32)
    A.eliminate_zeros()
    dangling = np.asarray(A.sum(axis=0)).ravel() == 0
    eng = PPREngine(A, block_size=4, device=device, dangling=dangling)
    ws = WindowStart(eng, leaves=1)
    # small sets look each seed up in the seed rows; the all-nodes set walks
    # the rows and looks their columns up in the seed list
    sets = [np.array([11]), np.array([11, 12, 13]), np.array([64, 65, 66, 67, 64]), np.arange(0, 2048, 61),
            np.arange(2048)]
    r = ws.cold_residuals(sets, 0.85)
    V = oppr.teleport_matrix(g.n, [np.unique(s) for s in sets])
    ref = ows.cold_residual(A, V, 0.85, dangling)
    assert np.allclose(r, ref, rtol=1e-6, atol=1e-9)


def test_warm_solve_same_fixed_point_fewer_iterations(device):
    from page_rank_gb300.engine import PPREngine
    from page_rank_gb300.window_start import WindowStart
    from page_rank_gb300 import synth
    g = _graph(14)
    eng = PPREngine(g.A, block_size=4, device=device)
    sets = synth.seed_sets(g.n, 24, 1, 32, seed=9)
    cold = eng.solve(sets, alpha=0.85, tol=1e-6)
    ws = WindowStart(eng, leaves=3)
    warm = ws.solve(sets, alpha=0.85, tol=1e-6)
    assert cold.converged.all() and warm.converged.all()
    assert warm.warm_columns.all()
    assert cold.iterations.mean() / warm.iterations.mean() >= 1.5, (cold.iterations.mean(),
                                                                    warm.iterations.mean())
    # both within the certified 1e-6 of the exact fixed point
    V = oppr.teleport_matrix(g.n, sets)
    exact, cert, _ = oppr.refine_fp64(g.A, cold.X.cpu().numpy().astype(np.float64), V, 0.85, g.dangling, 1e-10)
    assert cert.max() < 1e-10
    for res in (cold, warm):
        err = np.abs(res.X.cpu().numpy().astype(np.float64) - exact).sum(axis=0).max()
        assert err <= 1e-6, err


def test_fallback_to_cold_start(device, monkeypatch):
    from page_rank_gb300.engine import PPREngine
    from page_rank_gb300.window_start import WindowStart
    from page_rank_gb300 import synth
    g = _graph(12)
    eng = PPREngine(g.A, block_size=4, device=device)
    ws = WindowStart(eng, leaves=1)
    sets = synth.seed_sets(g.n, 6, 1, 8, seed=4)

    def far_away(V, st, tp):                  # all mass on one node far from every seed
        X = torch.zeros_like(V)
        X[g.n - 1] = 1.0
        return X
    monkeypatch.setattr(ws, "_start_from", far_away)
    warm = ws.solve(sets, alpha=0.85, tol=1e-6)
    cold = eng.solve(sets, alpha=0.85, tol=1e-6)
    assert not warm.warm_columns.any()
    assert np.array_equal(warm.iterations, cold.iterations)
    assert torch.equal(warm.X, cold.X)


def test_learned_far_field_gains_over_pagerank_far_field(device):
    """What the trained network gains: the window start whose far field the
    network predicts against the same start with the global PageRank
    vector as far field (the method without the network)."""
    from page_rank_gb300.engine import PPREngine
    from page_rank_gb300.warmstart import FarFieldModel
    from page_rank_gb300.window_start import WindowStart
    from page_rank_gb300 import synth
    g = _graph(15)
    eng = PPREngine(g.A, block_size=4, device=device)
    ws = WindowStart(eng, leaves=3, shape="pagerank")
    held = synth.seed_sets(g.n, 64, 1, 32, seed=21)
    base = ws.solve(held, alpha=0.85, tol=1e-6)
    model = FarFieldModel(device, seed=0)
    stats = model.fit(ws, 0.85, synth.seed_sets(g.n, 512, 1, 32, seed=22), epochs=20)
    # the network predicts the log-ratio to the expected far field, which for
    # uniformly drawn seed sets is already the target: the loss starts near
    # zero and must stay there
    assert np.isfinite(stats.losses).all() and stats.losses[-1] <= max(10 * stats.losses[0], 1e-3)
    ws.set_shape("learned", model)
    learned = ws.solve(held, alpha=0.85, tol=1e-6)
    ws.set_shape("expected")
    expected = ws.solve(held, alpha=0.85, tol=1e-6)
    assert base.converged.all() and learned.converged.all()
    assert learned.iterations.mean() < base.iterations.mean(), (learned.iterations.mean(), base.iterations.mean(),
                                                               expected.iterations.mean())
    assert (learned.X.double() - base.X.double()).abs().sum(dim=0).max().item() < 2e-6


def test_run_personalized_pagerank_warm_start_argument(device):
    """graph_link.run_personalized_pagerank(..., warm_start=X0): the same
    fixed point from a given start, fewer iterations from a good one."""
    from page_rank_gb300 import graph_link as gl
    from page_rank_gb300.engine import PPREngine
    from page_rank_gb300.window_start import WindowStart
    g = _graph(12)
    pbr = gl.csr_to_pbr(g.A, block_rows=4, block_cols=4, min_nnz_per_block=4).to(device)
    src = torch.tensor([3, 700, 4000], dtype=torch.int32, device=device)
    Xc, it_c, conv_c = gl.run_personalized_pagerank(pbr, src, tolerance=1e-7, max_iterations=500)
    eng = PPREngine(g.A, block_size=4, device=device)
    x0 = WindowStart(eng, leaves=4).start([[3], [700], [4000]], 0.85)
    Xw, it_w, conv_w = gl.run_personalized_pagerank(pbr, src, tolerance=1e-7, max_iterations=500, warm_start=x0)
    assert conv_c and conv_w and it_w < it_c
    assert (Xc.double() - Xw.double()).abs().sum(dim=0).max().item() < 2e-6
    with pytest.raises(ValueError):
        gl.run_personalized_pagerank(pbr, src, warm_start=x0[:, :2])


def test_ragged_graph_with_dangling_nodes(device):
    """n not a multiple of the window (a short last window), dangling nodes
    (their mass returns through each query's teleport vector in the solve;
    the start ignores it), a seed set inside the short window: start vectors
    against the oracle, the warm solve against the FP64 fixed point."""
    from page_rank_gb300.engine import PPREngine
    from page_rank_gb300.window_start import WindowStart
    n = 1000
    rng = np.random.default_rng(12)
    rows, cols = [], []
    for j in range(n):
        if j % 17 == 0:
            continue                                   # dangling
        deg = int(rng.integers(1, 9))
        loc = (j // 64) * 64 + rng.integers(0, 64, deg)        # mostly inside the window
        far = rng.integers(0, n, 2)
        for i in np.concatenate([loc, far]):
            if i < n:
                rows.append(i)
                cols.append(j)
    A = sp.csr_matrix((np.ones(len(rows)), (rows, cols)), shape=(n, n))
    A.sum_duplicates()
    colsum = np.asarray(A.sum(axis=0)).ravel()
    A = sp.csr_matrix(A @ sp.diags(np.where(colsum > 0, 1.0 / np.maximum(colsum, 1), 0.0)), dtype=np.float32)
    dangling = colsum == 0
    eng = PPREngine(A, block_size=4, device=device, dangling=dangling)
    ws = WindowStart(eng, leaves=3)
    sets = [np.array([990, 999]), np.array([5]), np.arange(0, 1000, 97)]
    x0 = ws.start(sets, 0.85).cpu().numpy().astype(np.float64)
    far = ws._prepare(0.85)["shape"].cpu().numpy().astype(np.float64)
    V = oppr.teleport_matrix(n, sets)
    ref = ows.window_start(A, V, 0.85, 3, far)
    assert np.abs(x0 - ref).sum(axis=0).max() <= 1e-5
    warm = ws.solve(sets, alpha=0.85, tol=1e-6)
    exact = oppr.direct_solve_fp64(A, V, 0.85, dangling)
    assert warm.converged.all()
    assert np.abs(warm.X.cpu().numpy().astype(np.float64) - exact).sum(axis=0).max() <= 1e-6
