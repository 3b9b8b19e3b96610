"""Learned warm start: the device MLP kernels against the FP64 oracle
(forward, gradients, Adam / BF16 rounding), and what the trained network
gains over the cold start with identical converged results."""
import numpy as np
import pytest
import torch

from oracle import mlp as omlp
from oracle import ppr as oppr

pytestmark = pytest.mark.gpu


def _params(seed=0):
    from page_rank_gb300 import warmstart as ws
    rng = np.random.default_rng(seed)
    W1 = rng.normal(0, 0.4, (ws.HIDDEN, ws.F_IN)).astype(np.float32)
    b1 = rng.normal(0, 0.1, ws.HIDDEN).astype(np.float32)
    w2 = rng.normal(0, 0.2, ws.HIDDEN).astype(np.float32)
    b2 = np.float32(0.3)
    return W1, b1, w2, b2


def _load(mlp, W1, b1, w2, b2):
    from page_rank_gb300 import warmstart as ws
    p = np.concatenate([W1.ravel(), b1, w2, [b2]]).astype(np.float32)
    mlp.params.copy_(torch.from_numpy(p))
    mlp._refresh_bf16()


def test_mlp_forward_matches_oracle(device):
    from page_rank_gb300 import warmstart as ws
    W1, b1, w2, b2 = _params()
    m = ws.MLP(device)
    _load(m, W1, b1, w2, b2)
    X = np.random.default_rng(1).normal(0, 1, (3000, ws.F_IN)).astype(np.float32)
    y = m.forward(torch.from_numpy(X).to(device)).cpu().numpy()
    ref, _ = omlp.forward(X, omlp.bf16_round(W1), b1, omlp.bf16_round(w2), b2)
    assert np.abs(y - ref).max() <= 1e-4 * max(1.0, np.abs(ref).max())
    # the device BF16 copies are the oracle's rounding
    assert np.array_equal(m.W1.cpu().numpy().view(np.uint16), omlp.bf16_bits(W1).ravel())


def test_mlp_gradient_matches_oracle(device):
    from page_rank_gb300 import warmstart as ws
    W1, b1, w2, b2 = _params(2)
    m = ws.MLP(device)
    _load(m, W1, b1, w2, b2)
    rng = np.random.default_rng(3)
    X = rng.normal(0, 1, (5000, ws.F_IN)).astype(np.float32)
    t = rng.normal(0, 1, 5000).astype(np.float32)
    g, loss = m.gradient(torch.from_numpy(X).to(device), torch.from_numpy(t).to(device))
    gref, lref = omlp.backward(X, t, omlp.bf16_round(W1), b1, omlp.bf16_round(w2), b2)
    g = g.cpu().numpy().astype(np.float64)
    assert abs(loss - lref) <= 1e-4 * abs(lref)
    assert np.abs(g - gref).max() <= 2e-4 * np.abs(gref).max()


def test_adam_step_moves_toward_lower_loss(device):
    from page_rank_gb300 import warmstart as ws
    m = ws.MLP(device, seed=5)
    rng = np.random.default_rng(4)
    X = torch.from_numpy(rng.normal(0, 1, (4096, ws.F_IN)).astype(np.float32)).to(device)
    t = torch.from_numpy(rng.normal(-5, 1, 4096).astype(np.float32)).to(device)
    losses = []
    for _ in range(60):
        _, loss = m.gradient(X, t)
        m.adam_step(4096, lr=5e-3)
        losses.append(loss)
    assert losses[-1] < 0.5 * losses[0]
    p = m.params.cpu().numpy()
    assert np.array_equal(m.W1.cpu().numpy().view(np.uint16),
                          omlp.bf16_bits(p[: ws.HIDDEN * ws.F_IN]))


def test_trained_warm_start_gains_iterations(device):
    """Train on plain-method PPR vectors of a small cluster / Zipf graph, then
    solve held-out seed sets from the predicted start: fewer iterations than
    the cold start, and the same converged vectors (certified 1e-6)."""
    from page_rank_gb300 import synth
    from page_rank_gb300.engine import PPREngine
    from page_rank_gb300.warmstart import WarmStart
    g = synth.cluster_zipf_graph(log2n=13, mean_degree=12.0, seed=7)
    eng = PPREngine(g.A, block_size=8, min_nnz_per_block=4, device=device, dangling=g.dangling)
    ws = WarmStart(eng, seed=0)
    stats = ws.train(num_vectors=2048, batch=256, nodes_per_vector=512, epochs=6)
    assert stats.losses[-1] < stats.losses[0]
    sets = synth.seed_sets(g.n, 64, 1, 32, seed=999)
    cold = eng.solve(sets, tol=1e-6)
    warm = ws.solve(sets, tol=1e-6)
    assert cold.converged.all() and warm.converged.all()
    assert warm.iterations.sum() < cold.iterations.sum()
    # FP64 fixed point by power iteration to 1e-14 (a sparse LU of this hub graph fills in)
    X64, _, ok, _ = oppr.power_iteration_fp64(g.A, oppr.teleport_matrix(g.n, sets), 0.85, 5000, 1e-14, g.dangling)
    assert ok
    for res in (cold, warm):
        l1 = np.abs(res.X.cpu().numpy().astype(np.float64) - X64).sum(axis=0)
        assert l1.max() <= 1e-6
    print(f"warm start: iterations cold {cold.iterations.sum()} warm {warm.iterations.sum()} "
          f"({cold.iterations.sum() / warm.iterations.sum():.2f}x), warm columns {warm.warm_columns.mean():.2f}")
