"""Continuous-batching server: every result is the same alone and in the
mix (within the stated tolerance), HBM-footprint admission, background loop."""
import time

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _graphs():
    from page_rank_gb300 import synth
    return {f"g{i}": synth.cluster_zipf_graph(log2n=lg, mean_degree=8.0, seed=20 + i)
            for i, lg in enumerate((10, 11, 12))}


def test_results_same_alone_and_in_the_mix(device):
    from page_rank_gb300.serving import PPRServer
    graphs = _graphs()
    srv = PPRServer(device=device, max_batch=16, chunk=4)
    for name, g in graphs.items():
        srv.add_graph(name, g.A, dangling=g.dangling, block_size=4)
    rng = np.random.default_rng(0)
    reqs = []
    for wave in range(5):                       # requests keep arriving while others run
        for _ in range(8):
            name = f"g{rng.integers(0, 3)}"
            n = graphs[name].n
            seeds = rng.choice(n, size=int(rng.integers(1, 65)), replace=False)
            alpha = float(rng.choice([0.8, 0.85, 0.9]))
            reqs.append(srv.submit(name, seeds, alpha=alpha, tol=1e-6))
        srv.step()
        srv.step()
    srv.run_until_idle()
    assert all(r.done.is_set() and r.converged for r in reqs)
    for r in reqs:
        alone = srv.engines[r.graph].solve([r.seeds], alpha=r.alpha, tol=1e-6)
        d = np.abs(alone.X[:, 0].double().cpu().numpy() - r.result.double().numpy()).sum()
        assert d <= 2e-6, (r.rid, d)        # both within 1e-6 of the fixed point


def test_admission_waits_for_memory(device):
    from page_rank_gb300.serving import PPRServer
    g = _graphs()["g2"]
    srv = PPRServer(device=device, max_batch=64, chunk=4, hbm_budget_bytes=1)
    srv.add_graph("g", g.A, dangling=g.dangling)
    srv.budget = srv.resident_bytes() + 2 * srv.column_bytes("g")     # two columns fit
    reqs = [srv.submit("g", [i, i + 1]) for i in range(6)]
    srv.step()
    live = sum(len(gr.reqs) + len(gr.joining) for gr in srv.groups.values())
    assert live <= 2 and srv.admission_waits > 0
    srv.run_until_idle()
    assert all(r.done.is_set() for r in reqs)


def test_background_loop_latency(device):
    from page_rank_gb300.serving import PPRServer, latency_summary
    graphs = _graphs()
    srv = PPRServer(device=device, chunk=8)
    for name, g in graphs.items():
        srv.add_graph(name, g.A, dangling=g.dangling)
    srv.start()
    try:
        rng = np.random.default_rng(1)
        reqs = []
        for _ in range(60):
            name = f"g{rng.integers(0, 3)}"
            reqs.append(srv.submit(name, rng.choice(graphs[name].n, 4, replace=False)))
            time.sleep(rng.exponential(0.001))
        for r in reqs:
            assert r.done.wait(60)
            assert r.error is None
    finally:
        srv.stop()
    s = latency_summary(reqs)
    assert s["completed"] == 60 and s["p99_ms"] >= s["p50_ms"] > 0


def test_top_k_requests(device):
    """Requests asking for their top nodes get exactly the k best entries of
    the vector they would have received in full (device selection), mixed
    in one batch with full-vector requests."""
    from oracle import topk as ot
    from page_rank_gb300.serving import PPRServer
    g = _graphs()["g2"]
    srv = PPRServer(device=device, max_batch=16, chunk=4)
    srv.add_graph("g", g.A, dangling=g.dangling, block_size=4)
    rng = np.random.default_rng(4)
    pairs = []
    for i in range(6):
        seeds = rng.choice(g.n, size=int(rng.integers(1, 9)), replace=False)
        pairs.append((srv.submit("g", seeds, tol=1e-6), srv.submit("g", seeds, tol=1e-6, top_k=[5, 40, 2048][i % 3])))
    srv.run_until_idle()
    for full, cut in pairs:
        assert full.done.is_set() and cut.done.is_set() and cut.result is None
        k = cut.top_k
        wv, wr = ot.topk_columns(full.result.numpy()[:, None], k)
        assert np.array_equal(cut.top_nodes, wr[0].astype(np.int64))
        assert np.array_equal(cut.top_values, wv[0])
    with pytest.raises(ValueError):
        srv.submit("g", [1], top_k=0)
