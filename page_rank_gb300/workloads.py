"""Measured workloads beyond the SpMM headline (used by ``bench.py --workload``).

* ``ppr_small``   — n = 4096 SBM, one seed set of 5 nodes, alpha 0.85,
  100 iterations / tol 1e-8, dangling mass to the personalization vector,
  PBR 4x4 min 4 (plain PPR).
* ``ppr_batched`` — n = 2**22 cluster / Zipf(2.1) graph, mean degree 20,
  256 seed sets of 1-32 seeds, alpha 0.85, per-column L1 1e-6 (certified:
  the stop threshold bounds the distance to the exact fixed point), converged
  columns retired, CUDA-graph chunks, layout chosen by the autotuner;
  compared with the plain one-query-at-a-time GPU path.
"""
from __future__ import annotations

import time

import numpy as np
import torch

from . import synth
from .autotune import autotune
from .engine import PPREngine


def ppr_small(device) -> dict:
    g = synth.sbm_graph(64, 64, 0.1, 0.0005, seed=1)
    seeds = np.sort(np.random.default_rng(5).choice(g.n, 5, replace=False))
    eng = PPREngine(g.A, block_size=4, min_nnz_per_block=4, device=device, dangling=g.dangling)
    eng.solve([seeds], alpha=0.85, tol=1e-8, max_iterations=100, certified=False, retire=False)  # warm
    t0 = time.perf_counter()
    reps = 20
    for _ in range(reps):
        r = eng.solve([seeds], alpha=0.85, tol=1e-8, max_iterations=100, certified=False, retire=False,
                      use_graphs=False)
    dt = (time.perf_counter() - t0) / reps
    return {"workload": "ppr_small: " + g.description + ", 5 seeds, alpha .85, 100 it / tol 1e-8, PBR 4x4 min 4",
            "n": g.n, "nnz": int(g.A.nnz), "iterations": int(r.launched_iterations),
            "converged": bool(r.converged[0]), "ms_per_query": round(dt * 1e3, 3),
            "final_update_l1": r.history[-1] if r.history else None}


def ppr_batched(device, log2n: int = 22, K: int = 256, plain_sample: int = 16, tune: bool = True) -> dict:
    t0 = time.perf_counter()
    g = synth.cluster_zipf_graph(log2n=log2n, mean_degree=20.0, seed=3, device=device)
    gen_s = time.perf_counter() - t0
    sets = synth.seed_sets(g.n, K, 1, 32, seed=11)
    tuned = None
    if tune:
        tuned = autotune(g.A, K, device=device)
        bs, mn, tile = tuned.block_size, tuned.min_nnz, tuned.column_tile
    else:
        bs, mn, tile = 8, 8, 0
    eng = PPREngine(g.A, block_size=bs, min_nnz_per_block=mn, device=device, dangling=g.dangling,
                    column_tile=tile)
    # batched: all K seed sets as columns, retirement + CUDA graphs
    eng.solve(sets[:8], alpha=0.85, tol=1e-6)                       # warm-up (captures, caches)
    torch.cuda.synchronize(device)
    rb = eng.solve(sets, alpha=0.85, tol=1e-6, retire=True, use_graphs=True)
    batched_qps = K / rb.seconds
    # plain: one query at a time on the same engine
    rp = eng.solve_plain(sets[:plain_sample], alpha=0.85, tol=1e-6)
    plain_qps = plain_sample / rp.seconds
    # same answers (both certified to 1e-6 of the fixed point)
    diff = (rb.X[:, :plain_sample].double() - rp.X.double()).abs().sum(dim=0).max().item()
    step_bytes = eng.iteration_bytes(K)
    return {
        "workload": f"ppr_batched: {g.description}, K={K} seed sets of 1-32, alpha .85, L1 1e-6 certified",
        "n": g.n, "nnz": int(g.A.nnz), "graph_gen_s": round(gen_s, 2),
        "layout": {"block": bs, "min_nnz": mn, "column_tile": tile,
                   "autotune": tuned.table if tuned else None},
        "batched": {"queries_per_s": round(batched_qps, 2), "seconds": round(rb.seconds, 4),
                    "launched_iterations": rb.launched_iterations, "column_steps": rb.column_steps,
                    "max_iterations_per_column": int(rb.iterations.max()),
                    "all_converged": bool(rb.converged.all())},
        "plain": {"queries_per_s": round(plain_qps, 2), "sample": plain_sample,
                  "seconds": round(rp.seconds, 4), "iterations_total": rp.launched_iterations},
        "speedup_batched_vs_plain": round(batched_qps / plain_qps, 2),
        "max_l1_batched_vs_plain": diff,
        "iteration_bytes_full_width": step_bytes,
    }
