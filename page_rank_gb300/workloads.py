"""Measured workloads beyond the SpMM headline (used by ``bench.py --workload``).

* ``ppr_small``   — n = 4096 SBM, one seed set of 5 nodes, alpha 0.85,
  100 iterations / tol 1e-8, dangling mass to the personalization vector,
  PBR 4x4 min 4 (plain PPR).
* ``ppr_batched`` — n = 2**22 cluster / Zipf(2.1) graph, mean degree 20,
  256 seed sets of 1-32 seeds, alpha 0.85, per-column L1 1e-6 (certified:
  the stop threshold bounds the distance to the exact fixed point), converged
  columns retired, CUDA-graph chunks, layout chosen by the autotuner;
  compared with the plain one-query-at-a-time GPU path.
* ``edges``       — the HTTP request path's edge list -> transition matrix
  step on the device against the host (scipy) path, and a request served
  twice (the second reuses the resident graph).
"""
from __future__ import annotations

import time

import numpy as np
import torch

from . import native, synth
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
    eng.solve(sets, alpha=0.85, tol=1e-6)      # warm-up: every launch shape and workspace once
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


def ppr_step(device, log2n: int = 22, K: int = 256, block: int = 4, min_nnz: int = 4, tile: int = 0,
             steps: int = 16) -> dict:
    """Fused power-iteration steps alone (``gl_ppr_step``, STOP_ALL, dense
    start columns) on the batched configuration's graph class with K
    columns: the kernel behind the batched queries/s, timed with CUDA events
    over ``steps`` steps after four warm-up steps."""
    from .graph_link.pbr_registry import get_pbr_gpu_meta
    from .pbr import pbr_from_device_csr
    from .ppr import PprRun, dangling_bitmap, teleport_from_seed_sets
    g = synth.cluster_zipf_graph(log2n=log2n, mean_degree=20.0, seed=3, device=device)
    A = g.A
    n = A.shape[0]
    indptr = torch.from_numpy(A.indptr.astype(np.int32)).to(device)
    indices = torch.from_numpy(A.indices.astype(np.int32)).to(device)
    data = torch.from_numpy(A.data.astype(np.float32)).to(device)
    dbits = dangling_bitmap(indices, n)
    pbr = pbr_from_device_csr(indptr, indices, data, n, n, block, block, min_nnz).to(device)
    meta = get_pbr_gpu_meta(pbr)
    meta["column_tile"] = tile
    rng = np.random.default_rng(0)
    seeds = torch.from_numpy(rng.integers(0, n, K).astype(np.int32)).to(device)
    sptr = torch.arange(K + 1, dtype=torch.int32, device=device)
    x = torch.rand((n, K), generator=torch.Generator(device=device).manual_seed(0), device=device)
    x /= x.sum(dim=0, keepdim=True)
    tp = teleport_from_seed_sets(sptr, seeds, n, block)
    run = PprRun(meta, n, n, block, block, tp, 0.85, steps + 4, 0.0, native.GL_PPR_STOP_ALL, dbits)
    run.init(x)
    run.launch_chunk(4)
    torch.cuda.synchronize(device)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    run.launch_chunk(steps)
    e1.record()
    torch.cuda.synchronize(device)
    ms = e0.elapsed_time(e1) / steps
    nb, packed, rem = meta["codes"].numel(), meta["data"].numel(), meta["rem_col_ind"].numel()
    B = 20 * nb + 4 * packed + 4 * (n + 1) + 8 * rem + 8 * n * K
    return {"workload": f"ppr_step: {g.description}, K={K} dense columns, PBR {block}x{block} min {min_nnz}, "
                        f"column tile {tile or 'automatic'}",
            "n": n, "nnz": int(A.nnz), "ms_per_step": round(ms, 4), "alg_bytes_per_step": B,
            "alg_GBs": round(B / ms / 1e6, 1)}


def warmstart(device, log2n: int = 21, train_vectors: int = 20000, K: int = 256, leaves=(2, 4, 6, 8, 10),
              layout=(4, 4, 0), mlp_start: bool = True, keep_x: bool = False) -> dict:
    """Warm starts on the cluster / Zipf graph class at n = 2**log2n, K held-out
    seed sets of 1-32 seeds, alpha 0.85, certified L1 1e-6, each solved cold
    and from every start (wall time includes computing the start):

    * the window-solve start with the global PageRank vector as far field,
      with the far field learned by ``FarFieldModel`` (trained on
      ``train_vectors`` plain-method vectors), and with the expected far
      field, for each number of window exits in ``leaves``;
    * with ``mlp_start``, the per-(node, query) network start
      (``WarmStart``, trained on the same number of vectors).

    The window start's per-graph setup (inverses, PageRank, far field) and the
    networks' training run before the timed solves and are reported."""
    from .warmstart import FarFieldModel, WarmStart
    from .window_start import WindowStart
    alpha, tol = 0.85, 1e-6
    g = synth.cluster_zipf_graph(log2n=log2n, mean_degree=20.0, seed=3, device=device)
    bs, mn, ct = layout
    eng = PPREngine(g.A, block_size=bs, min_nnz_per_block=mn, device=device, dangling=g.dangling, column_tile=ct)
    sets = synth.seed_sets(g.n, K, 1, 32, seed=424242)

    def timed(fn):
        # one untimed run first (allocations at this width, launch shapes),
        # then the timed one: every variant is measured the same way
        fn()
        torch.cuda.synchronize(device)
        t0 = time.perf_counter()
        r = fn()
        torch.cuda.synchronize(device)
        return r, time.perf_counter() - t0

    cold, t_cold = timed(lambda: eng.solve(sets, alpha=alpha, tol=tol))

    def record(res, secs):
        return {"iterations_sum": int(res.iterations.sum()), "iterations_mean": round(float(res.iterations.mean()), 2),
                "iterations_max": int(res.iterations.max()), "seconds": round(secs, 4),
                "queries_per_s": round(K / secs, 1), "column_steps": res.column_steps,
                "columns_using_start": float(np.mean(getattr(res, "warm_columns", np.zeros(1)))),
                "all_converged": bool(res.converged.all()),
                "iterations_cold_over_this": round(float(cold.iterations.sum()) / max(1, int(res.iterations.sum())), 3),
                "wall_cold_over_this": round(t_cold / secs, 3),
                "max_l1_vs_cold": float((res.X.double() - cold.X.double()).abs().sum(dim=0).max().item())}

    out = {"workload": f"warm starts: {g.description}; {K} held-out seed sets of 1-32 uniform seeds, alpha {alpha}, "
                       f"certified L1 {tol:g}, PBR {bs}x{bs} min {mn}",
           "n": g.n, "nnz": int(g.A.nnz), "cold": record(cold, t_cold), "starts": {}}
    ws = WindowStart(eng, leaves=max(leaves), shape="pagerank")
    torch.cuda.synchronize(device)
    t0 = time.perf_counter()
    ws.inverses(alpha)                          # inverses, PageRank, far field: once per graph and alpha
    torch.cuda.synchronize(device)
    setup = time.perf_counter() - t0
    out["window_setup_s"] = round(setup, 3)
    out["window_setup_phases"] = ws.setup_phases.get(round(float(alpha), 12))
    out["off_window_nnz"] = ws.off.nnz
    best = None
    for L in leaves:
        ws.leaves = L
        ws.set_shape("expected")
        res, t = timed(lambda: ws.solve(sets, alpha=alpha, tol=tol))
        _, t_start = timed(lambda: ws.start(sets, alpha))
        rec = record(res, t)
        rec["start_seconds"] = round(t_start, 4)
        out["starts"][f"window_expected_L{L}"] = rec
        if best is None or t < best[1]:
            best = (f"window_expected_L{L}", t, res, L)
    L = best[3]
    ws.leaves = L
    ws.set_shape("pagerank")
    res, t = timed(lambda: ws.solve(sets, alpha=alpha, tol=tol))
    out["starts"][f"window_pagerank_L{L}"] = record(res, t)
    model = FarFieldModel(device, seed=0)
    train_sets = synth.seed_sets(g.n, train_vectors, 1, 32, seed=7)
    t0 = time.perf_counter()
    stats = model.fit(ws, alpha, train_sets, tol=tol)
    train_s = time.perf_counter() - t0
    ws.set_shape("learned", model)
    res, t = timed(lambda: ws.solve(sets, alpha=alpha, tol=tol))
    rec = record(res, t)
    rec["train"] = {"vectors": stats.vectors, "examples": stats.examples, "seconds": round(train_s, 2),
                    "loss_first": round(stats.losses[0], 4), "loss_last": round(stats.losses[-1], 4)}
    pr = out["starts"][f"window_pagerank_L{L}"]["iterations_sum"]
    rec["iterations_pagerank_far_field_over_this"] = round(pr / max(1, int(res.iterations.sum())), 3)
    out["starts"][f"window_learned_L{L}"] = rec
    ws.set_shape("expected")
    if mlp_start:
        mw = WarmStart(eng, seed=0)
        t0 = time.perf_counter()
        ms = mw.train(num_vectors=train_vectors, batch=256, nodes_per_vector=512, epochs=3)
        mt = time.perf_counter() - t0
        res, t = timed(lambda: mw.solve(sets, alpha=alpha, tol=tol))
        rec = record(res, t)
        rec["train"] = {"vectors": ms.vectors, "examples": ms.examples, "seconds": round(mt, 2)}
        out["starts"]["mlp_node_query"] = rec
    out["start_kernels"] = window_start_kernels(ws, K)
    out["best"] = best[0]
    out["best_iterations_cold_over_warm"] = out["starts"][best[0]]["iterations_cold_over_this"]
    out["best_wall_cold_over_warm"] = out["starts"][best[0]]["wall_cold_over_this"]
    if keep_x:
        out["_X_best"] = best[2].X
        out["_sets"] = sets
        out["_graph"] = g
    return out


def window_start_kernels(ws, K: int, reps: int = 5) -> dict:
    """CUDA-event times of the window start's two kernels over K columns, as
    one window exit runs them: the off-window SpMM (``gl_pbr_spmm`` over M)
    and ``gl_window_apply`` (y = alpha B^-1 T written, added into the near
    field, per-window column sums updated).  Algorithmic bytes: the SpMM
    reads M (8 bytes per entry as CSR) and X and writes Y; the apply reads
    the inverses (16 KB per window) and T, writes y, reads and writes the
    near field and the column sums.  FLOPs of the apply: 2 * 64 per output."""
    eng = ws.eng
    dev = ws.dev
    n = eng.n
    L = native.lib()
    st = torch.cuda.current_stream(dev).cuda_stream
    inv = ws.inverses(0.85)
    gen = torch.Generator(device=dev).manual_seed(0)
    T = torch.rand((n, K), generator=gen, device=dev)
    Y = torch.empty_like(T)
    nf = torch.zeros_like(T)
    part = torch.zeros((ws.windows, K), device=dev)

    def apply():
        native.check(L.gl_window_apply(inv.data_ptr(), n, K, T.data_ptr(), 0.85, Y.data_ptr(), nf.data_ptr(),
                                       0.15, 0, part.data_ptr(), st))

    def spmm():
        ws.off.spmm(T, Y)

    out = {}
    for name, fn in (("window_apply", apply), ("off_window_spmm", spmm)):
        fn()
        torch.cuda.synchronize(dev)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(reps):
            fn()
        e1.record()
        torch.cuda.synchronize(dev)
        out[name] = {"ms": round(e0.elapsed_time(e1) / reps, 4)}
    W = ws.windows
    apply_bytes = W * 64 * 64 * 4 + 4 * n * K * 4 + 2 * W * K * 4
    ms = out["window_apply"]["ms"]
    out["window_apply"].update({"alg_bytes": apply_bytes, "alg_GBs": round(apply_bytes / ms / 1e6, 1),
                                "gflop": round(2 * 64 * n * K / 1e9, 2),
                                "tflops": round(2 * 64 * n * K / ms / 1e9, 2)})
    nnz = ws.off.nnz
    sp_bytes = 8 * nnz + 4 * (n + 1) + 8 * n * K
    out["off_window_spmm"].update({"nnz": nnz, "alg_bytes": sp_bytes,
                                   "alg_GBs": round(sp_bytes / out["off_window_spmm"]["ms"] / 1e6, 1)})
    out["columns"] = K
    return out


def window_kernels(device, log2n: int = 21, K: int = 256) -> dict:
    """The window start's two kernels alone (``window_start_kernels``) on the
    warm-start configuration's graph class at n = 2**log2n, K columns."""
    from .window_start import WindowStart
    g = synth.cluster_zipf_graph(log2n=log2n, mean_degree=20.0, seed=3, device=device)
    eng = PPREngine(g.A, block_size=4, min_nnz_per_block=4, device=device, dangling=g.dangling)
    ws = WindowStart(eng)
    ws.inverses(0.85)
    return {"workload": f"window start kernels: {g.description}, K={K}", "n": g.n, "nnz": int(g.A.nnz),
            **window_start_kernels(ws, K)}


def serving(device, rates=(200.0, 800.0, 3200.0), requests_per_rate: int = 400, graphs: int = 8,
            seed: int = 5) -> dict:
    """The serving configuration with the warm start on (as the
    configuration asks) and, for comparison, off."""
    on = serving_pass(device, rates, requests_per_rate, graphs, True, seed)
    off = serving_pass(device, rates, requests_per_rate, graphs, False, seed)
    return {"workload": on["workload"].replace(", warm start on", ""), "resident_bytes": on["resident_bytes"],
            "warm_start_on": {"start": on.get("warm_start"), "setup_s": on.get("warm_setup_s"),
                              "rates": on["rates"], "admission_waits": on["admission_waits"],
                              "gates": on.get("warm_gates")},
            "warm_start_off": {"rates": off["rates"], "admission_waits": off["admission_waits"]}}


def serving_pass(device, rates=(200.0, 800.0, 3200.0), requests_per_rate: int = 400, graphs: int = 8,
                 warm: bool = True, seed: int = 5) -> dict:
    """8 resident cluster / Zipf graphs with n log-uniform in 2**16 .. 2**22,
    Poisson arrivals at each rate, 1-64 seeds per request, alpha in
    {0.8, 0.85, 0.9}, certified L1 1e-6; p50 / p99 latency and queries/s."""
    from .serving import PPRServer, latency_summary
    from .warmstart import WarmStartGate
    from .window_start import WindowStart
    rng = np.random.default_rng(seed)
    sizes = np.sort(np.round(rng.uniform(16, 22, graphs)).astype(int))
    srv = PPRServer(device=device, chunk=8)
    descr = []
    setup_s = 0.0
    for i, lg in enumerate(sizes):
        g = synth.cluster_zipf_graph(log2n=int(lg), mean_degree=20.0, seed=200 + i, device=device)
        eng = srv.add_graph(f"g{i}", g.A, dangling=g.dangling, block_size=8, min_nnz=4)
        if warm:
            # window-solve start per graph; its gate keeps it only while the
            # iterations it saves outweigh its cost.  The per-alpha window
            # inverses and far-field shapes are built here, before the clock.
            t0 = time.perf_counter()
            w = WindowStart(eng, gate=WarmStartGate())
            for a in (0.8, 0.85, 0.9):
                w.inverses(a)
            setup_s += time.perf_counter() - t0
            srv.warm[f"g{i}"] = w
        descr.append(int(g.n))
    # warm up every graph once
    for i in range(graphs):
        srv.submit(f"g{i}", [0, 1])
    srv.run_until_idle()
    out = {"workload": f"serving: {graphs} cluster/Zipf graphs, n = {descr}, Poisson arrivals, 1-64 seeds, "
                       f"alpha in {{.8,.85,.9}}, certified L1 1e-6, warm start {'on' if warm else 'off'}",
           "resident_bytes": srv.resident_bytes(), "rates": []}
    if warm:
        out["warm_start"] = "window-solve start (8 window exits, expected far field), per-graph gate"
        out["warm_setup_s"] = round(setup_s, 2)
    srv.start()
    try:
        for lam in rates:
            srv.completed.clear()
            reqs = []
            t0 = time.perf_counter()
            for _ in range(requests_per_rate):
                i = int(rng.integers(0, graphs))
                n = descr[i]
                seeds = rng.choice(n, size=int(rng.integers(1, 65)), replace=False)
                reqs.append(srv.submit(f"g{i}", seeds, alpha=float(rng.choice([0.8, 0.85, 0.9])), tol=1e-6))
                time.sleep(float(rng.exponential(1.0 / lam)))
            for r in reqs:
                r.done.wait(600)
            wall = time.perf_counter() - t0
            s = latency_summary(reqs)
            s.update({"offered_qps": lam, "achieved_qps": round(len(reqs) / wall, 1),
                      "converged": int(sum(r.converged for r in reqs)),
                      "mean_iterations": round(float(np.mean([r.iterations for r in reqs])), 1)})
            out["rates"].append(s)
    finally:
        srv.stop()
    out["admission_waits"] = srv.admission_waits
    if warm:
        out["warm_gates"] = {name: w.gate.summary() for name, w in srv.warm.items() if w.gate is not None}
    return out


def kernels(device, log2n: int = 20, K: int = 64, examples: int = 1 << 20) -> dict:
    """The other kernel families on the SpMM configuration's graph, timed
    with CUDA events: a device build (8x8, min 8), eight fused PPR steps over
    K dense columns, and one forward / backward / Adam round of the
    warm-start network on ``examples`` rows, and the top 100 nodes of each of
    the K columns (``gl_topk_columns``, six passes over the columns)."""
    from .graph_link.pbr_registry import get_pbr_gpu_meta
    from .pbr import build_pbr_device, pbr_from_device_csr
    from .ppr import PprRun, teleport_from_seed_sets
    from .warmstart import F_IN, MLP

    g = synth.cluster_rmat_graph(log2n=log2n, cluster=64, mean_degree=16, p_intra=0.7, seed=2, device=device)
    A = g.A
    n = A.shape[0]
    ip = torch.from_numpy(A.indptr.astype(np.int32)).to(device)
    ix = torch.from_numpy(A.indices.astype(np.int32)).to(device)
    dv = torch.from_numpy(A.data.astype(np.float32)).to(device)

    def timed(fn, reps=3):
        fn()
        torch.cuda.synchronize(device)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(reps):
            fn()
        e1.record()
        torch.cuda.synchronize(device)
        return e0.elapsed_time(e1) / reps

    build_ms = timed(lambda: build_pbr_device(ip, ix, dv, n, n, 8, 8, 8))
    pd = pbr_from_device_csr(ip, ix, dv, n, n, 8, 8, 8).to(device)
    meta = get_pbr_gpu_meta(pd)
    rng = np.random.default_rng(0)
    seeds = torch.from_numpy(rng.integers(0, n, K).astype(np.int32)).to(device)
    tp = teleport_from_seed_sets(torch.arange(K + 1, dtype=torch.int32, device=device), seeds, n, 8)
    x0 = torch.rand((n, K), device=device)
    x0 /= x0.sum(dim=0, keepdim=True)
    run = PprRun(meta, n, n, 8, 8, tp, 0.85, 10_000, 0.0, native.GL_PPR_STOP_PER_COLUMN, None)
    run.init(x0)
    step_ms = timed(lambda: run.launch_chunk(8)) / 8
    from .topk import topk_columns
    topk_ms = timed(lambda: topk_columns(x0, 100))
    mlp = MLP(device, 0)
    Xf = torch.rand((examples, F_IN), device=device)
    T = torch.rand(examples, device=device)
    fwd_ms = timed(lambda: mlp.forward(Xf))
    bwd_ms = timed(lambda: mlp.gradient(Xf, T))
    return {"workload": f"kernels: n=2^{log2n} clustered R-MAT ({int(A.nnz)} nonzeros), PBR 8x8 min 8; "
                        f"PPR steps over {K} dense columns; MLP on {examples} rows",
            "build_ms": round(build_ms, 3), "ppr_step_ms": round(step_ms, 4),
            "ppr_step_bytes": int(pd.accounted_blocks() * 20 + pd.compressed_nnz() * 4 + 4 * (n + 1)
                                  + 8 * pd.remainder_nnz() + 8 * n * K),
            "topk100_ms": round(topk_ms, 4), "topk_bytes_per_pass": int(4 * n * K),
            "mlp_forward_ms": round(fwd_ms, 4), "mlp_backward_ms": round(bwd_ms, 4)}


def edges(device, log2n: int = 20, reps: int = 5, request_nodes: int = 20000) -> dict:
    """The HTTP request path's matrix step: edge list -> column-normalized
    transition matrix, on the 2^log2n clustered R-MAT edge list (16 edges per
    node in generation order, duplicates included, unit weights).

    * ``device_ms``: ``gl_edges_to_transition`` with the edges already in
      device memory (CUDA events, mean of ``reps``);
    * ``call_ms``: the Python call from host arrays (upload, workspace, the
      count read back), wall clock;
    * ``host_ms``: the same step on the host the way the reference does it
      (scipy COO -> CSR, then the normalize arithmetic), wall clock, once;
    * ``identical``: device and host results equal bit for bit;
    * ``request_first_ms`` / ``request_again_ms``: ``POST /api/ppr``'s body
      on a ``request_nodes``-node graph of the same class, first call (edge
      list -> PBR on the device) and a repeat (resident graph reused)."""
    from .transition import (clear_resident_graphs, device_transition, edge_list_csr, normalize_columns,
                             solve_edge_list_request)

    src, dst = synth.cluster_rmat_edges(log2n)
    n, m = 1 << log2n, int(src.size)
    w = np.ones(m)
    s_d = torch.from_numpy(src.astype(np.int32)).to(device)
    t_d = torch.from_numpy(dst.astype(np.int32)).to(device)
    w_d = torch.from_numpy(w).to(device)
    L = native.lib()
    ws_bytes = int(L.gl_edges_workspace_bytes(n, m))
    ws = torch.empty(ws_bytes, dtype=torch.uint8, device=device)
    indptr = torch.empty(n + 1, dtype=torch.int32, device=device)
    indices = torch.empty(m, dtype=torch.int32, device=device)
    data = torch.empty(m, dtype=torch.float32, device=device)
    dang = torch.empty(n, dtype=torch.uint8, device=device)
    nnz = torch.empty(1, dtype=torch.int64, device=device)
    st = torch.cuda.current_stream(device).cuda_stream

    def launch():
        native.check(L.gl_edges_to_transition(n, m, s_d.data_ptr(), t_d.data_ptr(), w_d.data_ptr(), 1,
                                              indptr.data_ptr(), indices.data_ptr(), data.data_ptr(),
                                              dang.data_ptr(), nnz.data_ptr(), ws.data_ptr(), ws_bytes, st))

    for _ in range(2):
        launch()
    torch.cuda.synchronize(device)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(reps):
        launch()
    e1.record()
    torch.cuda.synchronize(device)
    device_ms = e0.elapsed_time(e1) / reps

    device_transition(n, src, dst, w, device)
    torch.cuda.synchronize(device)
    t0 = time.perf_counter()
    ip, ix, dv, dg = device_transition(n, src, dst, w, device)
    call_ms = (time.perf_counter() - t0) * 1e3

    t0 = time.perf_counter()
    A_norm, dangling = normalize_columns(edge_list_csr(n, src, dst, w))
    host_ms = (time.perf_counter() - t0) * 1e3
    identical = (np.array_equal(ip.cpu().numpy(), A_norm.indptr) and np.array_equal(ix.cpu().numpy(), A_norm.indices)
                 and np.array_equal(dv.cpu().numpy().view(np.uint32), A_norm.data.view(np.uint32))
                 and np.array_equal(dg.cpu().numpy(), dangling))

    # request path: a small graph of the same class, twice
    rs, rd = synth.cluster_rmat_edges(int(np.ceil(np.log2(request_nodes))))
    keep = (rs < request_nodes) & (rd < request_nodes)
    rs, rd = rs[keep][: 8 * request_nodes], rd[keep][: 8 * request_nodes]
    ids = [str(i) for i in range(request_nodes)]
    index_of = {x: i for i, x in enumerate(ids)}
    src_ids, dst_ids = [ids[i] for i in rs], [ids[i] for i in rd]
    ones = [1.0] * len(src_ids)
    clear_resident_graphs()
    t0 = time.perf_counter()
    first = solve_edge_list_request(ids, index_of, src_ids, dst_ids, ones, [0, 1, 2], 0.85, 100, 1e-6)
    first_ms = (time.perf_counter() - t0) * 1e3
    t0 = time.perf_counter()
    again = solve_edge_list_request(ids, index_of, src_ids, dst_ids, ones, [0, 1, 2], 0.85, 100, 1e-6)
    again_ms = (time.perf_counter() - t0) * 1e3
    clear_resident_graphs()
    same_ranks = bool(np.array_equal(first["ranks"], again["ranks"]))
    return {"workload_detail": f"edge list of the n=2^{log2n} clustered R-MAT graph: {m} edges, unit weights; "
                               f"request graph {request_nodes} nodes / {len(src_ids)} edges",
            "edges": m, "nnz": int(ix.numel()), "device_ms": round(device_ms, 3),
            "device_edges_per_s": round(m / device_ms * 1e3, 1), "call_ms": round(call_ms, 2),
            "host_ms": round(host_ms, 1), "identical": bool(identical),
            "request_first_ms": round(first_ms, 2), "request_again_ms": round(again_ms, 2),
            "request_same_ranks": same_ranks}
