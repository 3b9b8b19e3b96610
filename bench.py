"""Benchmark: fused PBR + CSR-remainder SpMM on the 2**20-node clustered R-MAT graph.

Workload (one "step" = one SpMM of the whole matrix with one dense block):
  n = 2**20 nodes in 16384 clusters of 64, mean out-degree 16, 70% of edges
  to a uniform in-cluster target, 30% R-MAT (0.57, 0.19, 0.19, 0.05),
  values 1/out-degree (FP32); X ~ U[0,1) with 64 FP32 columns; PBR 8x8 blocks
  with min_nnz_per_block = 8 plus the CSR remainder.  Seeded synthetic data
  (no dataset is part of the reference).

Metric: algorithmic HBM bytes of one SpMM / time, in GB/s:
  B = 20 * blocks + 4 * packed + 4 * (n + 1) + 8 * remainder + 4 * n * F (X)
      + 4 * n * F (Y)
(code 8 + coords 8 + offset 4 per block; value 4 per packed entry; remainder
indptr 4 per row, column 4 + value 4 per entry; X read once, Y written once).

The same line carries ``parity`` (the device build of the timed matrix
against the CPU restatement of the reference builder, and the timed Y against
the FP64 product) and ``ppr``: the second half of the metric, queries/s of
batched, one-query-at-a-time and warm-started PPR on the 2**22-node
cluster / Zipf graph (256 seed sets of 1-32 seeds, L1 1e-6), their FP64
distance on sampled columns, and an FP64 CPU PPR baseline on all host cores.

Usage:
  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
Under torchrun (N > 1) every rank runs an independent replica on its own GPU
(the path has no exchange step); rank 0 prints the JSON line.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "SpMM HBM GB/s (frac of peak)"
UNIT = "GB/s"
def workload_name(log2n: int = 20) -> str:
    return (f"spmm: n=2^{log2n} clustered R-MAT ({(1 << log2n) // 64} clusters of 64, out-degree 16, 70% intra, "
            "30% R-MAT .57/.19/.19/.05), X 64 FP32 columns, PBR 8x8 min_nnz 8 + CSR remainder")
FALLBACK_HBM_GBS = 6800.0


# ---------------------------------------------------------------------------
def alg_bytes(nb: int, packed: int, rem: int, n: int, F: int, elem: int = 4) -> int:
    return 20 * nb + elem * packed + 4 * (n + 1) + (4 + elem) * rem + 2 * elem * n * F


def measured_peak():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.is_file():
        try:
            d = json.loads(p.read_text())
            return float(d["hbm_gbs"]), "measured"
        except Exception:
            pass
    return FALLBACK_HBM_GBS, "fallback"


def profile_traffic(log2n: int, features: int, kernel: str):
    """DRAM bytes per launch of this workload's kernel from the committed
    one-pass ncu capture (profiles/dram_traffic.json; None when that size /
    kernel was not captured)."""
    p = ROOT / "profiles" / "dram_traffic.json"
    if not p.is_file():
        return None
    try:
        entries = json.loads(p.read_text())["captures"]
    except (ValueError, KeyError):
        return None
    for e in entries:
        if e.get("log2n") == log2n and e.get("features") == features and e.get("kernel") == kernel:
            return int(e["dram_bytes_per_launch"])
    return None


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled while the timed region runs."""

    FIELDS = ("timestamp,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int, period_ms: int = 20):
        self.gpu_index = gpu_index
        self.period_ms = period_ms
        self.proc = None
        self.lines: list[tuple[float, str]] = []
        self._t = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu_index), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", str(self.period_ms)],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (FileNotFoundError, OSError):
            self.proc = None
            return
        self._t = threading.Thread(target=self._read, daemon=True)
        self._t.start()
        t0 = time.time()
        while not self.lines and time.time() - t0 < 5.0:
            time.sleep(0.01)

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append((time.time(), line.strip()))

    def stop(self):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self, t0: float, t1: float):
        rows = [l for (t, l) in self.lines if t0 <= t <= t1 + 0.05]
        if not rows:
            rows = [l for (_, l) in self.lines[-3:]]
        mhz, max_mhz, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            parts = [x.strip() for x in r.split(",")]
            if len(parts) < 9:
                continue
            try:
                mhz.append(float(parts[1]))
                max_mhz = float(parts[2])
            except ValueError:
                continue
            for name, val in zip(names, parts[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(name)
        if not mhz:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"], "samples": 0}
        return {"sm_mhz": statistics.median(mhz), "sm_max_mhz": max_mhz, "reasons": sorted(reasons),
                "samples": len(mhz)}


def replica_time(ms_local: float, world: int, device=None) -> float:
    """Slowest replica's time (ms): the whole job finishes when the last rank
    does.  Ranks are independent replicas (no data exchange); this max is the
    only collective."""
    if world <= 1:
        return ms_local
    import torch
    import torch.distributed as dist
    t = torch.tensor([ms_local], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_throughput(units_per_rank: float, world: int, ms_max: float) -> float:
    """Whole-job throughput: every rank processed units_per_rank in ms_max."""
    return world * units_per_rank / (ms_max / 1e3)


# ---------------------------------------------------------------------------
def build_workload(device, log2n: int = 20):
    from page_rank_gb300 import synth

    g = synth.cluster_rmat_graph(log2n=log2n, cluster=64, mean_degree=16, p_intra=0.7, seed=2, device=device)
    return g


def cpu_spmm_rate(A, X, total_bytes: int, budget_s: float = 10.0, max_reps: int = 50):
    """Single-core FP32 scipy CSR SpMM (the reference's CPU check,
    Tests/test_spmm.py:46), repeated on the full matrix for ~budget_s."""
    from oracle.spmm import spmm_csr_fp32

    spmm_csr_fp32(A, X)  # warm
    reps, t0 = 0, time.perf_counter()
    while reps < max_reps:
        spmm_csr_fp32(A, X)
        reps += 1
        if time.perf_counter() - t0 >= budget_s:
            break
    dt = (time.perf_counter() - t0) / reps
    return total_bytes / dt / 1e9, reps, dt


def run_ours(args, rank, world, local_rank):
    import torch
    import torch.distributed as dist

    from page_rank_gb300 import graph_link as gl
    from page_rank_gb300 import native
    from page_rank_gb300.pbr import matrix_desc, spmm_workspace

    dev = torch.device("cuda", local_rank)
    torch.cuda.set_device(dev)
    native.lib()
    g = build_workload(dev, args.log2n)
    A = g.A
    n, F = A.shape[0], 64
    t_b0 = time.perf_counter()
    pbr = gl.csr_to_pbr(A, block_rows=8, block_cols=8, min_nnz_per_block=8)
    torch.cuda.synchronize()
    build_s = time.perf_counter() - t_b0
    pd = pbr.to(dev)
    meta = gl.get_pbr_gpu_meta(pd)
    nb, packed, rem = pd.accounted_blocks(), pd.compressed_nnz(), pd.remainder_nnz()
    B = alg_bytes(nb, packed, rem, n, F)
    gen = torch.Generator(device=dev)
    gen.manual_seed(1234 + rank)
    X = torch.rand((n, F), generator=gen, device=dev, dtype=torch.float32)
    Y = torch.empty((n, F), device=dev, dtype=torch.float32)
    # the kernel choice rides in the matrix's metadata, so the end-to-end
    # arm (which builds its own descriptor) runs the same kernel
    meta["kernel"] = {"auto": 0, "stripe": 1, "window": 2}[args.kernel]
    desc = matrix_desc(meta, n, n, 8, 8)
    L = native.lib()
    stream = torch.cuda.current_stream(dev)
    sh = stream.cuda_stream
    ws = spmm_workspace(meta, desc, 1, F, dev)
    ws_ptr, ws_bytes = (ws.data_ptr(), ws.numel()) if ws is not None else (None, 0)
    del g
    torch.cuda.empty_cache()

    def step():
        native.check(L.gl_pbr_spmm(desc, X.data_ptr(), Y.data_ptr(), 1, F, ws_ptr, ws_bytes, sh))

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()

    sampler = ClockSampler(local_rank)
    sampler.start()
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    t0 = time.time()
    ev0.record(stream)
    for _ in range(args.steps):
        step()
    ev1.record(stream)
    torch.cuda.synchronize()
    t1 = time.time()
    if world > 1:
        dist.barrier()
    sampler.stop()
    ms = ev0.elapsed_time(ev1)
    ms_max = replica_time(ms, world, dev)
    ms_per_step = ms_max / args.steps
    value = replica_throughput(B * args.steps, world, ms_max) / 1e9
    kernel_gbs = B / (ms / args.steps / 1e3) / 1e9

    # ---- end to end through the public API with host buffers ---------------
    # page_rank_gb300.streaming.spmm_host_batches: pinned host X in, host Y
    # out, copies of neighbouring batches overlapped with the SpMM
    from page_rank_gb300.hostmem import bind_to_device_cpus, restore_cpus
    from page_rank_gb300.streaming import spmm_host_batches
    # pinned buffers are placed by first touch: allocate and fill them from
    # the CPUs next to the GPU
    placement = bind_to_device_cpus(dev)
    nb_e2e = 4
    xs = [torch.empty((n, F), dtype=torch.float32, pin_memory=True) for _ in range(nb_e2e)]
    ys = [torch.empty((n, F), dtype=torch.float32, pin_memory=True) for _ in range(nb_e2e)]
    xh = X.cpu()
    for x in xs:
        x.copy_(xh)
    spmm_host_batches(pd, xs[:2], ys[:2])                 # warm (streams, workspace)
    torch.cuda.synchronize()
    # one call streams all e2e steps (the 4 host buffer pairs in turn), so
    # the copy pipeline fills once rather than once per 4 batches
    steps_e2e = max(nb_e2e, args.e2e_steps)
    xs_all = [xs[i % nb_e2e] for i in range(steps_e2e)]
    ys_all = [ys[i % nb_e2e] for i in range(steps_e2e)]
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    spmm_host_batches(pd, xs_all, ys_all)
    e1.record(stream)
    torch.cuda.synchronize()
    restore_cpus(placement)                                # the CPU legs use every host core again
    e2e_ms = replica_time(e0.elapsed_time(e1) / steps_e2e, world, dev)
    e2e_value = replica_throughput(B, world, e2e_ms) / 1e9
    x_host, y_host = xs[0], ys[0]
    # every e2e batch carried X, so each host result must equal the device Y
    # of the timed loop bit for bit (the kernel is deterministic)
    y_dev = Y.cpu()
    e2e_exact = all(torch.equal(y, y_dev) for y in ys)
    ys = xs = xs_all = ys_all = None
    clocks = sampler.summary(t0, t1)

    out = None
    if rank == 0:
        peak, peak_kind = measured_peak()
        traffic = profile_traffic(args.log2n, F, "window_kernel" if args.kernel == "window" else "stripe_kernel")
        out = {
            "metric": METRIC, "value": round(value, 1), "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms_per_step, 5),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded clustered R-MAT graph, X ~ U[0,1))",
            "config": {"workload": workload_name(args.log2n), "n": n, "features": F, "nnz": int(A.nnz),
                       "blocks": nb, "packed_nnz": packed, "remainder_nnz": rem,
                       "alg_bytes_per_step": B,
                       "l2": "inputs larger than L2: %.0f MB touched per step vs 129 MB L2" % (B / 1e6),
                       "parallelism": f"replicas x{world}", "gpu_build_s": round(build_s, 3)},
            "roofline": {"bound": "hbm", "achieved": round(kernel_gbs, 1), "peak": peak, "unit": "GB/s",
                         "frac": round(kernel_gbs / peak, 4), "peak_source": peak_kind,
                         "traffic": traffic,
                         "kernel": ("window_kernel<8> (gl_pbr_spmm kernel = 2: staged 64-row X windows)"
                                    if args.kernel == "window" else
                                    "stripe_kernel<float,8,8,V=4,C=16> (gl_pbr_spmm: half-warps with float4 "
                                    "lanes, stripes drawn 64-row window by window)"),
                         "heavy_pieces": int(desc.num_pieces), "heavy_stripes": int(desc.num_heavy)},
            "e2e": {"value": round(e2e_value, 1), "unit": UNIT, "ms_per_step": round(e2e_ms, 4),
                    "h2d_bytes_per_step": int(x_host.numel() * 4),
                    "d2h_bytes_per_step": int(y_host.numel() * 4),
                    "api": "page_rank_gb300.streaming.spmm_host_batches (pinned host X -> device SpMM -> "
                           "host Y, one call streaming all steps through 4 host buffer pairs, copies of "
                           "neighbouring batches overlapped)",
                    "host_result_equals_device_result": bool(e2e_exact), "host_placement": placement},
            "gpu_launches": args.steps,
            "clocks": clocks,
        }
        if world == 1 and not args.no_cpu_baseline:
            Xn = X.cpu().numpy()
            gbs, reps, dt = cpu_spmm_rate(A, Xn, B, budget_s=args.cpu_budget)
            out["cpu_baseline"] = {"value": round(gbs, 3), "unit": UNIT, "cores": 1, "kind": "port",
                                   "sample": f"full SpMM (scipy FP32 CSR @ X, the reference's CPU "
                                             f"check), {reps} reps, {dt * 1e3:.1f} ms each",
                                   "cpu": host_cpu()}
            out["parity"] = cpu_spmm_checks(A, pbr, Xn, y_dev.numpy())
    if rank == 0 and world == 1 and not args.no_ppr:
        del X, Y, ws, pd, pbr, A
        torch.cuda.empty_cache()
        out["ppr"] = run_ppr(dev, args)
    return out


def host_cpu() -> dict:
    """Host core count and CPU model (lscpu), reported beside CPU numbers."""
    model = None
    try:
        txt = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in txt.splitlines():
            if line.startswith("Model name:"):
                model = line.split(":", 1)[1].strip()
                break
    except (OSError, subprocess.SubprocessError):
        pass
    return {"nproc": os.cpu_count(), "model": model}


def cpu_spmm_checks(A, pbr, X: np.ndarray, Y: np.ndarray) -> dict:
    """CPU side of the SpMM line: the CPU restatement of the reference builder
    (pbr_matrix.cpp:340-477) timed on the same matrix and compared array by
    array with the device build that was timed, and the timed Y against the
    FP64 product (row-split over the host cores)."""
    import oracle
    from oracle.ppr import RowSplitMatrix

    n = A.shape[0]
    t0 = time.perf_counter()
    o = oracle.csr_to_pbr(A.indptr, A.indices, A.data, n, n, 8, 8, 8)
    build_s = time.perf_counter() - t0
    exact = True
    for k in ("block_codes", "block_coords", "block_offsets", "block_data",
              "remainder_indptr", "remainder_col_ind", "remainder_data"):
        a, b = np.asarray(getattr(pbr, k)), np.asarray(o[k])
        exact &= a.shape == b.shape and np.array_equal(a.view(np.uint8), b.view(np.uint8))
    M = RowSplitMatrix(A.astype(np.float64))
    try:
        Yref = M @ X.astype(np.float64)
    finally:
        M.close()
    rel = np.abs(Y.astype(np.float64) - Yref) / np.maximum(np.abs(Yref), 1e-30)
    return {"build_exact": bool(exact), "cpu_build_s": round(build_s, 2),
            "cpu_build": "single-threaded CPU restatement of the reference builder",
            "spmm_max_rel": float(rel.max()), "spmm_tol": 1e-5,
            "spmm_reference": "FP64 scipy CSR product of the same matrix and X"}


# ---------------------------------------------------------------------------
# PPR queries/s: the second half of the metric
PPR_ALPHA = 0.85
PPR_TOL = 1e-6


def run_ppr(dev, args) -> dict:
    """Batched vs one-query-at-a-time vs warm-started PPR on the 2**22-node
    cluster / Zipf graph (mean distinct out-degree 20, 80% of each node's
    edges inside its 64-node cluster), 256 seed sets of 1-32 uniform seeds,
    alpha 0.85, per-column certified L1 1e-6, converged columns retired,
    CUDA-graph chunks, layout from the autotuner.  Graph generation, the
    autotuner and the warm start's training run before the timed solves and
    are reported in seconds.  The CPU leg solves a sample of the same queries
    with the FP64 power iteration on all host cores; its vectors are the
    references the GPU columns are compared with."""
    import torch

    from page_rank_gb300 import synth, workloads
    from page_rank_gb300.autotune import autotune
    from page_rank_gb300.engine import PPREngine
    from page_rank_gb300.window_start import WindowStart

    K = 256
    t0 = time.perf_counter()
    g = synth.cluster_zipf_graph(log2n=args.ppr_log2n, mean_degree=20.0, seed=3, device=dev)
    gen_s = time.perf_counter() - t0
    sets = synth.seed_sets(g.n, K, 1, 32, seed=11)
    t0 = time.perf_counter()
    tuned = autotune(g.A, K, device=dev)
    tune_s = time.perf_counter() - t0
    eng = PPREngine(g.A, block_size=tuned.block_size, min_nnz_per_block=tuned.min_nnz, device=dev,
                    dangling=g.dangling, column_tile=tuned.column_tile)
    eng.solve(sets, alpha=PPR_ALPHA, tol=PPR_TOL)           # every launch shape and workspace once
    torch.cuda.synchronize(dev)
    sampler = ClockSampler(dev.index or 0)
    sampler.start()
    c0 = time.time()
    rb = eng.solve(sets, alpha=PPR_ALPHA, tol=PPR_TOL, retire=True, use_graphs=True)
    c1 = time.time()
    clocks = sampler.summary(c0, c1)
    plain_n = 16
    eng.solve_plain(sets[:2], alpha=PPR_ALPHA, tol=PPR_TOL)
    rp = eng.solve_plain(sets[:plain_n], alpha=PPR_ALPHA, tol=PPR_TOL)
    sampler.stop()
    # warm start: the window-solve start (8 window exits, expected far
    # field; its per-graph setup runs before the clock and is reported)
    wst = WindowStart(eng)
    t0 = time.perf_counter()
    wst.inverses(PPR_ALPHA)
    torch.cuda.synchronize(dev)
    warm_setup_s = time.perf_counter() - t0
    wst.solve(sets[:8], alpha=PPR_ALPHA, tol=PPR_TOL)        # launch shapes and workspaces once
    torch.cuda.synchronize(dev)
    rw = wst.solve(sets, alpha=PPR_ALPHA, tol=PPR_TOL, retire=True, use_graphs=True)
    warm_leaves = wst.leaves
    qps_b = K / rb.seconds
    qps_p = plain_n / rp.seconds
    qps_w = K / rw.seconds
    same = float((rb.X.double() - rw.X.double()).abs().sum(dim=0).max().item())
    # the warm-start configuration (2**21 nodes of the same class): cold and
    # every start on the same held-out seed sets
    layout = (tuned.block_size, tuned.min_nnz, tuned.column_tile)
    warm_setup_phases = wst.setup_phases.get(round(PPR_ALPHA, 12))
    del wst
    torch.cuda.empty_cache()
    wcfg = workloads.warmstart(dev, log2n=args.warm_log2n, train_vectors=args.ppr_train_vectors, K=K,
                               layout=layout, mlp_start=False, keep_x=not args.no_cpu_baseline)
    out = {
        "workload": f"batched PPR: {g.description}; {K} seed sets of 1-32 uniform seeds, alpha {PPR_ALPHA}, "
                    f"per-column L1 {PPR_TOL:g} to the fixed point (certified stop), retirement + CUDA graphs",
        "n": g.n, "nnz": int(g.A.nnz), "graph_gen_s": round(gen_s, 2), "autotune_s": round(tune_s, 2),
        "layout": {"block": tuned.block_size, "min_nnz": tuned.min_nnz, "column_tile": tuned.column_tile},
        "batched": {"queries_per_s": round(qps_b, 2), "seconds": round(rb.seconds, 4),
                    "iterations_sum": int(rb.iterations.sum()), "launched_steps": rb.launched_iterations,
                    "column_steps": rb.column_steps, "all_converged": bool(rb.converged.all())},
        "plain": {"queries_per_s": round(qps_p, 2), "sample": plain_n, "seconds": round(rp.seconds, 4),
                  "iterations_sum": int(rp.iterations.sum())},
        "batched_warm": {"queries_per_s": round(qps_w, 2), "seconds_including_start": round(rw.seconds, 4),
                         "start": f"window-solve start: {warm_leaves} window exits, expected far field, cold fallback",
                         "setup_s": round(warm_setup_s, 2), "setup_phases": warm_setup_phases,
                         "iterations_sum": int(rw.iterations.sum()), "column_steps": rw.column_steps,
                         "columns_using_start": float(np.mean(rw.warm_columns)),
                         "all_converged": bool(rw.converged.all())},
        "speedup_batched_vs_plain": round(qps_b / qps_p, 2),
        "speedup_batched_warm_vs_plain": round(qps_w / qps_p, 2),
        "iterations_cold_over_warm": round(float(rb.iterations.sum()) / max(1, int(rw.iterations.sum())), 3),
        "wall_cold_over_warm": round(rb.seconds / rw.seconds, 3),
        "max_l1_cold_vs_warm": same,
        "clocks": clocks,
        "warm_start_config": {k: v for k, v in wcfg.items() if not k.startswith("_")},
    }
    if not args.no_cpu_baseline:
        cores = os.cpu_count() or 1
        sample = list(range(min(cores, K)))
        cpu = cpu_ppr_leg(g, [sets[i] for i in sample], cores)
        Xg = rb.X[:, torch.tensor(sample, device=dev)].double().cpu().numpy()
        Xw = rw.X[:, torch.tensor(sample, device=dev)].double().cpu().numpy()
        d_b = np.abs(Xg - cpu["X"]).sum(axis=0) + cpu["bound"]
        d_w = np.abs(Xw - cpu["X"]).sum(axis=0) + cpu["bound"]
        out["parity"] = {"max_l1_vs_fp64": float(d_b.max()), "max_l1_warm_vs_fp64": float(d_w.max()),
                         "tol": PPR_TOL, "columns": len(sample),
                         "reference": "FP64 power iteration continued to a certified distance "
                                      f"< {cpu['bound'].max():.1e} of the exact fixed point"}
        out["cpu_baseline"] = {"value": round(cpu["qps"], 4), "unit": "queries/s", "cores": cpu["cores"],
                               "kind": "port", "cpu": host_cpu(),
                               "sample": f"{len(sample)} of the seed sets, one per process, FP64 scipy power "
                                         f"iteration (the reference update and stop rule, certified L1 "
                                         f"{PPR_TOL:g}), {cpu['seconds']:.1f} s wall"}
        out["speedup_batched_vs_cpu"] = round(qps_b / cpu["qps"], 1)
        out["warm_start_config"]["parity"] = warm_config_parity(wcfg, cores)
    return out


def warm_config_parity(wcfg: dict, cores: int, columns: int = 16) -> dict:
    """The best warm start's columns of the warm-start configuration against
    the FP64 fixed point: FP64 power iteration continued from them to a
    certified distance (the CPU leg's checker)."""
    from oracle.ppr import refine_fp64, teleport_matrix

    g = wcfg["_graph"]
    sets = wcfg["_sets"][:columns]
    X = wcfg["_X_best"][:, :columns].double().cpu().numpy()
    V = teleport_matrix(g.n, sets)
    ref, cert, its = refine_fp64(g.A, X, V, PPR_ALPHA, g.dangling, 1e-9, threads=cores)
    d = np.abs(X - ref).sum(axis=0) + cert
    return {"start": wcfg["best"], "columns": len(sets), "max_l1_vs_fp64": float(d.max()), "tol": PPR_TOL,
            "reference": f"FP64 power iteration from the GPU columns to a certified distance < {cert.max():.1e}"}


def _ppr_worker(args):
    """One query of the CPU PPR baseline (runs in a spawned process): FP64
    power iteration x <- alpha A x + (1 - alpha) v, timed to the certified
    stop, then continued (untimed) to a tight reference."""
    from multiprocessing import shared_memory

    import scipy.sparse as sp

    names, shapes, dtypes, n, seeds, alpha, thr, ref_bound, q = args
    shms = [shared_memory.SharedMemory(name=nm) for nm in names]
    try:
        indptr, indices, data, out = [np.ndarray(s, dtype=d, buffer=m.buf) for m, s, d in zip(shms, shapes, dtypes)]
        A = sp.csr_matrix((data, indices, indptr), shape=(n, n))
        v = np.zeros(n)
        v[np.asarray(seeds, dtype=np.int64)] = 1.0 / len(seeds)
        x = v.copy()
        t0 = time.perf_counter()
        dt = None
        cert = np.inf
        for _ in range(100000):
            xn = alpha * (A @ x) + (1.0 - alpha) * v
            upd = float(np.abs(xn - x).sum())
            x = xn
            if dt is None and upd < thr:
                dt = time.perf_counter() - t0
            cert = alpha / (1.0 - alpha) * upd
            if cert < ref_bound:
                break
        out[:, q] = x
        return dt, cert
    finally:
        for m in shms:
            m.close()


def cpu_ppr_leg(g, seed_sets, cores: int) -> dict:
    """FP64 power iteration for each seed set, one per spawned process (all
    host cores): queries/s to the certified L1 stop, and the FP64 vectors
    continued to a certified distance below 1e-10 of the fixed point."""
    import multiprocessing as mp
    from multiprocessing import shared_memory

    assert not np.any(g.dangling), "the CPU leg covers graphs without dangling nodes"
    n = g.n
    A = g.A
    arrays = [A.indptr.astype(np.int32), A.indices.astype(np.int32), A.data.astype(np.float64),
              np.zeros((n, len(seed_sets)), np.float64)]
    shms, names = [], []
    for a in arrays:
        m = shared_memory.SharedMemory(create=True, size=max(1, a.nbytes))
        np.ndarray(a.shape, dtype=a.dtype, buffer=m.buf)[...] = a
        shms.append(m)
        names.append(m.name)
    shapes = [a.shape for a in arrays]
    dtypes = [a.dtype for a in arrays]
    thr = PPR_TOL * (1.0 - PPR_ALPHA) / PPR_ALPHA
    jobs = [(names, shapes, dtypes, n, list(map(int, s)), PPR_ALPHA, thr, 1e-10, q)
            for q, s in enumerate(seed_sets)]
    try:
        with mp.get_context("spawn").Pool(min(cores, len(jobs))) as pool:
            t0 = time.perf_counter()
            res = pool.map(_ppr_worker, jobs)
            wall = time.perf_counter() - t0
        X = np.ndarray(shapes[3], dtype=dtypes[3], buffer=shms[3].buf).copy()
    finally:
        for m in shms:
            m.close()
            m.unlink()
    times = np.array([r[0] for r in res], dtype=np.float64)
    # all queries ran concurrently: the slowest one's time to its stop bounds
    # the batch's wall time
    span = float(times.max())
    return {"qps": len(seed_sets) / span, "seconds": span, "cores": min(cores, len(jobs)), "X": X,
            "bound": np.array([r[1] for r in res]), "total_wall_s": wall}


# ---------------------------------------------------------------------------
def _ref_worker(args):
    """One row range of the CPU SpMM (runs in a spawned process)."""
    from multiprocessing import shared_memory

    import scipy.sparse as sp

    names, shapes, dtypes, r0, r1, n, F, reps = args
    shms = [shared_memory.SharedMemory(name=nm) for nm in names]
    arrs = [np.ndarray(s, dtype=d, buffer=m.buf) for m, s, d in zip(shms, shapes, dtypes)]
    indptr, indices, data, X, Y = arrs
    lo, hi = int(indptr[r0]), int(indptr[r1])
    sub = sp.csr_matrix((data[lo:hi], indices[lo:hi], indptr[r0:r1 + 1] - lo), shape=(r1 - r0, n))
    for _ in range(reps):
        Y[r0:r1] = sub @ X
    for m in shms:
        m.close()
    return r1 - r0


def run_reference(args, rank, world):
    """CPU SpMM of the same workload on all host cores (the reference's CPU
    path: FP32 scipy CSR @ X, the check in Tests/test_spmm.py:46), row-split
    over a spawned process pool.  Each step is a bounded row sample so the
    whole run stays within a few minutes."""
    if rank != 0:
        return None
    import multiprocessing as mp
    from multiprocessing import shared_memory

    g = build_workload(None, args.log2n)
    A = g.A
    n, F = A.shape[0], 64
    X = np.random.default_rng(1234).random((n, F), dtype=np.float32)
    cores = os.cpu_count() or 1
    arrays = [A.indptr.astype(np.int64), A.indices, A.data, X, np.zeros((n, F), np.float32)]
    shms, names = [], []
    for a in arrays:
        m = shared_memory.SharedMemory(create=True, size=max(1, a.nbytes))
        np.ndarray(a.shape, dtype=a.dtype, buffer=m.buf)[...] = a
        shms.append(m)
        names.append(m.name)
    shapes = [a.shape for a in arrays]
    dtypes = [a.dtype for a in arrays]
    B_full = alg_bytes(0, 0, int(A.nnz), n, F)   # CSR only: indptr + col/val per nnz + X + Y
    ctx = mp.get_context("spawn")
    try:
        with ctx.Pool(cores) as pool:
            def run_rows(frac, reps):
                rows = max(cores, int(n * frac))
                bounds = np.linspace(0, rows, cores + 1).astype(int)
                jobs = [(names, shapes, dtypes, int(bounds[i]), int(bounds[i + 1]), n, F, reps)
                        for i in range(cores) if bounds[i + 1] > bounds[i]]
                t0 = time.perf_counter()
                pool.map(_ref_worker, jobs)
                return time.perf_counter() - t0, rows
            run_rows(0.05, 1)                           # warm the pool
            t_full, _ = run_rows(1.0, 1)                # calibrate one full SpMM
            budget = max(0.02, 150.0 / max(1, args.steps + args.warmup))
            frac = min(1.0, budget / max(t_full, 1e-6))
            for _ in range(args.warmup):
                run_rows(frac, 1)
            t0 = time.perf_counter()
            rows_done = 0
            for _ in range(args.steps):
                _, rows = run_rows(frac, 1)
                rows_done += rows
            dt = time.perf_counter() - t0
    finally:
        for m in shms:
            m.close()
            m.unlink()
    frac_eff = rows_done / (n * args.steps)
    value = B_full * frac_eff * args.steps / dt / 1e9
    ms = dt / args.steps * 1e3
    return {
        "metric": METRIC, "value": round(value, 3), "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(ms, 3), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded clustered R-MAT graph, X ~ U[0,1))",
        "config": {"workload": workload_name(args.log2n), "n": n, "features": F, "nnz": int(A.nnz),
                   "parallelism": f"{cores} host processes"},
        "impl": "reference",
        "cpu_baseline": {"value": round(value, 3), "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": f"rows [0, {int(n * frac_eff)}) of the matrix per step "
                                   f"({frac_eff:.3f} of the SpMM), FP32 scipy CSR @ X, "
                                   f"row-split over {cores} processes"},
        "e2e": {"value": round(value, 3), "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--e2e-steps", type=int, default=50)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-ppr", action="store_true", help="skip the PPR queries/s part of the line")
    ap.add_argument("--kernel", choices=["auto", "stripe", "window"], default="auto",
                    help="SpMM kernel (auto: the library's choice, the stripe kernel)")
    ap.add_argument("--ppr-log2n", type=int, default=22)
    ap.add_argument("--ppr-train-vectors", type=int, default=1024)
    ap.add_argument("--warm-log2n", type=int, default=21)
    ap.add_argument("--cpu-budget", type=float, default=10.0)
    ap.add_argument("--log2n", type=int, default=None,
                    help="graph size (2**log2n nodes); default: the workload's configuration size")
    ap.add_argument("--workload", choices=["spmm", "ppr_small", "ppr_batched", "ppr_step", "warmstart", "serving",
                                           "kernels", "edges", "window_kernels"],
                    default="spmm",
                    help="spmm (default, the headline line) or a secondary PPR workload")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3

    if args.workload == "spmm" and args.log2n is None:
        args.log2n = 20
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))

    if args.workload != "spmm":
        import torch
        from page_rank_gb300 import workloads
        dev = torch.device("cuda", local_rank)
        torch.cuda.set_device(dev)
        fn = getattr(workloads, args.workload)
        default_log2n = {"ppr_batched": 22, "ppr_step": 22, "warmstart": 21, "kernels": 20, "edges": 20,
                         "window_kernels": 21}
        out = fn(dev) if args.workload in ("ppr_small", "serving") else \
            fn(dev, log2n=args.log2n if args.log2n is not None else default_log2n[args.workload])
        out = {"workload": args.workload, **out}
    elif args.impl == "reference":
        out = run_reference(args, rank, world)
    else:
        if world > 1:
            import torch
            import torch.distributed as dist
            torch.cuda.set_device(local_rank)
            dist.init_process_group("nccl", device_id=torch.device("cuda", local_rank))
        out = run_ours(args, rank, world, local_rank)
        if world > 1:
            import torch.distributed as dist
            dist.destroy_process_group()
    if out is not None and rank == 0:
        print(json.dumps(out), flush=True)


if __name__ == "__main__":
    main()
