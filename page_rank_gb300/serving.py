"""Continuous-batching PPR serving on one GPU.

Graphs stay resident in HBM as PBR matrices (one :class:`PPREngine` each).
Requests (graph, seed set, alpha, tolerance) arrive at any time; the
scheduler keeps one *slot batch* per graph: the columns of one fused power
iteration, each column with its own alpha and certified threshold (one pass
over the matrix serves every request of the graph).  Between chunks of
iterations it

* retires columns whose update fell below their (certified) tolerance and
  hands their vectors to the waiting callers,
* admits queued requests into free slots — as long as the HBM footprint of
  all live columns plus the resident graphs stays within the budget —
  starting them from the teleport vector or from the learned warm start,
* and launches the next chunk of every active group on that group's own CUDA
  stream, so work of different graphs overlaps on the device.

A request's result does not depend on what it is batched with: each column
of the fused step is independent (per-column teleport, dangling mass and
residual), and a column runs until its own residual certifies the
tolerance.
"""
from __future__ import annotations

import collections
import itertools
import queue
import threading
import time
from dataclasses import dataclass, field

import numpy as np
import torch

from . import native
from .engine import PPREngine, certified_tolerance
from .ppr import PprRun, teleport_from_seed_sets
from .topk import topk_columns
from .trace import nvtx_range


@dataclass
class Request:
    graph: str
    seeds: np.ndarray
    alpha: float = 0.85
    tol: float = 1e-6
    max_iterations: int = 1000
    top_k: int | None = None       # set: only the k best nodes come back (top_values / top_nodes)
    rid: int = 0
    t_submit: float = 0.0
    t_admit: float = 0.0
    t_done: float = 0.0
    iterations: int = 0
    converged: bool = False
    result: torch.Tensor | None = None
    top_values: np.ndarray | None = None
    top_nodes: np.ndarray | None = None
    error: BaseException | None = None
    done: threading.Event = field(default_factory=threading.Event)

    @property
    def latency(self) -> float:
        return self.t_done - self.t_submit


class _Group:
    """The slot batch of one graph."""

    def __init__(self, server: "PPRServer", graph: str):
        self.server = server
        self.graph = graph
        self.eng: PPREngine = server.engines[graph]
        self.stream = torch.cuda.Stream(server.device)
        self.reqs: list[Request] = []          # live columns, in column order
        self.col_iters: list[int] = []         # iterations run per live column
        self.joining: list[Request] = []
        self.pre_pending = None                 # (first column, iterations already taken) of joiners
        self.run: PprRun | None = None
        self.x = None                          # current iterate [n, K]
        self.pending = False                   # a chunk is in flight on self.stream
        self.chunk_steps = 0

    def bytes_per_column(self) -> int:
        return self.server.column_bytes(self.graph)

    def rebuild(self, x_keep: torch.Tensor | None):
        """New run over the live + joining columns (at a chunk boundary)."""
        reqs = self.reqs + self.joining
        dev = self.server.device
        with torch.cuda.stream(self.stream):
            sets = [r.seeds for r in reqs]
            ptr, rows, w = self.eng.teleport(sets)
            tp = teleport_from_seed_sets(ptr, rows, self.eng.n, self.eng.block_size, w)
            alphas = np.array([r.alpha for r in reqs], dtype=np.float64)
            thr = np.array([certified_tolerance(r.tol, r.alpha) for r in reqs], dtype=np.float64)
            max_it = max(r.max_iterations for r in reqs)
            run = PprRun(self.eng.meta, self.eng.n, self.eng.n, self.eng.block_size, self.eng.block_size, tp,
                         alphas, max_it, thr, native.GL_PPR_STOP_PER_COLUMN, self.eng.dbits)
            if self.joining:
                x0 = torch.empty((self.eng.n, len(reqs)), dtype=torch.float32, device=dev)
                if x_keep is not None and self.reqs:
                    x0[:, : len(self.reqs)] = x_keep
                j0 = len(self.reqs)
                x_new, pre = self.server.start_vectors(self.graph, [r.seeds for r in self.joining],
                                                       np.array([r.alpha for r in self.joining]), self.stream)
                x0[:, j0:] = x_new
            else:
                x0 = x_keep
                pre = None
            run.init(x0, adopt=True)        # x0 was built here (or gathered from the last run)
        if pre is not None:
            # iterations the start already took, per joining column: a device
            # tensor, read at the next harvest (which waits for the stream)
            self.pre_pending = (len(self.col_iters), pre)
        self.col_iters = self.col_iters + [0] * len(self.joining)
        self.reqs = reqs
        self.joining = []
        self.run = run
        self.chunk_steps = 0

    def launch(self, chunk: int):
        with torch.cuda.stream(self.stream):
            self.run.launch_chunk(chunk)
        self.pending = True

    def harvest(self, chunk: int, now_fn) -> int:
        """After a chunk: retire converged columns; returns how many finished.
        Every device operation is ordered on this group's stream."""
        run = self.run
        t0 = self.chunk_steps
        n_valid = min(chunk, run.max_iterations - t0)
        with torch.cuda.stream(self.stream):
            res = run.res_hist[t0:t0 + n_valid].cpu().numpy() if n_valid > 0 else \
                np.zeros((0, len(self.reqs)))
            if self.pre_pending is not None:
                j0, pre = self.pre_pending
                pre = pre.cpu().numpy() if isinstance(pre, torch.Tensor) else np.asarray(pre)
                for i, p in enumerate(pre):
                    self.col_iters[j0 + i] += int(p)
                self.pre_pending = None
        self.chunk_steps += chunk
        self.pending = False
        finished = []
        for c, r in enumerate(self.reqs):
            thr_c = certified_tolerance(r.tol, r.alpha)
            col = res[:, c] if res.size else np.zeros(0)
            hit = np.nonzero(col < thr_c)[0]
            if hit.size:
                self.col_iters[c] += int(hit[0]) + 1
                r.converged = True
                finished.append(c)
            else:
                self.col_iters[c] += n_valid
                if self.col_iters[c] >= r.max_iterations:
                    finished.append(c)
        steps_written = min(self.chunk_steps, run.max_iterations)
        X = run.bufs[steps_written % 2]
        if not finished:
            self.x = X
            return 0
        fin = set(finished)
        keep = [c for c in range(len(self.reqs)) if c not in fin]
        full = [c for c in finished if self.reqs[c].top_k is None]
        cut = [c for c in finished if self.reqs[c].top_k is not None]
        with torch.cuda.stream(self.stream):
            out = X.index_select(1, torch.tensor(full, device=X.device)).cpu() if full else None
            tops = {}
            if cut:
                kmax = max(self.reqs[c].top_k for c in cut)
                tv, tr = topk_columns(X, kmax, cut)
                tv, tr = tv.cpu().numpy(), tr.cpu().numpy()
                tops = {c: (tv[i], tr[i]) for i, c in enumerate(cut)}
            x_keep = X.index_select(1, torch.tensor(keep, device=X.device)) if keep else None
        now = now_fn()
        col_of_full = {c: i for i, c in enumerate(full)}
        for c in finished:
            r = self.reqs[c]
            if c in col_of_full:
                r.result = out[:, col_of_full[c]]
            else:
                tv, tr = tops[c]
                r.top_values, r.top_nodes = tv[: r.top_k].copy(), tr[: r.top_k].astype(np.int64)
            r.iterations = self.col_iters[c]
            r.t_done = now
            r.done.set()
            self.server.completed.append(r)
        self.reqs = [self.reqs[c] for c in keep]
        self.col_iters = [self.col_iters[c] for c in keep]
        self.run = None
        self.x = x_keep
        return len(finished)


class PPRServer:
    """Resident graphs + continuous batching + HBM-footprint admission."""

    def __init__(self, device=None, hbm_budget_bytes: int | None = None, max_batch: int = 256, chunk: int = 8):
        dev = torch.device(device) if device is not None else torch.device("cuda")
        self.device = dev if dev.index is not None else torch.device("cuda", torch.cuda.current_device())
        self.engines: dict[str, PPREngine] = {}
        self.warm: dict[str, object] = {}
        self.max_batch = max_batch
        self.chunk = chunk
        if hbm_budget_bytes is None:
            free, _ = torch.cuda.mem_get_info(self.device)
            hbm_budget_bytes = int(free * 0.8)
        self.budget = int(hbm_budget_bytes)
        self.queue: "queue.Queue[Request]" = queue.Queue()
        self.waiting: collections.deque[Request] = collections.deque()
        self.groups: dict[tuple, _Group] = {}
        self._ids = itertools.count()
        self._stop = threading.Event()
        self._thread: threading.Thread | None = None
        self.t0 = time.perf_counter()
        self.completed: list[Request] = []
        self.admission_waits = 0

    # -- graphs -----------------------------------------------------------------
    def add_graph(self, name: str, A, dangling=None, block_size: int = 8, min_nnz: int | None = None,
                  warm_start=None):
        eng = PPREngine(A, block_size=block_size, min_nnz_per_block=min_nnz, device=self.device,
                        dangling=dangling)
        self.engines[name] = eng
        if warm_start is not None:
            self.warm[name] = warm_start
        return eng

    def resident_bytes(self) -> int:
        return sum(e.matrix_bytes() for e in self.engines.values())

    def column_bytes(self, graph: str) -> int:
        n = self.engines[graph].n
        return 2 * 4 * n + 2 * 8 * 1024        # two iterate columns + residual/dangling history rows

    def live_bytes(self) -> int:
        tot = 0
        for g in self.groups.values():
            tot += (len(g.reqs) + len(g.joining)) * self.column_bytes(g.graph)
        return tot

    def start_vectors(self, graph: str, seed_sets, alpha, stream):
        """(initial columns, iterations already taken per column) for newly
        admitted requests: the graph's warm start where it has one (with its
        cold-start fallback; requests are grouped by damping factor, which
        the start's precomputation depends on), else the teleport vectors."""
        eng = self.engines[graph]
        ws = self.warm.get(graph)
        k = len(seed_sets)
        with torch.cuda.stream(stream):
            if ws is None:
                return eng.teleport_columns(seed_sets), np.zeros(k, dtype=np.int64)
            alpha = np.broadcast_to(np.asarray(alpha, dtype=np.float64), (k,))
            X = torch.empty((eng.n, k), dtype=torch.float32, device=eng.device)
            pre = torch.zeros(k, dtype=torch.int64, device=eng.device)     # read at the next harvest
            for a in np.unique(alpha):
                sel = np.nonzero(alpha == a)[0]
                idx = torch.from_numpy(sel).pin_memory().to(eng.device, non_blocking=True)
                xs, used = ws.start_vectors([seed_sets[i] for i in sel], float(a))
                X[:, idx] = xs
                used = torch.as_tensor(used, device=eng.device)
                pre[idx] = used.to(torch.int64) * int(getattr(ws, "pre_steps", 0))
            return X, pre

    # -- requests -----------------------------------------------------------------
    def submit(self, graph: str, seeds, alpha: float = 0.85, tol: float = 1e-6,
               max_iterations: int = 1000, top_k: int | None = None) -> Request:
        """Queue a query; ``top_k`` returns only the k highest-ranked nodes
        (``Request.top_values`` / ``top_nodes``, selected on the device)
        instead of the full vector (``Request.result``)."""
        if graph not in self.engines:
            raise KeyError(f"unknown graph {graph!r}")
        seeds = np.asarray(seeds, dtype=np.int64)
        n = self.engines[graph].n
        if seeds.size == 0 or seeds.min() < 0 or seeds.max() >= n:
            raise ValueError("seeds must be a non-empty set of node ids of the graph")
        if top_k is not None and not 1 <= int(top_k) <= native.GL_TOPK_MAX:
            raise ValueError(f"top_k must be in [1, {native.GL_TOPK_MAX}]")
        r = Request(graph=graph, seeds=seeds, alpha=float(alpha), tol=float(tol), max_iterations=max_iterations,
                    top_k=None if top_k is None else int(top_k), rid=next(self._ids), t_submit=time.perf_counter())
        self.queue.put(r)
        return r

    def _admit(self):
        while True:
            try:
                self.waiting.append(self.queue.get_nowait())
            except queue.Empty:
                break
        budget_left = self.budget - self.resident_bytes() - self.live_bytes()
        still = collections.deque()
        while self.waiting:
            r = self.waiting.popleft()
            key = r.graph
            g = self.groups.get(key)
            live = (len(g.reqs) + len(g.joining)) if g else 0
            need = self.column_bytes(r.graph)
            if live >= self.max_batch or need > budget_left:
                still.append(r)
                self.admission_waits += 1
                continue
            if g is None:
                g = self.groups[key] = _Group(self, r.graph)
            g.joining.append(r)
            r.t_admit = time.perf_counter()
            budget_left -= need
        self.waiting = still

    def step(self) -> int:
        """One scheduling round; returns the number of requests finished."""
        with nvtx_range("serving.round"):
            return self._step()

    def _step(self) -> int:
        self._admit()
        active = []
        for g in self.groups.values():
            if g.joining or (g.reqs and g.run is None):
                g.rebuild(g.x if g.reqs else None)
            if g.reqs:
                g.launch(self.chunk)
                active.append(g)
        finished = 0
        for g in active:
            finished += g.harvest(self.chunk, time.perf_counter)
        for key in [k for k, g in self.groups.items() if not g.reqs and not g.joining]:
            del self.groups[key]
        return finished

    def idle(self) -> bool:
        return self.queue.empty() and not self.waiting and not self.groups

    def run_until_idle(self, timeout: float = 600.0):
        t_end = time.perf_counter() + timeout
        while not self.idle() and time.perf_counter() < t_end:
            self.step()

    # -- background loop -----------------------------------------------------------
    def start(self):
        def loop():
            torch.cuda.set_device(self.device)
            while not self._stop.is_set():
                if self.idle():
                    time.sleep(0.0002)
                    continue
                try:
                    self.step()
                except BaseException as exc:       # fail every pending request, keep serving
                    self._fail_all(exc)
        self._thread = threading.Thread(target=loop, daemon=True)
        self._thread.start()

    def _fail_all(self, exc: BaseException):
        pending = list(self.waiting)
        while True:
            try:
                pending.append(self.queue.get_nowait())
            except queue.Empty:
                break
        for g in self.groups.values():
            pending.extend(g.reqs + g.joining)
        self.waiting.clear()
        self.groups.clear()
        now = time.perf_counter()
        for r in pending:
            r.error = exc
            r.t_done = now
            r.done.set()

    def stop(self):
        self._stop.set()
        if self._thread is not None:
            self._thread.join(timeout=30)


def latency_summary(reqs) -> dict:
    lat = np.array([r.latency for r in reqs if r.done.is_set()])
    if lat.size == 0:
        return {"completed": 0}
    return {"completed": int(lat.size), "p50_ms": round(float(np.percentile(lat, 50)) * 1e3, 3),
            "p99_ms": round(float(np.percentile(lat, 99)) * 1e3, 3),
            "mean_ms": round(float(lat.mean()) * 1e3, 3)}
