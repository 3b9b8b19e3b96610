"""Batched multi-seed Personalized PageRank on a resident graph.

:class:`PPREngine` keeps one transition matrix resident in device memory as a
PBR matrix and answers many personalization vectors at once: every query
(a seed set, uniform weights) is one column of the iterate, so one fused
kernel launch per iteration advances all of them (``gl_ppr_step``).

Per-column retirement: columns whose L1 update falls below the tolerance are
frozen by the kernel (STOP_PER_COLUMN) and, at chunk boundaries, removed from
the working set — the still-active columns are gathered into a narrower
iterate, so later iterations move fewer bytes.  Iteration chunks are captured
once per working-set shape as CUDA graphs and replayed.

Dangling nodes (sources without out-edges) send their mass to the teleport
vector of each query (the missing-mass update of the reference's
``batched_ppr_update_kernel``, ``kernels/ppr_kernel.cu:57-97``), so the matrix
stays sparse (the reference's ``normalize_transition_matrix`` instead adds a
dense 1/N column per dangling node, ``graph_link/__init__.py:200-206``).
"""
from __future__ import annotations

import time
from dataclasses import dataclass, field

import numpy as np
import scipy.sparse as sp
import torch

from . import native
from .pbr import _ptr, pbr_from_device_csr
from .ppr import PprRun, dangling_bitmap, teleport_from_seed_sets
from .trace import nvtx_range


def certified_tolerance(tol: float, alpha: float) -> float:
    """Update-size threshold that bounds the distance to the fixed point.

    The iteration is an alpha-contraction in L1 on probability vectors, so
    ||x_t - x*|| <= alpha / (1 - alpha) * ||x_t - x_{t-1}||; stopping when the
    update is below tol * (1 - alpha) / alpha guarantees ||x_t - x*|| <= tol."""
    return tol * (1.0 - alpha) / alpha


@dataclass
class BatchResult:
    X: torch.Tensor                     # [n, K] final vectors, column k = query k
    iterations: np.ndarray              # per column: iterations to convergence (-1 = not converged)
    launched_iterations: int            # fused steps launched over the whole batch
    converged: np.ndarray
    seconds: float
    column_steps: int = 0               # sum over launched steps of the working-set width
    history: list = field(default_factory=list)


class PPREngine:
    """A transition matrix resident on one GPU, ready for batched PPR."""

    def __init__(self, A: sp.csr_matrix, block_size: int = 8, min_nnz_per_block: int | None = None,
                 device=None, dangling: np.ndarray | None = None, column_tile: int = 0):
        dev = torch.device(device) if device is not None else torch.device("cuda")
        self.device = dev if dev.index is not None else torch.device("cuda", torch.cuda.current_device())
        if A.shape[0] != A.shape[1]:
            raise ValueError("transition matrix must be square")
        if not A.has_canonical_format:
            A = A.copy()
            A.sum_duplicates()
        self.n = A.shape[0]
        self.block_size = int(block_size)
        self.min_nnz = int(block_size if min_nnz_per_block is None else min_nnz_per_block)
        with torch.cuda.device(self.device):
            indptr = torch.from_numpy(A.indptr.astype(np.int32)).to(self.device)
            indices = torch.from_numpy(A.indices.astype(np.int32)).to(self.device)
            data = torch.from_numpy(A.data.astype(np.float32)).to(self.device)
            self.pbr = pbr_from_device_csr(indptr, indices, data, self.n, self.n, self.block_size,
                                           self.block_size, self.min_nnz)
            # the device CSR stays resident for the window-solve warm start
            self.csr = (indptr, indices, data)
            self.mat = self.pbr.to(self.device)
            from .graph_link.pbr_registry import get_pbr_gpu_meta
            self.meta = get_pbr_gpu_meta(self.mat)
            self.meta["column_tile"] = int(column_tile)
            if dangling is None:
                self.dbits = dangling_bitmap(indices, self.n)
            else:
                self.dbits = _bitmap_from_mask(np.asarray(dangling, bool), self.device)
        self.nnz = int(A.nnz)
        self.host_indptr = A.indptr
        self.host_indices = A.indices
        self._graphs: dict = {}

    # -- sizes ----------------------------------------------------------------
    def matrix_bytes(self) -> int:
        """Device bytes of the resident matrix (PBR arrays, stripe index,
        load-balance schedule)."""
        tot = sum(t.numel() * t.element_size() for t in self.meta.values() if isinstance(t, torch.Tensor))
        sched = self.meta.get("schedule")
        if sched is not None:
            tot += sched["buffer"].numel() * sched["buffer"].element_size()
        return int(tot + self.dbits.numel() * self.dbits.element_size())

    def iteration_bytes(self, k: int) -> int:
        """Algorithmic HBM bytes of one fused step with k columns: the matrix
        structure once, X_t read once, X_{t+1} written once."""
        nb = self.meta["codes"].numel()
        packed = self.meta["data"].numel()
        rem = self.meta["rem_col_ind"].numel()
        return 20 * nb + 4 * packed + 4 * (self.n + 1) + 8 * rem + 8 * self.n * k

    # -- queries --------------------------------------------------------------
    def teleport(self, seed_sets) -> tuple:
        """(seed_ptr [K+1], unique seed rows, weights) on the device: column k
        teleports to the distinct seeds of set k, each weighted by its
        multiplicity over the set's size (duplicates inside a set merge into
        one weighted entry, so the step's epilogue sees unique (row, column)
        pairs)."""
        ptr, rows, w = seed_set_index(seed_sets)
        dev = self.device
        return (torch.from_numpy(ptr).to(dev), torch.from_numpy(rows).to(dev), torch.from_numpy(w).to(dev))

    def teleport_columns(self, seed_sets, tel: tuple | None = None) -> torch.Tensor:
        """Dense teleport (personalization) vectors [n, K] of the seed sets
        (``tel``: their ``teleport()`` index, when the caller has it)."""
        ptr, rows, w = self.teleport(seed_sets) if tel is None else tel
        tp = teleport_from_seed_sets(ptr, rows, self.n, self.block_size, w)
        V = torch.empty((self.n, len(seed_sets)), dtype=torch.float32, device=self.device)
        native.check(native.lib().gl_ppr_init(tp.desc(), self.n, len(seed_sets), native.GL_F32, V.data_ptr(),
                                              None, None, torch.cuda.current_stream(self.device).cuda_stream))
        return V

    def solve(self, seed_sets, alpha: float = 0.85, tol: float = 1e-6, max_iterations: int = 1000,
              certified: bool = True, retire: bool = True, chunk: int = 8, x0: torch.Tensor | None = None,
              use_graphs: bool = True, compact_ratio: float = 0.75, warm_start=None) -> BatchResult:
        """Personalized PageRank for every seed set (one column each).

        ``certified`` stops a column once its update is below
        ``certified_tolerance(tol, alpha)`` so its distance to the exact fixed
        point is at most ``tol`` in L1; otherwise the update itself is compared
        with ``tol`` (the reference's rule).  ``warm_start`` (a trained
        ``warmstart.WarmStart`` of this engine) supplies the start columns
        when ``x0`` is not given; the fixed point is the same."""
        with nvtx_range(f"engine.solve K={len(seed_sets)}"):
            return self._solve(seed_sets, alpha, tol, max_iterations, certified, retire, chunk, x0, use_graphs,
                               compact_ratio, warm_start)

    def _solve(self, seed_sets, alpha, tol, max_iterations, certified, retire, chunk, x0, use_graphs,
               compact_ratio, warm_start) -> BatchResult:
        K = len(seed_sets)
        dev = self.device
        t0 = time.perf_counter()   # the solve's time includes the warm start's prediction
        warm_columns = None
        pre_steps = 0
        x0_owned = False                # x0 is ours to overwrite (not the caller's)
        if warm_start is not None and x0 is None:
            x0, warm_columns = warm_start.start_vectors(seed_sets, alpha)
            # steps the start already took from its vector (they count as
            # iterations of the columns that kept it)
            pre_steps = int(getattr(warm_start, "pre_steps", 0))
            x0_owned = True
        thr = certified_tolerance(tol, alpha) if certified else tol
        with torch.cuda.device(dev):
            ptr, rows, w = self.teleport(seed_sets)
            out = None                  # allocated when a run ends with columns still going
            col_iter = np.full(K, -1, dtype=np.int64)
            active = np.arange(K)
            cur_x0 = x0
            done = 0
            launched = 0
            column_steps = 0
            history = []
            while active.size and done < max_iterations:
                sub_ptr, sub_rows, sub_w = _select_columns(ptr, rows, w, active)
                tp = teleport_from_seed_sets(sub_ptr, sub_rows, self.n, self.block_size, sub_w)
                run = PprRun(self.meta, self.n, self.n, self.block_size, self.block_size, tp, alpha,
                             max_iterations - done, thr,
                             native.GL_PPR_STOP_PER_COLUMN if retire else native.GL_PPR_STOP_ALL,
                             self.dbits)
                run.init(cur_x0, adopt=x0_owned or cur_x0 is not x0)
                graph = None
                steps = 0            # steps launched in this run
                written = 0          # steps that wrote a new iterate
                stop_all_at = None
                fin = np.zeros(active.size, dtype=bool)
                while steps < run.max_iterations:
                    # a run's first chunk is launched directly: warm-started
                    # and nearly finished runs often end inside it, where a
                    # captured graph would not repay its capture
                    if use_graphs and steps > 0:
                        if graph is None:
                            graph = self._capture(run, chunk)
                        graph.replay()
                    else:
                        run.launch_chunk(chunk)
                    n_valid = min(chunk, run.max_iterations - steps)
                    res = run.res_hist[steps:steps + n_valid].cpu().numpy()   # syncs
                    for t in range(n_valid):
                        row = res[t]
                        history.append(float(row.max()))
                        newly = (~fin) & (row < thr)
                        col_iter[active[newly]] = done + steps + t + 1
                        fin |= newly
                        if not retire and (row < thr).all():
                            stop_all_at = steps + t + 1
                            break
                    launched += n_valid if stop_all_at is None else stop_all_at - steps
                    column_steps += (n_valid if stop_all_at is None else stop_all_at - steps) * active.size
                    steps += n_valid
                    written = steps if stop_all_at is None else stop_all_at
                    if fin.all() or stop_all_at is not None:
                        break
                    if retire and fin.any() and fin.sum() >= (1.0 - compact_ratio) * active.size:
                        break   # compact: restart with the still-active columns
                Xcur = run.bufs[written % 2]
                done += written
                keep = ~fin if retire else np.zeros(active.size, dtype=bool)
                if not retire or done >= max_iterations:
                    keep_out = np.ones(active.size, dtype=bool)
                else:
                    keep_out = ~keep
                sel = np.nonzero(keep_out)[0]
                if sel.size == K and out is None:
                    out = Xcur          # the whole batch ended in this run, in column order
                elif sel.size:
                    if out is None:
                        out = torch.empty((self.n, K), dtype=torch.float32, device=dev)
                    out[:, torch.from_numpy(active[sel]).to(dev)] = Xcur[:, torch.from_numpy(sel).to(dev)]
                if retire and keep.any() and done < max_iterations:
                    cur_x0 = Xcur[:, torch.from_numpy(np.nonzero(keep)[0]).to(dev)].contiguous()
                    active = active[keep]
                else:
                    active = active[:0]
            if out is None:             # max_iterations = 0
                out = torch.empty((self.n, K), dtype=torch.float32, device=dev)
            torch.cuda.synchronize(dev)
        if isinstance(warm_columns, torch.Tensor):
            warm_columns = warm_columns.cpu().numpy()
        if pre_steps:
            col_iter[np.asarray(warm_columns, bool) & (col_iter >= 0)] += pre_steps
            launched += pre_steps
            column_steps += pre_steps * K
        res = BatchResult(X=out, iterations=col_iter, launched_iterations=launched,
                          converged=col_iter >= 0, seconds=time.perf_counter() - t0,
                          column_steps=column_steps, history=history)
        if warm_columns is not None:
            res.warm_columns = warm_columns
        return res

    def solve_plain(self, seed_sets, alpha: float = 0.85, tol: float = 1e-6, max_iterations: int = 1000,
                    certified: bool = True) -> BatchResult:
        """One query at a time (K = 1 per run): the plain GPU path batched
        queries are compared against."""
        K = len(seed_sets)
        t0 = time.perf_counter()
        out = torch.empty((self.n, K), dtype=torch.float32, device=self.device)
        its = np.full(K, -1, dtype=np.int64)
        launched = 0
        for k, s in enumerate(seed_sets):
            r = self.solve([s], alpha, tol, max_iterations, certified=certified, retire=False, chunk=8,
                           use_graphs=False)
            out[:, k] = r.X[:, 0]
            its[k] = r.iterations[0]
            launched += r.launched_iterations
        torch.cuda.synchronize(self.device)
        return BatchResult(X=out, iterations=its, launched_iterations=launched, converged=its >= 0,
                           seconds=time.perf_counter() - t0, column_steps=launched)

    def _capture(self, run: PprRun, chunk: int):
        """CUDA graph of one chunk of steps for this run's buffers."""
        return run.capture(chunk)


def seed_set_index(seed_sets) -> tuple[np.ndarray, np.ndarray, np.ndarray]:
    """Host CSR of seed sets: (ptr int32 [K+1], distinct rows per set in
    increasing order int32, weight float32 = multiplicity / set size)."""
    K = len(seed_sets)
    lens = np.fromiter((len(s) for s in seed_sets), count=K, dtype=np.int64)
    if K == 0 or lens.sum() == 0:
        return np.zeros(K + 1, np.int32), np.zeros(0, np.int32), np.zeros(0, np.float32)
    cols = np.repeat(np.arange(K, dtype=np.int64), lens)
    idx = np.concatenate([np.asarray(s, dtype=np.int64).ravel() for s in seed_sets])
    order = np.lexsort((idx, cols))
    c, r = cols[order], idx[order]
    head = np.ones(r.size, dtype=bool)
    head[1:] = (c[1:] != c[:-1]) | (r[1:] != r[:-1])
    starts = np.flatnonzero(head)
    mult = np.diff(np.append(starts, r.size))
    uc, ur = c[starts], r[starts]
    ptr = np.zeros(K + 1, dtype=np.int32)
    ptr[1:] = np.cumsum(np.bincount(uc, minlength=K))
    w = (mult / lens[uc]).astype(np.float32)
    return ptr, ur.astype(np.int32), w


def _select_columns(ptr: torch.Tensor, rows: torch.Tensor, w: torch.Tensor, active: np.ndarray):
    p = ptr.cpu().numpy()
    r = rows.cpu().numpy()
    ww = w.cpu().numpy()
    lens = p[active + 1] - p[active]
    new_ptr = np.zeros(len(active) + 1, dtype=np.int32)
    new_ptr[1:] = np.cumsum(lens)
    idx = np.concatenate([np.arange(p[a], p[a + 1]) for a in active]) if len(active) else np.zeros(0, np.int64)
    dev = ptr.device
    return (torch.from_numpy(new_ptr).to(dev), torch.from_numpy(r[idx].astype(np.int32)).to(dev),
            torch.from_numpy(ww[idx].astype(np.float32)).to(dev))


def _bitmap_from_mask(mask: np.ndarray, device) -> torch.Tensor:
    n = mask.size
    words = max(1, -(-n // 32))
    pad = np.zeros(words * 32, dtype=np.uint64)
    pad[:n] = mask
    packed = (pad.reshape(words, 32) << np.arange(32, dtype=np.uint64)).sum(axis=1).astype(np.uint32)
    return torch.from_numpy(packed.view(np.int32)).to(device)
