"""Device-side Personalized PageRank runs over a registered PBR matrix.

One run owns two [rows, K] iterate buffers, a residual history
[max_iterations, K] and a dangling-mass history [max_iterations + 1, K]
(float64), and a device iteration counter.  Steps are launched in chunks;
each step is one fused kernel (``gl_ppr_step``) that skips itself once the
run has converged, so the host only synchronizes once per chunk instead of
once per iteration (the reference syncs every iteration with ``.item()``,
``graph_link/__init__.py:262``).
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np
import torch

from . import native
from .pbr import _ptr, matrix_desc
from .trace import nvtx_range


@dataclass
class Teleport:
    """Teleport vectors indexed by stripe (see ``gl_teleport``)."""

    stripe_ptr: torch.Tensor
    row: torch.Tensor
    col: torch.Tensor
    weight: torch.Tensor
    num_columns: int

    def desc(self) -> native.TeleportDesc:
        d = native.TeleportDesc()
        d.stripe_ptr = _ptr(self.stripe_ptr)
        d.row = _ptr(self.row)
        d.col = _ptr(self.col)
        d.weight = _ptr(self.weight)
        d.num_entries = int(self.row.numel())
        return d


def teleport_from_seed_sets(seed_ptr: torch.Tensor, seed_idx: torch.Tensor, rows: int,
                            block_rows: int, seed_weight: torch.Tensor | None = None) -> Teleport:
    """Column k teleports to seeds ``seed_idx[seed_ptr[k]:seed_ptr[k+1]]``, each
    with weight ``seed_weight`` (default 1/|set|)."""
    dev = seed_idx.device
    K = int(seed_ptr.numel()) - 1
    n = int(seed_idx.numel())
    ns = -(-rows // block_rows)
    seed_ptr = seed_ptr.to(dev, torch.int32).contiguous()
    seed_idx = seed_idx.to(dev, torch.int32).contiguous()
    if seed_weight is not None:
        seed_weight = seed_weight.to(dev, torch.float32).contiguous()
    tp = Teleport(stripe_ptr=torch.empty(ns + 1, dtype=torch.int32, device=dev),
                  row=torch.empty(n, dtype=torch.int32, device=dev),
                  col=torch.empty(n, dtype=torch.int32, device=dev),
                  weight=torch.empty(n, dtype=torch.float32, device=dev),
                  num_columns=K)
    scratch = torch.empty(ns + 1, dtype=torch.int32, device=dev)
    native.check(native.lib().gl_ppr_teleport_index(
        rows, block_rows, K, seed_ptr.data_ptr(), _ptr(seed_idx), _ptr(seed_weight), n,
        tp.stripe_ptr.data_ptr(), _ptr(tp.row), _ptr(tp.col), _ptr(tp.weight),
        scratch.data_ptr(), torch.cuda.current_stream(dev).cuda_stream))
    return tp


def dangling_bitmap(col_ind: torch.Tensor, rows: int) -> torch.Tensor:
    """uint32 bitmap (as int32 tensor) of the columns with no stored entry.

    For a column-normalized transition matrix those are the dangling nodes
    (no out-edges), whose mass the dangling update sends to the teleport
    vector."""
    dev = col_ind.device
    present = torch.zeros(rows, dtype=torch.bool, device=dev)
    if col_ind.numel():
        present[col_ind.long()] = True
    dang = (~present).to(torch.int64)
    words = -(-rows // 32)
    pad = torch.zeros(words * 32, dtype=torch.int64, device=dev)
    pad[:rows] = dang
    weights = (torch.ones(32, dtype=torch.int64, device=dev) << torch.arange(32, device=dev))
    packed = (pad.view(words, 32) * weights).sum(dim=1)
    return packed.to(torch.int64).bitwise_and(0xFFFFFFFF).to(torch.int32) if words else \
        torch.zeros(1, dtype=torch.int32, device=dev)


@dataclass
class PprResult:
    X: torch.Tensor
    iterations: int
    converged: bool
    history: list = field(default_factory=list)
    column_iterations: np.ndarray | None = None


class PprRun:
    """State of one batched power iteration (K columns) over one matrix."""

    def __init__(self, meta: dict, rows: int, cols: int, block_rows: int, block_cols: int,
                 teleport: Teleport, alpha: float, max_iterations: int, tol: float,
                 stop_mode: int = native.GL_PPR_STOP_ALL, dangling_bits: torch.Tensor | None = None,
                 dangling_target: int = native.GL_DANGLING_TO_TELEPORT):
        if rows != cols:
            raise ValueError("personalized PageRank needs a square matrix")
        self.meta = meta
        self.rows, self.cols = rows, cols
        self.block_rows, self.block_cols = block_rows, block_cols
        self.tp = teleport
        self.K = teleport.num_columns
        dev = meta["data"].device
        # alpha / tol: one value for all columns, or one per column (a column
        # of the batch then runs exactly as it would alone with its own pair)
        self.col_alpha = self.col_tol = None
        if np.ndim(alpha):
            a = np.asarray(alpha, dtype=np.float64)
            if a.shape != (self.K,):
                raise ValueError("alpha must be a scalar or have one entry per column")
            self.col_alpha = torch.from_numpy(a).to(dev)
            alpha = float(a.max()) if a.size else 0.85
        if np.ndim(tol):
            tv = np.asarray(tol, dtype=np.float64)
            if tv.shape != (self.K,):
                raise ValueError("tol must be a scalar or have one entry per column")
            self.col_tol = torch.from_numpy(tv).to(dev)
            self.tol_host = tv
            tol = float(tv.min()) if tv.size else 0.0
        else:
            self.tol_host = np.full(self.K, float(tol))
        self.alpha = float(alpha)
        self.max_iterations = int(max_iterations)
        self.tol = float(tol)
        self.stop_mode = stop_mode
        self.dangling_bits = dangling_bits
        self.dangling_target = dangling_target
        dtype = meta["data"].dtype
        self.device = dev
        self.bufs = [torch.empty((rows, self.K), dtype=dtype, device=dev),
                     torch.empty((rows, self.K), dtype=dtype, device=dev)]
        self.res_hist = torch.zeros((max(self.max_iterations, 1), self.K), dtype=torch.float64, device=dev)
        self.dang_hist = torch.zeros((self.max_iterations + 1, self.K), dtype=torch.float64, device=dev)
        self.chunk_base = torch.zeros(1, dtype=torch.int32, device=dev)
        self._desc = matrix_desc(meta, rows, cols, block_rows, block_cols)
        nbytes = int(native.lib().gl_pbr_spmm_workspace_bytes(self._desc, 1, self.K))
        # owned by this run: a run's steps are stream-ordered, never concurrent
        self.ws = torch.zeros(max(nbytes, 1), dtype=torch.uint8, device=dev)
        self._ws_bytes = max(nbytes, 0)
        self._tpd = teleport.desc()
        self._vtype = native.GL_F32 if dtype == torch.float32 else native.GL_F64
        self._params = []

    def _stream(self) -> int:
        return torch.cuda.current_stream(self.device).cuda_stream

    def init(self, x0: torch.Tensor | None = None, adopt: bool = False) -> None:
        """Start from the teleport vectors, or from x0 (copied; with ``adopt``
        a contiguous x0 of the right shape and type becomes the first
        iterate buffer itself and is overwritten by the run)."""
        L = native.lib()
        st = self._stream()
        dbits = _ptr(self.dangling_bits)
        if x0 is None:
            native.check(L.gl_ppr_init(self._tpd, self.rows, self.K, self._vtype,
                                       self.bufs[0].data_ptr(), dbits,
                                       self.dang_hist[0].data_ptr() if dbits else None, st))
        else:
            if (adopt and x0.is_contiguous() and x0.shape == self.bufs[0].shape and x0.dtype == self.bufs[0].dtype
                    and x0.device == self.bufs[0].device and x0.data_ptr() != self.bufs[1].data_ptr()):
                self.bufs[0] = x0
            else:
                self.bufs[0].copy_(x0)
            if dbits:
                native.check(L.gl_ppr_dangling_mass(self.bufs[0].data_ptr(), self.rows, self.K,
                                                    self._vtype, dbits, self.dang_hist[0].data_ptr(),
                                                    st))

    def _step_params(self, i: int) -> native.PprStepParams:
        while len(self._params) <= i:
            p = native.PprStepParams()
            p.alpha = self.alpha
            p.tol = self.tol
            p.stop_mode = self.stop_mode
            p.max_iterations = self.max_iterations
            p.step_in_chunk = len(self._params)
            p.chunk_base = self.chunk_base.data_ptr()
            p.residual_hist = self.res_hist.data_ptr()
            p.dangling_hist = self.dang_hist.data_ptr()
            p.dangling_bitmap = _ptr(self.dangling_bits)
            p.dangling_target = self.dangling_target
            p.column_alpha = _ptr(self.col_alpha)
            p.column_tol = _ptr(self.col_tol)
            self._params.append(p)
        return self._params[i]

    def _warm_params(self, n: int) -> None:
        """Create the step parameters for a chunk of n steps and make the
        launcher run its one-time occupancy query with a step that returns at
        once (iteration index past max_iterations), so that a following CUDA
        graph capture records kernel launches only."""
        for i in range(n):
            self._step_params(i)
        p = native.PprStepParams()
        ctypes_copy = self._step_params(0)
        for name, _ in native.PprStepParams._fields_:
            setattr(p, name, getattr(ctypes_copy, name))
        p.step_in_chunk = 1 << 30
        native.check(native.lib().gl_ppr_step(self._desc, self._tpd, self.bufs[0].data_ptr(),
                                              self.bufs[1].data_ptr(), self.K, p, self.ws.data_ptr(),
                                              self._ws_bytes, self._stream()))

    def launch_chunk(self, n: int) -> None:
        """Launch n (even) steps starting at the device counter, then advance it."""
        L = native.lib()
        st = self._stream()
        with nvtx_range(f"ppr.chunk K={self.K}"):
            for i in range(n):
                native.check(L.gl_ppr_step(self._desc, self._tpd, self.bufs[i % 2].data_ptr(),
                                           self.bufs[(i + 1) % 2].data_ptr(), self.K,
                                           self._step_params(i), self.ws.data_ptr(), self._ws_bytes, st))
            native.check(L.gl_counter_add(self.chunk_base.data_ptr(), n, st))

    def run_native(self, chunk: int = 8, x0: torch.Tensor | None = None) -> PprResult:
        """The same run with the loop inside the library (``gl_ppr_run``):
        chunks of fused steps, one residual read per chunk."""
        chunk = max(2, chunk + (chunk % 2))
        if x0 is not None:
            self.bufs[0].copy_(x0)
        p = self._step_params(0)
        out = native.PprRunResult()
        col_it = np.full(self.K, -1, dtype=np.int32)
        native.check(native.lib().gl_ppr_run(
            self._desc, self._tpd, self.bufs[0].data_ptr(), self.bufs[1].data_ptr(), self.K, p,
            1 if x0 is None else 0, chunk, self.ws.data_ptr(), self._ws_bytes,
            col_it.ctypes.data if self.K else None, out, self._stream()))
        return PprResult(X=self.bufs[out.result_in_x1], iterations=int(out.iterations),
                         converged=bool(out.converged), column_iterations=col_it.astype(np.int64))

    def capture(self, chunk: int):
        """CUDA graph of one chunk of steps over this run's buffers (the steps
        read their iteration number from the device counter, so one graph
        serves every chunk)."""
        dev = self.device
        s = torch.cuda.Stream(dev)
        s.wait_stream(torch.cuda.current_stream(dev))
        g = torch.cuda.CUDAGraph()
        with torch.cuda.stream(s):
            self._warm_params(chunk)
        with torch.cuda.graph(g, stream=s):
            self.launch_chunk(chunk)
        torch.cuda.current_stream(dev).wait_stream(s)
        return g   # capturing does not execute: the counter is still at its base

    def run(self, chunk: int = 8, x0: torch.Tensor | None = None, use_graph: bool = False) -> PprResult:
        """Iterate until the stop rule holds; ``use_graph`` replays one
        captured chunk (capturing costs about as much as the launches it
        saves for one query, so it pays only when a run is long)."""
        chunk = max(2, chunk + (chunk % 2))
        self.init(x0)
        graph = self.capture(chunk) if use_graph else None
        history: list[float] = []
        col_iter = np.full(self.K, -1, dtype=np.int64)
        iterations = self.max_iterations
        converged = False
        done = 0
        while done < self.max_iterations:
            if graph is not None:
                graph.replay()
            else:
                self.launch_chunk(chunk)
            n = min(chunk, self.max_iterations - done)
            res = self.res_hist[done:done + n].cpu().numpy()  # synchronizes the stream
            finished = False
            for t in range(n):
                row = res[t]
                history.append(float(row.max()) if self.K else 0.0)
                newly = (col_iter < 0) & (row < self.tol_host)
                col_iter[newly] = done + t + 1
                if self.stop_mode == native.GL_PPR_STOP_ALL:
                    if self.K and row.max() < self.tol:
                        iterations = done + t + 1
                        converged = True
                        finished = True
                        break
                elif (col_iter >= 0).all():
                    iterations = done + t + 1
                    converged = True
                    finished = True
                    break
            done += n
            if finished:
                break
        if self.stop_mode == native.GL_PPR_STOP_PER_COLUMN:
            # Every launched step wrote the next buffer (frozen columns are
            # copied), so the final state is the last buffer written.
            steps_run = min(done, self.max_iterations)
            X = self.bufs[steps_run % 2]
        else:
            X = self.bufs[iterations % 2]
        return PprResult(X=X, iterations=iterations, converged=converged, history=history,
                         column_iterations=col_iter)
