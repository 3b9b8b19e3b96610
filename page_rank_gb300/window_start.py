"""Window-solve warm start for batched PPR.

The PPR vector of a seed set solves (I - alpha A) x = (1 - alpha) v.  With the
node order cut into windows of 64 rows, A = D + M splits into its diagonal
64 x 64 window blocks D and the edges M that leave their window, and

    x = (1 - alpha) (y_0 + y_1 + ...),   y_0 = B^-1 v,   y_k = B^-1 (alpha M y_{k-1}),

with B = I - alpha D (block diagonal).  The k-th term is the mass of walks
that left their window k times; on graphs whose node order keeps
communities together (the cluster / Zipf class keeps 80 % of each node's
edges inside its 64-node cluster) the first few terms hold most of the mass.
The start vector is that truncated series (the "near field", computed
exactly: ``leaves`` applications of M, each followed by the windows' dense
inverses, ``csrc/window_start.cu``) plus the mass it misses, spread along a
far-field shape:

* ``"expected"`` (default): the far field of the uniform teleport vector,
  normalized — solved directly as the PPR vector whose teleport is where
  the uniform vector's next window exits land.  For seed sets drawn
  uniformly at random this is the expected far field of a query (PPR is
  linear in v), computed once per graph and damping factor.
* ``"pagerank"``: the global PageRank vector.
* ``"learned"``: a per-node density predicted by the warm-start network
  (``warmstart.FarFieldModel``) from node features, trained on far fields of
  PPR vectors the plain method computed.

The power iteration then runs from that vector to the usual certified
tolerance, so the fixed point does not depend on the start.  A column falls
back to the cold start (its teleport vector) when one step from the window
start leaves a larger residual than one step from the teleport vector would
(the teleport vector's residual is computed exactly from the seed rows,
``gl_cold_residual``); the step taken from the window start is the first
iteration of the columns that keep it.
"""
from __future__ import annotations

import time

import numpy as np
import torch

from . import native
from .engine import PPREngine
from .pbr import matrix_desc, pbr_from_device_csr, spmm_workspace
from .ppr import PprRun, teleport_from_seed_sets

WINDOW = 64
SHAPES = ("expected", "pagerank", "learned")
# window exits the start follows by default: on the cluster / Zipf class the
# wall time of a 256-query batch fell up to 8 (2**21 nodes: 0.280 s cold,
# 0.084 s from the start with 8 exits)
DEFAULT_LEAVES = 8


def _stream(dev) -> int:
    return torch.cuda.current_stream(dev).cuda_stream


class _OffWindow:
    """The edges of A that leave their 64-row window, as a resident PBR matrix."""

    def __init__(self, eng: PPREngine):
        indptr, indices, data = eng.csr
        n = eng.n
        dev = eng.device
        counts = (indptr[1:] - indptr[:-1]).to(torch.int64)
        rows = torch.repeat_interleave(torch.arange(n, device=dev, dtype=torch.int64), counts)
        keep = (rows >> 6) != (indices.to(torch.int64) >> 6)
        rows = rows[keep]
        self.nnz = int(rows.numel())
        ind = indices[keep].contiguous()
        val = data[keep].contiguous()
        # per source node: the transition mass that leaves its window
        self.leak = torch.zeros(n, dtype=torch.float64, device=dev).index_add_(
            0, ind.to(torch.int64), val.to(torch.float64)).to(torch.float32)
        ptr = torch.zeros(n + 1, dtype=torch.int64, device=dev)
        ptr[1:] = torch.cumsum(torch.bincount(rows, minlength=n), 0)
        del rows, keep
        self.pbr = pbr_from_device_csr(ptr.to(torch.int32), ind, val, n, n, eng.block_size, eng.block_size,
                                       eng.min_nnz).to(dev)
        from .graph_link.pbr_registry import get_pbr_gpu_meta
        self.meta = get_pbr_gpu_meta(self.pbr)
        self.desc = matrix_desc(self.meta, n, n, eng.block_size, eng.block_size)
        self.n = n
        self.dev = dev

    def spmm(self, X: torch.Tensor, Y: torch.Tensor) -> None:
        K = X.shape[1]
        ws = spmm_workspace(self.meta, self.desc, 1, K, self.dev)     # cached per shape and stream
        native.check(native.lib().gl_pbr_spmm(self.desc, X.data_ptr(), Y.data_ptr(), 1, K,
                                              ws.data_ptr() if ws is not None else None,
                                              ws.numel() if ws is not None else 0, _stream(self.dev)))


class WindowStart:
    """Window-solve start vectors for one engine (see the module docstring).

    Per damping factor the windows' inverses and the far-field shape are
    built on first use and kept; ``leaves`` is the number of times the
    series follows the edges that leave a window."""

    def __init__(self, engine: PPREngine, leaves: int = DEFAULT_LEAVES, shape: str = "expected", gate=None,
                 fallback: bool = True, far_field_model=None):
        if shape not in SHAPES:
            raise ValueError(f"shape must be one of {SHAPES}")
        if leaves < 0:
            raise ValueError("leaves must be >= 0")
        if shape == "learned" and far_field_model is None:
            raise ValueError("shape 'learned' needs a trained far_field_model")
        self.eng = engine
        self.dev = engine.device
        self.leaves = int(leaves)
        self.shape_kind = shape
        self.gate = gate
        self.fallback = bool(fallback)
        self.model = far_field_model
        self.windows = -(-engine.n // WINDOW)
        self.pre_steps = 0
        self._pending: list = []
        self._alpha: dict = {}
        self.setup_seconds: dict = {}
        self.setup_phases: dict = {}
        with torch.cuda.device(self.dev):
            self.off = _OffWindow(engine)
            indptr, indices, data = engine.csr
            self.colsum = torch.zeros(engine.n, dtype=torch.float64, device=self.dev)
            self.colsum.index_add_(0, indices.to(torch.int64), data.to(torch.float64))

    # -- per damping factor -----------------------------------------------------
    def inverses(self, alpha: float) -> torch.Tensor:
        return self._prepare(alpha)["inv"]

    def _prepare(self, alpha: float) -> dict:
        key = round(float(alpha), 12)
        st = self._alpha.get(key)
        if st is not None:
            return st
        t0 = time.perf_counter()
        eng = self.eng
        L = native.lib()
        s = _stream(self.dev)
        indptr, indices, data = eng.csr
        inv = torch.empty((self.windows, WINDOW, WINDOW), dtype=torch.float32, device=self.dev)
        native.check(L.gl_window_blocks(indptr.data_ptr(), indices.data_ptr(), data.data_ptr(), eng.n,
                                        float(alpha), inv.data_ptr(), s))
        status = torch.zeros(1, dtype=torch.int32, device=self.dev)
        native.check(L.gl_window_invert(inv.data_ptr(), eng.n, status.data_ptr(), s))
        if int(status.item()) != 0:
            raise ValueError("a window block is not invertible without pivoting: the transition matrix's "
                             "columns must sum to at most 1")
        t1 = time.perf_counter()       # the status read above waited for the inversion
        st = {"inv": inv, "alpha": float(alpha)}
        self._alpha[key] = st          # the far-field shapes below use the inverses
        try:
            st["near_uniform"], st["expected"] = self._expected_far_field(alpha)
            st["shape"] = self._shape(st)
        except BaseException:
            del self._alpha[key]
            raise
        torch.cuda.synchronize(self.dev)
        t2 = time.perf_counter()
        self.setup_seconds[key] = t2 - t0
        self.setup_phases[key] = {"inverses_s": round(t1 - t0, 4), "far_field_s": round(t2 - t1, 4)}
        return st

    def pagerank(self, alpha: float) -> torch.Tensor:
        """Global PageRank (uniform teleport) of the engine's graph, FP32 [n]
        (computed on first use: the ``pagerank`` shape and the learned model's
        features need it, the default start does not)."""
        st = self._prepare(alpha)
        if "pagerank" not in st:
            n = self.eng.n
            res = self.eng.solve([np.arange(n)], alpha=alpha, tol=1e-6, max_iterations=1000, retire=False,
                                 use_graphs=False)
            x = res.X[:, 0].clamp_min(0)
            st["pagerank"] = (x / x.sum()).contiguous()
        return st["pagerank"]

    def _shape(self, st: dict) -> torch.Tensor:
        if self.shape_kind == "expected":
            return st["expected"]
        if self.shape_kind == "pagerank":
            return self.pagerank(st["alpha"])
        return self.model.shape(self, st["alpha"])

    def set_shape(self, shape: str, far_field_model=None) -> None:
        """Switch the far-field shape (the inverses and PageRank vectors are
        kept); ``"learned"`` needs a trained model."""
        if shape not in SHAPES:
            raise ValueError(f"shape must be one of {SHAPES}")
        if shape == "learned" and far_field_model is None and self.model is None:
            raise ValueError("shape 'learned' needs a trained far_field_model")
        self.shape_kind = shape
        if far_field_model is not None:
            self.model = far_field_model
        for st in self._alpha.values():
            st["shape"] = self._shape(st)

    def _expected_far_field(self, alpha: float):
        """(near field of the uniform teleport vector u, u's far field
        normalized).

        The far field is the series' tail, (1 - alpha) sum_{k > L} y_k =
        (1 - alpha) (I - alpha A)^-1 (alpha M y_L): the PPR vector whose
        teleport is where the next window exits land, M y_L.  It is solved
        as such (one column, no dangling term in the landing vector; the
        graph's dangling mass returns through it as for any query) rather
        than as PageRank minus the near field, whose difference is a small
        fraction of either (about 1 % after 8 exits) and would carry their
        rounding and truncation errors magnified by that factor."""
        eng = self.eng
        n = eng.n
        _, tp, V = self._teleport([np.arange(n)])
        near, _, y_last = self._near_field(V, tp, alpha, want_last=True)
        land = torch.empty_like(y_last)
        self.off.spmm(y_last, land)
        land = land[:, 0].clamp_min(0)
        tot = land.sum()
        near = near[:, 0].contiguous()
        if not bool(tot > 0):                   # nothing leaves the windows: any shape will do
            return near, torch.full((n,), 1.0 / n, dtype=torch.float32, device=self.dev)
        land = (land / tot).to(torch.float32)
        rows = torch.nonzero(land > 0).flatten().to(torch.int32)
        ptr = torch.tensor([0, rows.numel()], dtype=torch.int32, device=self.dev)
        tpl = teleport_from_seed_sets(ptr, rows, n, eng.block_size, land[rows.long()].contiguous())
        run = PprRun(eng.meta, n, n, eng.block_size, eng.block_size, tpl, alpha, 1000,
                     1e-6 * (1.0 - alpha) / alpha, native.GL_PPR_STOP_ALL, eng.dbits)
        res = run.run(chunk=8)
        far = res.X[:, 0].clamp_min(0)
        return near, (far / far.sum()).contiguous()

    # -- start vectors ------------------------------------------------------------
    def _teleport(self, seed_sets, tel: tuple | None = None):
        """(teleport index, stripe-indexed teleport, dense teleport columns)."""
        eng = self.eng
        tel = eng.teleport(seed_sets) if tel is None else tel
        ptr, rows, w = tel
        tp = teleport_from_seed_sets(ptr, rows, eng.n, eng.block_size, w)
        return tel, tp, eng.teleport_columns(seed_sets, tel)

    def _near_field(self, V: torch.Tensor, tp, alpha: float, want_last: bool = False):
        """(near field [n, K], per-window column sums [windows, K]) of the
        teleport columns V.

        The series is summed term by term: y_0 = B^-1 v, then ``leaves``
        times T = M y (the off-window SpMM) and y = alpha B^-1 T, each term
        added into the near field as it is made (one fused apply).  Summing
        the terms keeps the rounding of the large early terms out of the
        later ones; re-solving the whole near field in every sweep (the
        equivalent block-Jacobi iteration nf <- B^-1 (alpha M nf + (1 - alpha)
        v)) put FP32 rounding of the full vector into each sweep and needed
        two more certification steps at 8 exits on the 2**21-node graph.
        ``tp`` (the same vectors, stripe-indexed) is not needed here."""
        st = self._prepare(alpha)
        L = native.lib()
        s = _stream(self.dev)
        n, K = V.shape
        inv = st["inv"]
        a = float(alpha)
        nf = torch.empty_like(V)
        partial = torch.empty((self.windows, K), dtype=torch.float32, device=self.dev)
        Y = torch.empty_like(V) if (self.leaves or want_last) else None
        native.check(L.gl_window_apply(inv.data_ptr(), n, K, V.data_ptr(), 1.0,
                                       Y.data_ptr() if Y is not None else None, nf.data_ptr(), 1.0 - a, 1,
                                       partial.data_ptr(), s))
        if self.leaves:
            T = torch.empty_like(V)
            for k in range(1, self.leaves + 1):
                self.off.spmm(Y, T)
                last = k == self.leaves and not want_last
                native.check(L.gl_window_apply(inv.data_ptr(), n, K, T.data_ptr(), a,
                                               None if last else Y.data_ptr(), nf.data_ptr(), 1.0 - a, 0,
                                               partial.data_ptr(), s))
        if want_last:
            return nf, partial, Y
        return nf, partial

    def near_field(self, seed_sets, alpha: float) -> torch.Tensor:
        """The exact truncated series (no far field) for the seed sets [n, K]."""
        _, tp, V = self._teleport(seed_sets)
        return self._near_field(V, tp, alpha)[0]

    def start(self, seed_sets, alpha: float = 0.85) -> torch.Tensor:
        """Window-start columns [n, K] (each sums to 1) for the seed sets."""
        st = self._prepare(alpha)
        _, tp, V = self._teleport(seed_sets)
        return self._start_from(V, st, tp)

    def _start_from(self, V: torch.Tensor, st: dict, tp) -> torch.Tensor:
        n, K = V.shape
        nf, partial = self._near_field(V, tp, st["alpha"])
        nbytes = native.lib().gl_window_finalize_workspace_bytes(n, K)
        ws = torch.empty(max(int(nbytes), 1), dtype=torch.uint8, device=self.dev)
        native.check(native.lib().gl_window_finalize(nf.data_ptr(), n, K, partial.data_ptr(),
                                                     st["shape"].data_ptr(), ws.data_ptr(), ws.numel(),
                                                     _stream(self.dev)))
        return nf

    def _cold_residuals_device(self, seed_sets, alpha: float, tel: tuple | None = None) -> torch.Tensor:
        eng = self.eng
        ptr, rows, w = eng.teleport(seed_sets) if tel is None else tel
        out = torch.empty(len(seed_sets), dtype=torch.float64, device=self.dev)
        indptr, indices, data = eng.csr
        native.check(native.lib().gl_cold_residual(
            indptr.data_ptr(), indices.data_ptr(), data.data_ptr(), self.colsum.data_ptr(),
            eng.dbits.data_ptr() if eng.dbits is not None else None, eng.n, ptr.data_ptr(), rows.data_ptr(),
            w.data_ptr(), len(seed_sets), float(alpha), out.data_ptr(), _stream(self.dev)))
        return out

    def cold_residuals(self, seed_sets, alpha: float) -> np.ndarray:
        """||P(v) - v||_1 per column for the teleport vectors v (exact)."""
        r = self._cold_residuals_device(seed_sets, alpha).cpu().numpy()
        if (r < 0).any():
            raise ValueError("a seed is outside [0, n)")
        return r

    def _drain_gate(self) -> None:
        """Feed the gate the measurements of earlier starts whose work has
        finished (CUDA events on the launching stream; nothing waits)."""
        keep = []
        for ev, done, k, host in self._pending:
            if not done.query():
                keep.append((ev, done, k, host))
                continue
            r = host.numpy()
            self.gate.record(ev[0].elapsed_time(ev[1]) / 1e3, ev[1].elapsed_time(ev[2]) / 1e3, k, r[0], r[1])
        self._pending = keep

    def start_vectors(self, seed_sets, alpha):
        """(start columns, which columns use the window start) for
        ``PPREngine.solve`` and the server: one step from the window start,
        kept where its residual is not above the teleport vector's (that step
        then counts as the column's first iteration: ``pre_steps``).  Nothing
        here waits for the device once the per-alpha setup exists: the
        choice is a device mask, and the gate's timings are CUDA events read
        when they have completed."""
        eng = self.eng
        k = len(seed_sets)
        self.pre_steps = 0
        if self.gate is not None:
            self._drain_gate()
            if not self.gate.want_prediction():
                return eng.teleport_columns(seed_sets), np.zeros(k, dtype=bool)
        st = self._prepare(alpha)
        # the teleport index once, before any start kernel is queued (its
        # host-to-device copies would otherwise wait for them)
        tel = eng.teleport(seed_sets)
        ev = None
        if self.gate is not None:
            ev = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
            ev[0].record()
        tel, tp, V = self._teleport(seed_sets, tel)
        x0 = self._start_from(V, st, tp)
        if ev is not None:
            ev[1].record()
        if not self.fallback:
            return x0, np.ones(k, dtype=bool)
        run = PprRun(eng.meta, eng.n, eng.n, eng.block_size, eng.block_size, tp, alpha, 1, 0.0,
                     native.GL_PPR_STOP_ALL, eng.dbits)
        run.init(x0, adopt=True)
        del x0
        run.launch_chunk(1)
        if ev is not None:
            ev[2].record()
        r_warm = run.res_hist[0]
        r_cold = self._cold_residuals_device(seed_sets, alpha, tel)
        use = r_warm <= r_cold
        self.pre_steps = 1
        X = run.bufs[1]
        torch.where(use[None, :], X, V, out=X)      # the teleport vector where the start lost
        if ev is not None:
            host = torch.empty((2, k), dtype=torch.float64, pin_memory=True)
            host[0].copy_(r_warm, non_blocking=True)
            host[1].copy_(r_cold, non_blocking=True)
            done = torch.cuda.Event()
            done.record()
            self._pending.append((ev, done, k, host))
        return X, use

    def solve(self, seed_sets, alpha: float = 0.85, tol: float = 1e-6, max_iterations: int = 1000, **kw):
        """Batched solve from the window start (per-column cold fallback)."""
        return self.eng.solve(seed_sets, alpha=alpha, tol=tol, max_iterations=max_iterations, warm_start=self,
                              **kw)
