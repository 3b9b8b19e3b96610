"""Learned warm start for batched PPR.

A 2-layer MLP (10 inputs -> 128 ReLU -> 1; BF16 weight matrices, FP32
accumulation; trained and run by this library's own kernels
``gl_mlp_forward / gl_mlp_backward / gl_mlp_adam``) predicts log-PPR of every
(node, query) pair from per-node features:

  log(1 + in-degree), log(1 + out-degree),
  one-hot hop distance to the nearest seed (0, 1, 2, 3, 4, farther),
  log of the 1-step and 2-step propagated seed mass (A v, A^2 v).

The features come from the fused SpMM (``gl_pbr_spmm``) applied to the seed
vectors and to reachability indicators.  The prediction, exponentiated and
normalized per column, starts the power iteration; the iteration then runs
to the same tolerance, so the fixed point and its accuracy do not depend on
the network.  A column whose first-step residual from the predicted start is
larger than from the cold start (the teleport vector) falls back to the cold
start.

:class:`WarmStartGate` decides per batch whether predicting is worth it: each
prediction measures its own cost (seconds per column) and, from the two
first-step residuals, the iterations it saves (the error shrinks about
geometrically, so a start whose residual is r_warm instead of r_cold saves
log(r_cold / r_warm) / log(1 / rate) iterations); a fused step of the same
batch gives the cost of one iteration per column.  Later batches predict
only while the estimated saving exceeds the cost, with a probe every
``probe_every`` batches to follow changes.
"""
from __future__ import annotations

import math
import time
from dataclasses import dataclass, field

import numpy as np
import torch

from . import native
from .engine import PPREngine
from .pbr import _ptr, matrix_desc, spmm_workspace
from .ppr import PprRun, teleport_from_seed_sets

F_IN = 10
HIDDEN = native.GL_MLP_HIDDEN
N_PARAMS = HIDDEN * F_IN + 2 * HIDDEN + 1
LOG_FLOOR = 1e-10


class MLP:
    """Parameters and optimizer state of the warm-start network (device)."""

    def __init__(self, device, seed: int = 0, f_in: int = F_IN, out_bias: float = math.log(1e-7)):
        if not 1 <= f_in <= native.GL_MLP_MAX_IN:
            raise ValueError(f"f_in must be in 1..{native.GL_MLP_MAX_IN}")
        self.f_in = f_in = int(f_in)
        n_params = HIDDEN * f_in + 2 * HIDDEN + 1
        g = torch.Generator().manual_seed(seed)
        p = torch.zeros(n_params, dtype=torch.float32)
        bound1 = 1.0 / math.sqrt(f_in)
        p[: HIDDEN * f_in] = (torch.rand(HIDDEN * f_in, generator=g) * 2 - 1) * bound1
        p[HIDDEN * f_in: HIDDEN * f_in + HIDDEN] = 0.01
        bound2 = 1.0 / math.sqrt(HIDDEN)
        p[HIDDEN * f_in + HIDDEN: HIDDEN * f_in + 2 * HIDDEN] = (torch.rand(HIDDEN, generator=g) * 2 - 1) * bound2
        p[-1] = out_bias
        self.device = device
        self.params = p.to(device)
        self.m = torch.zeros_like(self.params)
        self.v = torch.zeros_like(self.params)
        self.grad = torch.zeros_like(self.params)
        self.W1 = torch.zeros(HIDDEN * f_in, dtype=torch.int16, device=device)
        self.w2 = torch.zeros(HIDDEN, dtype=torch.int16, device=device)
        self.loss = torch.zeros(1, dtype=torch.float64, device=device)
        self.step = 0
        self._refresh_bf16()

    def _refresh_bf16(self):
        # round-to-nearest-even BF16 copies of the FP32 master weights
        def to_bf16_bits(t):
            u = t.contiguous().view(torch.int32).to(torch.int64) & 0xFFFFFFFF
            lsb = (u >> 16) & 1
            r = (u + 0x7FFF + lsb) >> 16
            return (r & 0xFFFF).to(torch.int32).to(torch.int16)
        f = self.f_in
        self.W1.copy_(to_bf16_bits(self.params[: HIDDEN * f]))
        self.w2.copy_(to_bf16_bits(self.params[HIDDEN * f + HIDDEN: HIDDEN * f + 2 * HIDDEN]))

    @property
    def b1(self) -> torch.Tensor:
        return self.params[HIDDEN * self.f_in: HIDDEN * self.f_in + HIDDEN]

    def b2(self) -> float:
        return float(self.params[-1].item())

    def forward(self, X: torch.Tensor, b2: float | None = None) -> torch.Tensor:
        X = X.contiguous()
        out = torch.empty(X.shape[0], dtype=torch.float32, device=self.device)
        native.check(native.lib().gl_mlp_forward(
            _ptr(X), X.shape[0], self.f_in, self.W1.data_ptr(), self.b1.data_ptr(), self.w2.data_ptr(),
            self.b2() if b2 is None else b2, _ptr(out), torch.cuda.current_stream(self.device).cuda_stream))
        return out

    def gradient(self, X: torch.Tensor, target: torch.Tensor) -> tuple[torch.Tensor, float]:
        self.grad.zero_()
        self.loss.zero_()
        native.check(native.lib().gl_mlp_backward(
            _ptr(X.contiguous()), _ptr(target.contiguous()), X.shape[0], self.f_in, self.W1.data_ptr(),
            self.b1.data_ptr(), self.w2.data_ptr(), self.b2(), self.grad.data_ptr(), self.loss.data_ptr(),
            torch.cuda.current_stream(self.device).cuda_stream))
        return self.grad, float(self.loss.item())

    def adam_step(self, n_examples: int, lr: float = 2e-3):
        self.step += 1
        native.check(native.lib().gl_mlp_adam(
            self.params.data_ptr(), self.grad.data_ptr(), self.m.data_ptr(), self.v.data_ptr(),
            self.params.numel(), lr, 0.9, 0.999, 1e-8, 1.0 / max(1, n_examples), self.step, self.W1.data_ptr(),
            self.w2.data_ptr(), self.f_in, torch.cuda.current_stream(self.device).cuda_stream))


@dataclass
class TrainStats:
    vectors: int
    examples: int
    seconds: float
    losses: list = field(default_factory=list)


class WarmStartGate:
    """Cost / benefit record of the warm start's predictions (see the module
    docstring).  Exponential moving averages; ``rate`` is the assumed
    per-iteration contraction of the error (the damping factor bounds it)."""

    def __init__(self, probe_every: int = 16, rate: float = 0.85, smoothing: float = 0.5):
        self.probe_every = int(probe_every)
        self.rate = float(rate)
        self.smoothing = float(smoothing)
        self.pred_s_per_col: float | None = None     # prediction seconds per column
        self.saved_iters: float | None = None        # estimated iterations saved per column
        self.iter_s_per_col: float | None = None     # seconds of one iteration per column
        self.calls = 0
        self.predictions = 0

    def _ema(self, old, new):
        return new if old is None else self.smoothing * old + (1.0 - self.smoothing) * new

    def want_prediction(self) -> bool:
        self.calls += 1
        if None in (self.pred_s_per_col, self.saved_iters, self.iter_s_per_col):
            return True
        if self.probe_every > 0 and self.calls % self.probe_every == 0:
            return True
        return self.saved_iters * self.iter_s_per_col > self.pred_s_per_col

    def record(self, pred_seconds: float, step_seconds: float, columns: int, r_warm: np.ndarray,
               r_cold: np.ndarray) -> None:
        k = max(1, int(columns))
        ratio = np.maximum(np.asarray(r_cold, np.float64), 1e-300) / np.maximum(np.asarray(r_warm, np.float64),
                                                                               1e-300)
        saved = np.where(ratio > 1.0, np.log(ratio) / math.log(1.0 / self.rate), 0.0)
        self.pred_s_per_col = self._ema(self.pred_s_per_col, pred_seconds / k)
        self.iter_s_per_col = self._ema(self.iter_s_per_col, step_seconds / k)
        self.saved_iters = self._ema(self.saved_iters, float(saved.mean()))
        self.predictions += 1

    def summary(self) -> dict:
        return {"predictions": self.predictions, "batches": self.calls,
                "prediction_s_per_column": self.pred_s_per_col, "saved_iterations_per_column": self.saved_iters,
                "iteration_s_per_column": self.iter_s_per_col}


class WarmStart:
    """Feature extraction, training and warm-started solves for one engine."""

    def __init__(self, engine: PPREngine, seed: int = 0, gate: WarmStartGate | None = None):
        self.eng = engine
        self.gate = gate
        self.dev = engine.device
        self.mlp = MLP(self.dev, seed)
        n = engine.n
        A_rows = torch.as_tensor(np.diff(engine.host_indptr), device=self.dev, dtype=torch.float32)
        out_deg = torch.bincount(torch.as_tensor(engine.host_indices, device=self.dev, dtype=torch.int64),
                                 minlength=n).to(torch.float32)
        self.log_in = torch.log1p(A_rows)
        self.log_out = torch.log1p(out_deg)
        self._desc = matrix_desc(engine.meta, n, n, engine.block_size, engine.block_size)

    # -- features -------------------------------------------------------------
    def _spmm(self, X: torch.Tensor) -> torch.Tensor:
        K = X.shape[1]
        Y = torch.empty_like(X)
        ws = spmm_workspace(self.eng.meta, self._desc, 1, K, self.dev)
        native.check(native.lib().gl_pbr_spmm(self._desc, X.data_ptr(), Y.data_ptr(), 1, K,
                                              ws.data_ptr() if ws is not None else None,
                                              ws.numel() if ws is not None else 0,
                                              torch.cuda.current_stream(self.dev).cuda_stream))
        return Y

    def seed_matrix(self, seed_sets) -> torch.Tensor:
        return self.eng.teleport_columns(seed_sets)

    def raw_features(self, V: torch.Tensor):
        """(m1, m2, hop) for the columns of V; hop in 0..5 (5 = farther than 4)."""
        m1 = self._spmm(V)
        m2 = self._spmm(m1)
        reach = V > 0
        hop = torch.full(V.shape, 5, dtype=torch.uint8, device=self.dev)
        hop[reach] = 0
        r1 = (m1 > 0) & ~reach
        hop[r1] = 1
        reach |= r1
        r2 = (m2 > 0) & ~reach
        hop[r2] = 2
        reach |= r2
        frontier = reach.to(torch.float32)
        for h in (3, 4):
            nxt = (self._spmm(frontier) > 0) & ~reach
            hop[nxt] = h
            reach |= nxt
            frontier = reach.to(torch.float32)
        return m1, m2, hop

    def assemble(self, rows: torch.Tensor, m1: torch.Tensor, m2: torch.Tensor, hop: torch.Tensor) -> torch.Tensor:
        """Feature rows for nodes `rows` (1-D) of one column's m1/m2/hop (1-D)."""
        f = torch.empty((rows.numel(), F_IN), dtype=torch.float32, device=self.dev)
        f[:, 0] = self.log_in[rows]
        f[:, 1] = self.log_out[rows]
        oh = torch.nn.functional.one_hot(hop.long(), 6).to(torch.float32)
        f[:, 2:8] = oh
        f[:, 8] = torch.log(m1 + LOG_FLOOR) / 10.0
        f[:, 9] = torch.log(m2 + LOG_FLOOR) / 10.0
        return f

    # -- training ---------------------------------------------------------------
    def train(self, num_vectors: int = 20000, batch: int = 256, nodes_per_vector: int = 512,
              alpha: float = 0.85, tol: float = 1e-6, lr: float = 3e-3, minibatch: int = 8192,
              epochs: int = 6, seed: int = 100) -> TrainStats:
        """Solve num_vectors seed sets (sizes 1-32) with the plain method (the
        engine without warm start) and fit the network to their log-PPR on
        sampled nodes (most by PPR mass, some uniform)."""
        from . import synth
        t0 = time.perf_counter()
        gen = torch.Generator(device=self.dev).manual_seed(seed)
        feats, targs = [], []
        done = 0
        while done < num_vectors:
            k = min(batch, num_vectors - done)
            sets = synth.seed_sets(self.eng.n, k, 1, 32, seed=seed + done)
            res = self.eng.solve(sets, alpha=alpha, tol=tol)
            V = self.seed_matrix(sets)
            m1, m2, hop = self.raw_features(V)
            X = res.X.clamp_min(0)
            n_mass = nodes_per_vector * 3 // 4
            n_uni = nodes_per_vector - n_mass
            idx_mass = torch.multinomial(X.T + 1e-30, n_mass, replacement=True, generator=gen)   # [k, n_mass]
            idx_uni = torch.randint(0, self.eng.n, (k, n_uni), device=self.dev, generator=gen)
            idx = torch.cat([idx_mass, idx_uni], dim=1)                                          # [k, S]
            cols = torch.arange(k, device=self.dev)[:, None].expand_as(idx)
            rows = idx.reshape(-1)
            cc = cols.reshape(-1)
            f = self.assemble(rows, m1[rows, cc], m2[rows, cc], hop[rows, cc])
            feats.append(f)
            targs.append(torch.log(X[rows, cc] + LOG_FLOOR))
            done += k
        Xf = torch.cat(feats)
        T = torch.cat(targs)
        n = Xf.shape[0]
        losses = []
        steps_total = epochs * ((n + minibatch - 1) // minibatch)
        step = 0
        for _ in range(epochs):
            perm = torch.randperm(n, device=self.dev, generator=gen)
            for s0 in range(0, n, minibatch):
                sel = perm[s0:s0 + minibatch]
                _, loss = self.mlp.gradient(Xf[sel], T[sel])
                # cosine decay from lr to lr / 10
                cur = lr * (0.1 + 0.9 * 0.5 * (1.0 + math.cos(math.pi * step / max(1, steps_total))))
                self.mlp.adam_step(sel.numel(), cur)
                losses.append(loss / sel.numel())
                step += 1
        torch.cuda.synchronize(self.dev)
        return TrainStats(vectors=num_vectors, examples=n, seconds=time.perf_counter() - t0, losses=losses)

    # -- inference ----------------------------------------------------------------
    def predict(self, seed_sets, chunk: int = 32) -> torch.Tensor:
        """Predicted start vectors [n, K] (each column sums to 1)."""
        n = self.eng.n
        out = torch.empty((n, len(seed_sets)), dtype=torch.float32, device=self.dev)
        all_rows = torch.arange(n, device=self.dev)
        for c0 in range(0, len(seed_sets), chunk):
            sets = seed_sets[c0:c0 + chunk]
            V = self.seed_matrix(sets)
            m1, m2, hop = self.raw_features(V)
            for k in range(len(sets)):
                f = self.assemble(all_rows, m1[:, k], m2[:, k], hop[:, k])
                y = self.mlp.forward(f)
                x = torch.exp(y - y.max())
                out[:, c0 + k] = x / x.sum()
        return out

    def start_vectors(self, seed_sets, alpha) -> tuple[torch.Tensor, np.ndarray]:
        """Start columns: the prediction where its first residual is below the
        cold start's, else the teleport vector; and which columns use it.
        With a gate that finds the prediction not worth its cost, every
        column starts cold and nothing is predicted."""
        if self.gate is not None and not self.gate.want_prediction():
            return self.seed_matrix(seed_sets), np.zeros(len(seed_sets), dtype=bool)
        timed = self.gate is not None
        if timed:
            torch.cuda.synchronize(self.dev)
        t0 = time.perf_counter()
        x_warm = self.predict(seed_sets)
        if timed:
            torch.cuda.synchronize(self.dev)
        t1 = time.perf_counter()
        V = self.seed_matrix(seed_sets)
        r_warm = self.first_residual(seed_sets, x_warm, alpha)
        if timed:
            r_cold, step_s = self.first_residual(seed_sets, V, alpha, timing=True)
            self.gate.record(t1 - t0, step_s, len(seed_sets), r_warm, r_cold)
        else:
            r_cold = self.first_residual(seed_sets, V, alpha)
        use_warm = r_warm < r_cold
        return torch.where(torch.from_numpy(use_warm).to(self.dev)[None, :], x_warm, V), use_warm

    def solve(self, seed_sets, alpha: float = 0.85, tol: float = 1e-6, max_iterations: int = 1000, **kw):
        """Warm-started batched solve with per-column fallback to the cold start."""
        return self.eng.solve(seed_sets, alpha=alpha, tol=tol, max_iterations=max_iterations, warm_start=self, **kw)

    def first_residual(self, seed_sets, x0: torch.Tensor, alpha: float, timing: bool = False):
        """||P(x0) - x0||_1 per column (one fused step); with ``timing`` also
        the seconds of one fused step over these columns (CUDA events)."""
        ptr, rows, w = self.eng.teleport(seed_sets)
        tp = teleport_from_seed_sets(ptr, rows, self.eng.n, self.eng.block_size, w)
        run = PprRun(self.eng.meta, self.eng.n, self.eng.n, self.eng.block_size, self.eng.block_size, tp,
                     alpha, 2, 0.0, native.GL_PPR_STOP_ALL, self.eng.dbits)
        run.init(x0)
        if not timing:
            run.launch_chunk(2)
            return run.res_hist[0].cpu().numpy()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        run.launch_chunk(2)
        e1.record()
        res = run.res_hist[0].cpu().numpy()
        return res, e0.elapsed_time(e1) / 2e3


FAR_F_IN = 6


class FarFieldModel:
    """Learned far-field shape for the window-solve start
    (``window_start.WindowStart(shape="learned")``).

    The window start computes a query's near field exactly and must place
    the mass it misses (the walks that leave their window more often than the
    start follows them) somewhere.  This network predicts, per node, the log
    of the ratio between that far field and the uniform teleport vector's
    far field (the ``expected`` shape), from a per-graph basis of vectors
    computed once (PageRank, the near field of the uniform teleport vector
    and that vector's far field) and node features:

      log(n PageRank_i), log(n near_i), log(n far_i), log(1 + in-degree),
      log(1 + out-degree), and the transition mass that leaves i's window.

    It is trained on far fields of PPR vectors the plain method computed
    (the batched engine without a warm start): for each training column the
    exact vector minus the window start's near field, normalized, averaged
    over the columns, with nodes sampled by mass (most) and uniformly.  For
    seed sets drawn uniformly at random that average tends to the uniform
    vector's far field (PPR is linear in the teleport vector), so the basis
    vector ``far`` is already close to the target; the network learns the
    per-node correction between the two.  Predicting the ratio rather than
    the density itself (with the last layer starting at zero) keeps an
    untrained or unsure network at the basis shape: reproducing the shape
    through BF16 weights put about 1 % errors into the far field and cost a
    certification step at 8 window exits."""

    def __init__(self, device, seed: int = 0):
        self.device = device
        self.mlp = MLP(device, seed, f_in=FAR_F_IN, out_bias=0.0)
        # last layer at zero: the untrained network is the basis shape itself
        h, f = HIDDEN, FAR_F_IN
        self.mlp.params[h * f + h: h * f + 2 * h] = 0.0
        self.mlp._refresh_bf16()
        self.stats: TrainStats | None = None
        self._shapes: dict = {}

    def features(self, ws, alpha: float) -> torch.Tensor:
        st = ws._prepare(alpha)
        eng = ws.eng
        n = eng.n
        dev = self.device
        indptr, indices, _ = eng.csr
        in_deg = (indptr[1:] - indptr[:-1]).to(torch.float32)
        out_deg = torch.bincount(indices.to(torch.int64), minlength=n).to(torch.float32)
        f = torch.empty((n, FAR_F_IN), dtype=torch.float32, device=dev)
        f[:, 0] = torch.log(n * ws.pagerank(alpha).clamp_min(0) + 1e-6) / 10.0
        f[:, 1] = torch.log(n * st["near_uniform"].clamp_min(0) + 1e-6) / 10.0
        f[:, 2] = torch.log(n * st["expected"].clamp_min(0) + 1e-6) / 10.0
        f[:, 3] = torch.log1p(in_deg)
        f[:, 4] = torch.log1p(out_deg)
        f[:, 5] = ws.off.leak
        return f

    def fit(self, ws, alpha: float, seed_sets, tol: float = 1e-6, epochs: int = 30, minibatch: int = 8192,
            lr: float = 3e-3, samples_per_epoch: int = 1 << 20, seed: int = 100, batch: int = 256) -> TrainStats:
        """Train on the far fields of ``seed_sets`` solved by the plain method
        (in slices of ``batch`` columns)."""
        t0 = time.perf_counter()
        eng = ws.eng
        n = eng.n
        acc = torch.zeros(n, dtype=torch.float64, device=self.device)
        for c0 in range(0, len(seed_sets), batch):
            sl = seed_sets[c0:c0 + batch]
            res = eng.solve(sl, alpha=alpha, tol=tol)
            near = ws.near_field(sl, alpha)
            far = (res.X - near).clamp_min(0)
            far = far / far.sum(dim=0, keepdim=True).clamp_min(1e-30)
            acc += far.sum(dim=1, dtype=torch.float64)
            del far, near, res
        target_mass = (acc / max(1, len(seed_sets))).to(torch.float32)   # [n], sums to 1
        base = ws._prepare(alpha)["expected"]
        T = torch.log(n * target_mass + 1e-6) - torch.log(n * base.clamp_min(0) + 1e-6)
        F = self.features(ws, alpha)
        gen = torch.Generator(device=self.device).manual_seed(seed)
        losses = []
        steps_total = epochs * ((samples_per_epoch + minibatch - 1) // minibatch)
        step = 0
        for _ in range(epochs):
            n_mass = samples_per_epoch * 3 // 4
            idx = torch.cat([torch.multinomial(target_mass + 1e-12, n_mass, replacement=True, generator=gen),
                             torch.randint(0, n, (samples_per_epoch - n_mass,), device=self.device,
                                           generator=gen)])
            idx = idx[torch.randperm(idx.numel(), device=self.device, generator=gen)]
            for s0 in range(0, idx.numel(), minibatch):
                sel = idx[s0:s0 + minibatch]
                _, loss = self.mlp.gradient(F[sel], T[sel])
                cur = lr * (0.1 + 0.9 * 0.5 * (1.0 + math.cos(math.pi * step / max(1, steps_total))))
                self.mlp.adam_step(sel.numel(), cur)
                losses.append(loss / sel.numel())
                step += 1
        torch.cuda.synchronize(self.device)
        self._shapes.clear()
        self.stats = TrainStats(vectors=len(seed_sets), examples=epochs * samples_per_epoch,
                                seconds=time.perf_counter() - t0, losses=losses)
        return self.stats

    def shape(self, ws, alpha: float) -> torch.Tensor:
        """Predicted far-field density [n] (sums to 1) for this graph and alpha."""
        key = (id(ws), round(float(alpha), 12))
        if key not in self._shapes:
            y = self.mlp.forward(self.features(ws, alpha))
            base = ws._prepare(alpha)["expected"].clamp_min(0)
            x = base * torch.exp(y - y.max())
            tot = x.sum()
            self._shapes[key] = (x / tot).contiguous() if bool(tot > 0) else base
        return self._shapes[key]
