"""Learned Newton warm start for Monte Carlo DC sweeps.

A BF16 MLP maps a sample's sweep parameters to its DC operating point.  It is
trained on solutions produced by the plain FP64 GPU path (sweep indices
0..N-1 of a training seed, 7 in the benchmark workload), and at sweep time
its prediction is the Newton initial guess.  Plain Newton from the circuit's
nodeset, then gmin and source stepping, is the fallback whenever the guess
misses convergence (sp_newton_dc_learned_device).

Inputs are a subset of the random parameters chosen by greedy forward
selection (largest explained variance of the standardised solution under a
linear model); inputs and outputs are standardised with the draw
distributions and the training-set moments respectively.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field
from typing import List, Optional

import numpy as np

from . import _abi as abi
from .api import Context, Mlp, Topology, newton_dc_learned_device
from .circuit import Circuit


def param_normalization(circuit: Circuit, slot: int):
    """(mean, scale) of parameter slot `slot` under its draw distribution."""
    kind, _idx, a, b = circuit.params[slot]
    if kind == abi.SP_DRAW_GAUSS:
        return a, (b if b > 0 else 1.0)
    if kind in (abi.SP_DRAW_UNIFORM, abi.SP_DRAW_LOGUNIFORM):
        return 0.5 * (a + b), max(abs(b - a) / math.sqrt(12.0), 1e-300)
    if kind == abi.SP_DRAW_FIXED:
        return a, 1.0
    return 0.0, 1.0


def random_slots(circuit: Circuit) -> List[int]:
    return [k for k, row in enumerate(circuit.params)
            if row[0] in (abi.SP_DRAW_GAUSS, abi.SP_DRAW_UNIFORM, abi.SP_DRAW_LOGUNIFORM)]


def newton_tolerance(circuit: Circuit, X: np.ndarray, reltol=1e-3, vntol=1e-6, abstol=1e-12) -> np.ndarray:
    """Per-unknown convergence tolerance of check_convergence
    (crates/spicier-solver/src/newton.rs:134-159) at the typical solution."""
    absx = np.abs(X).mean(0)
    tol = reltol * absx
    tol[:circuit.num_nodes] += vntol
    tol[circuit.num_nodes:] += abstol
    return tol


def select_inputs(P: np.ndarray, X: np.ndarray, candidates: List[int], k: int,
                  tol: Optional[np.ndarray] = None) -> List[int]:
    """Greedy forward selection of k parameter columns of P maximising the
    variance of the solution X explained by a linear model, with each unknown
    measured in units of its Newton tolerance `tol` (standard deviations
    when tol is None)."""
    Xs = (X - X.mean(0)) / (tol if tol is not None else np.maximum(X.std(0), 1e-300))
    Ps = (P - P.mean(0)) / np.maximum(P.std(0), 1e-300)
    chosen: List[int] = []
    for _ in range(min(k, len(candidates))):
        best, best_r = None, -1.0
        for c in candidates:
            if c in chosen:
                continue
            A = np.column_stack([Ps[:, chosen + [c]], np.ones(len(Ps))])
            coef, *_ = np.linalg.lstsq(A, Xs, rcond=None)
            r = 1.0 - ((Xs - A @ coef) ** 2).sum() / max((Xs ** 2).sum(), 1e-300)
            if r > best_r:
                best, best_r = c, r
        chosen.append(best)
    return chosen


@dataclass
class TrainReport:
    samples: int
    converged: int
    inputs: List[int]
    input_labels: List[str]
    epoch_loss: List[float] = field(default_factory=list)
    seconds: float = 0.0


class WarmStart:
    """The trained network plus its wiring to one circuit."""

    def __init__(self, ctx: Context, circuit: Circuit, n_inputs: int = 10, n_hidden: int = 128, n_layers: int = 3,
                 seed: int = 0):
        self.ctx, self.circuit = ctx, circuit
        self.n_inputs = n_inputs
        self.mlp = Mlp(ctx, n_inputs, circuit.n, n_hidden, n_layers, seed)
        self.inputs: List[int] = []
        self.report: Optional[TrainReport] = None

    def train(self, topo: Topology, seed: int = 7, samples: int = 1 << 20, epochs: int = 16, batch: int = 4096,
              lr: float = 2e-3, select_rows: int = 16384) -> TrainReport:
        """Generate `samples` plain-FP64 solutions with `seed` and fit the network."""
        import time

        import torch
        t0 = time.perf_counter()
        c = self.circuit
        n, npar = c.n, len(c.params)
        dev = torch.device("cuda", self.ctx.device)
        x = torch.empty((samples, n), dtype=torch.float64, device=dev)
        st = torch.empty(samples, dtype=torch.uint8, device=dev)
        res = torch.empty(samples, dtype=torch.float64, device=dev)
        P = torch.empty((samples, npar), dtype=torch.float64, device=dev)
        cfg = abi.newton_config(precision=abi.SP_PREC_FP64)
        self.ctx.newton_dc_device(topo, cfg, seed, samples, x, status=st, resid=res, params=P)
        ok = (st & 0x0F) == 0
        x, P = x[ok], P[ok]
        rows = (x.shape[0] // batch) * batch
        x, P = x[:rows], P[:rows]
        cand = random_slots(c)
        sub = slice(0, min(select_rows, rows))
        xs = x[sub].cpu().numpy()
        tol = newton_tolerance(c, xs)
        if self.n_inputs >= len(cand):
            self.inputs = list(cand)
        else:
            # ascending slots: the specialised kernel then takes the linear term
            # as a launch parameter (the evaluation order is the slots' order)
            self.inputs = sorted(select_inputs(P[sub].cpu().numpy(), xs, cand, self.n_inputs, tol))
        in_mean = np.array([param_normalization(c, s)[0] for s in self.inputs])
        in_scale = np.array([param_normalization(c, s)[1] for s in self.inputs])
        self.tolerance = tol
        # FP64 linear term: least squares of x on the centred inputs (normal
        # equations, all on the device); the network learns the remainder
        Pc = P[:, self.inputs] - torch.tensor(in_mean, device=dev)
        A = torch.cat([Pc / torch.tensor(in_scale, device=dev), torch.ones((rows, 1), dtype=torch.float64,
                                                                             device=dev)], 1)
        # Gram matrices on the device, the (n_in+1)^2 solve on the host
        coef = torch.tensor(np.linalg.solve((A.T @ A).cpu().numpy(), (A.T @ x).cpu().numpy()),
                            device=dev)  # [n_in + 1][n]
        lin = (coef[:-1] / torch.tensor(in_scale, device=dev)[:, None]).T.contiguous()  # [n][n_in], raw units
        resid_t = x - coef[-1] - Pc @ lin.T
        out_mean = (coef[-1] + resid_t.mean(0)).cpu().numpy()
        out_std = resid_t.std(0).cpu().numpy()
        # unknowns the linear term explains exactly (supply rails) get scale 0
        out_scale = np.where(out_std > 1e-9 * np.maximum(np.abs(out_mean), 1e-30) + 1e-300, out_std, 0.0)
        safe = torch.tensor(np.where(out_scale > 0, out_scale, 1.0), device=dev)
        Xin = (Pc / torch.tensor(in_scale, device=dev)).to(torch.float32).contiguous()
        T = ((x - torch.tensor(out_mean, device=dev) - Pc @ lin.T) / safe).to(torch.float32).contiguous()
        self._lin = lin.cpu().numpy()
        self.mlp.set_linear(self._lin)
        loss = torch.zeros(epochs, dtype=torch.float32, device=dev)
        stream = torch.cuda.current_stream().cuda_stream
        self.mlp.train_device(Xin, T, rows, batch, epochs, lr, loss, stream=stream)
        torch.cuda.synchronize()
        self.mlp.set_io(self.inputs, in_mean, in_scale, out_mean, out_scale)
        self._io = (out_mean, out_scale)
        self._in = (in_mean, in_scale)
        per_epoch = rows // batch
        self.report = TrainReport(samples, int(ok.sum().item()), list(self.inputs),
                                  [c.param_labels[s] for s in self.inputs],
                                  [float(v) / per_epoch for v in loss.cpu().numpy()],
                                  time.perf_counter() - t0)
        return self.report

    def prediction_error(self, topo: Topology, seed: int, count: int) -> np.ndarray:
        """RMS error of the network's prediction per MNA unknown, in units of
        that unknown's Newton tolerance, over `count` samples of `seed`."""
        import torch
        c = self.circuit
        dev = torch.device("cuda", self.ctx.device)
        x = torch.empty((count, c.n), dtype=torch.float64, device=dev)
        st = torch.empty(count, dtype=torch.uint8, device=dev)
        P = torch.empty((count, len(c.params)), dtype=torch.float64, device=dev)
        self.ctx.newton_dc_device(topo, abi.newton_config(precision=abi.SP_PREC_FP64), seed, count, x, status=st,
                                  params=P)
        in_mean = torch.tensor([param_normalization(c, s)[0] for s in self.inputs], device=dev)
        in_scale = torch.tensor([param_normalization(c, s)[1] for s in self.inputs], device=dev)
        Xin = ((P[:, self.inputs] - in_mean) / in_scale).to(torch.float32).contiguous()
        y = torch.empty((count, c.n), dtype=torch.float32, device=dev)
        self.mlp.forward_device(Xin, count, y)
        torch.cuda.synchronize()
        io = self._io
        Pc = (P[:, self.inputs] - in_mean.double()).cpu().numpy()
        pred = io[0] + io[1] * y.double().cpu().numpy() + Pc @ self._lin.T
        err = pred - x.cpu().numpy()
        return np.sqrt((err ** 2).mean(0)) / self.tolerance

    def use_network(self, on: bool = True):
        """With on=False the warm start is the fitted linear term alone,
        out_mean + lin (p - in_mean) in FP32, evaluated by the sweep's draw
        kernel (SP_MLP_KERNEL_LINEAR: no inference kernel runs); on=True
        restores the network (the tcgen05 kernel where the shape allows).
        Comparing the two isolates what the trained network adds over the
        linear fit, and what it costs."""
        self.mlp.set_inference_kernel(abi.SP_MLP_KERNEL_AUTO if on else abi.SP_MLP_KERNEL_LINEAR)

    WARM_MAX_ITERATIONS = 8  # a miss restarts cold after this many iterations

    def sweep_device(self, topo: Topology, cfg, seed: int, count: int, x, first: int = 0, iters=None, status=None,
                     resid=None, moments=None, stream: int = 0):
        if cfg.warm_max_iterations == 0:
            cfg = abi.SpNewtonConfig.from_buffer_copy(cfg)
            cfg.warm_max_iterations = self.WARM_MAX_ITERATIONS
        newton_dc_learned_device(self.ctx, topo, self.mlp, cfg, seed, count, x, first=first, iters=iters,
                                 status=status, resid=resid, moments=moments, stream=stream)
