"""Host-side mirror of Spicier's batched-sweep interface over the C ABI.

Names, argument meanings and error behaviour follow the reference:
  BatchedLuSolver / BatchedSolveResult / GpuBatchConfig / BackendType
      crates/spicier-batched-sweep/src/solver.rs:15-135
  BatchedSweepError -> SpicierError (kind = variant name)
      crates/spicier-batched-sweep/src/error.rs:7-43
  ParameterVariation, SweepPoint, Monte Carlo / corner / linear generators
      crates/spicier-solver/src/sweep.rs:15-266
  solve_batched_sweep_gpu, GpuBatchedSweepResult
      crates/spicier-batched-sweep/src/sweep.rs:15-217
  ConvergenceCriteria + stepping parameters -> _abi.newton_config()
      crates/spicier-solver/src/newton.rs:9-34, 173-231
The Newton sweep (solve_newton_sweep_gpu) has no counterpart in the
reference's sweep API, which is linear-only; it batches solve_newton_raphson
(crates/spicier-solver/src/newton.rs:70-131) per sweep point.
"""
from __future__ import annotations

import ctypes as C
import enum
import math
from dataclasses import dataclass, field
from typing import List, Optional, Sequence

import numpy as np

from . import _abi as abi
from ._lib import SpicierError, check, load
from .circuit import Circuit

MAX_BATCH_SIZE = 65535  # the reference's cuBLAS cap (solver.rs:5); not a limit here
MIN_BATCH_SIZE = 16
MIN_MATRIX_SIZE = 32


def _vp(a) -> Optional[int]:
    if a is None:
        return None
    if isinstance(a, np.ndarray):
        return a.ctypes.data
    return int(a.data_ptr())  # torch tensor


class BackendType(enum.IntEnum):
    Cuda = abi.SP_BACKEND_CUDA
    Metal = abi.SP_BACKEND_METAL
    Mps = abi.SP_BACKEND_MPS
    Accelerate = abi.SP_BACKEND_ACCELERATE
    Faer = abi.SP_BACKEND_FAER
    Cpu = abi.SP_BACKEND_CPU
    Gb300 = abi.SP_BACKEND_GB300


@dataclass
class GpuBatchConfig:
    min_batch_size: int = MIN_BATCH_SIZE
    min_matrix_size: int = 1
    max_batch_per_launch: int = 1 << 26

    def should_use_gpu(self, matrix_size: int, batch_size: int) -> bool:
        return matrix_size >= self.min_matrix_size and batch_size >= self.min_batch_size


@dataclass
class BatchedSolveResult:
    solutions: np.ndarray
    singular_indices: List[int]
    n: int
    batch_size: int

    def solution(self, index: int):
        if index >= self.batch_size:
            return None
        return self.solutions[index * self.n:(index + 1) * self.n]

    def is_singular(self, index: int) -> bool:
        return index in self.singular_indices

    def num_solved(self) -> int:
        return self.batch_size - len(self.singular_indices)


@dataclass
class NewtonResult:
    """Per-sample outputs of a batched DC operating-point sweep."""
    x: np.ndarray
    iters: np.ndarray
    status: np.ndarray
    resid: Optional[np.ndarray] = None
    params: Optional[np.ndarray] = None
    moments: Optional[list] = None

    @property
    def converged(self) -> np.ndarray:
        return (self.status & abi.SP_ST_MASK) == abi.SP_ST_CONVERGED

    @property
    def converged_count(self) -> int:
        return int(self.converged.sum())


class Topology:
    """A circuit uploaded to the device (sp_topology)."""

    def __init__(self, ctx: "Context", circuit: Circuit):
        self.ctx = ctx
        self.circuit = circuit
        self._ptr = C.c_void_p()
        cc = circuit.to_c()
        check(ctx._ptr, load().sp_topology_create(ctx._ptr, C.byref(cc), C.byref(self._ptr)))
        self.n = load().sp_topology_size(self._ptr)

    def close(self):
        if self._ptr:
            load().sp_topology_destroy(self._ptr)
            self._ptr = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Context:
    """One device context (sp_ctx)."""

    def __init__(self, device: int = 0):
        L = load()
        self._ptr = C.c_void_p()
        rc = L.sp_ctx_create(device, C.byref(self._ptr))
        if rc != 0:
            raise SpicierError(rc, f"cannot open CUDA device {device}")
        self.device = device

    def close(self):
        if self._ptr:
            load().sp_ctx_destroy(self._ptr)
            self._ptr = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @staticmethod
    def version() -> str:
        return load().sp_version().decode()

    # -- BatchedLuSolver ---------------------------------------------------
    def config(self) -> GpuBatchConfig:
        c = abi.SpBatchConfig()
        check(self._ptr, load().sp_get_config(self._ptr, C.byref(c)))
        return GpuBatchConfig(c.min_batch_size, c.min_matrix_size, c.max_batch_per_launch)

    def set_config(self, cfg: GpuBatchConfig):
        c = abi.SpBatchConfig(cfg.min_batch_size, cfg.min_matrix_size, cfg.max_batch_per_launch)
        check(self._ptr, load().sp_set_config(self._ptr, C.byref(c)))

    def solve_batch(self, matrices, rhs, n: int, batch_size: int) -> BatchedSolveResult:
        mats = np.ascontiguousarray(matrices, dtype=np.float64).ravel()
        b = np.ascontiguousarray(rhs, dtype=np.float64).ravel()
        if mats.size != batch_size * n * n:
            raise SpicierError(abi.SP_ERR_INVALID_DIMENSION,
                               f"Expected {batch_size * n * n} matrix elements, got {mats.size}")
        if b.size != batch_size * n:
            raise SpicierError(abi.SP_ERR_INVALID_DIMENSION, f"Expected {batch_size * n} RHS elements, got {b.size}")
        sol = np.zeros(batch_size * n)
        sing = np.zeros(max(batch_size, 1), np.uint64)
        ns = C.c_uint64(0)
        check(self._ptr, load().sp_solve_batch(self._ptr, _vp(mats), _vp(b), n, batch_size, _vp(sol), _vp(sing),
                                               C.byref(ns)))
        return BatchedSolveResult(sol, [int(i) for i in sing[:ns.value]], n, batch_size)

    def solve_batch_device(self, d_mats, d_rhs, n, batch, d_sol, d_sing, precision=abi.SP_PREC_FP64,
                           refine_steps=2, stream=0):
        check(self._ptr, load().sp_solve_batch_device(self._ptr, _vp(d_mats), _vp(d_rhs), n, batch, _vp(d_sol),
                                                      _vp(d_sing), precision, refine_steps, stream))

    # -- Newton sweeps -------------------------------------------------------
    def topology(self, circuit: Circuit) -> Topology:
        return Topology(self, circuit)

    def newton_dc(self, circuit: Circuit, cfg: abi.SpNewtonConfig, seed: int, count: int, first: int = 0,
                  table=None, x0=None, params: bool = False, resid: bool = True,
                  moments: bool = False) -> NewtonResult:
        """Host-buffer batched DC operating points (sp_newton_dc)."""
        n = circuit.n
        x = np.zeros((count, n))
        iters = np.zeros(count, np.int32)
        status = np.zeros(count, np.uint8)
        r = np.zeros(count) if resid else None
        p = np.zeros((count, max(len(circuit.params), 1))) if params else None
        m = (abi.SpMoments * n)() if moments else None
        cols = 0
        if table is not None:
            table = np.ascontiguousarray(table, dtype=np.float64)
            cols = table.shape[1]
        if x0 is not None:
            x0 = np.ascontiguousarray(x0, dtype=np.float64)
        cc = circuit.to_c()
        check(self._ptr, load().sp_newton_dc(self._ptr, C.byref(cc), C.byref(cfg), seed, first, count, _vp(table),
                                             cols, _vp(x0), _vp(x), _vp(iters), _vp(status), _vp(r), _vp(p),
                                             C.cast(m, C.c_void_p) if m is not None else None))
        mom = None
        if m is not None:
            mom = [dict(count=mm.count, sum=mm.sum, sum_sq=mm.sum_sq, min=mm.min, max=mm.max) for mm in m]
        return NewtonResult(x, iters, status, r, p[:, :len(circuit.params)] if p is not None else None, mom)

    def newton_dc_device(self, topo: Topology, cfg: abi.SpNewtonConfig, seed: int, count: int, x, first: int = 0,
                         table=None, x0=None, iters=None, status=None, resid=None, params=None, moments=None,
                         stream: int = 0):
        """Device-buffer batched DC operating points (sp_newton_dc_device);
        buffers are torch CUDA tensors (or raw device pointers via .data_ptr())."""
        cols = 0 if table is None else int(table.shape[1])
        check(self._ptr, load().sp_newton_dc_device(self._ptr, topo._ptr, C.byref(cfg), seed, first, count,
                                                    _vp(table), cols, _vp(x0), _vp(x), _vp(iters), _vp(status),
                                                    _vp(resid), _vp(params), _vp(moments), stream))

    def rng_fill_device(self, kind: int, seed: int, first: int, param: int, count: int, out, stream: int = 0):
        check(self._ptr, load().sp_rng_fill_device(self._ptr, kind, seed, first, param, count, _vp(out), stream))

    def specialize(self, topo: Topology, precision: int = abi.SP_PREC_MIXED, enable: bool = True) -> str:
        """Build (NVRTC) and enable / disable the topology-specialised kernel."""
        log = C.create_string_buffer(1 << 16)
        check(self._ptr, load().sp_topology_specialize(self._ptr, topo._ptr, precision, 1 if enable else 0, log,
                                                       len(log)))
        return log.value.decode(errors="replace")

    def profile_enable(self, on: bool = True):
        check(self._ptr, load().sp_profile_enable(self._ptr, 1 if on else 0))

    # -- ladder transients -----------------------------------------------------
    def ladder_transient(self, cfg, seed: int, count: int, first: int = 0) -> dict:
        """Host-buffer batched RC-diode ladder transients (sp_ladder_transient):
        dict of x (final state [count][max_sections+2]), n, accepted, rejected,
        iterations, status, probe [count][num_probe]."""
        ld = cfg.max_sections + 2
        out = dict(x=np.zeros((count, ld)), n=np.zeros(count, np.int32), accepted=np.zeros(count, np.int32),
                   rejected=np.zeros(count, np.int32), iterations=np.zeros(count, np.int32),
                   status=np.zeros(count, np.uint8), probe=np.zeros((count, max(cfg.num_probe, 1))))
        check(self._ptr, load().sp_ladder_transient(self._ptr, C.byref(cfg), seed, first, count, _vp(out["x"]),
                                                    _vp(out["n"]), _vp(out["accepted"]), _vp(out["rejected"]),
                                                    _vp(out["iterations"]), _vp(out["status"]),
                                                    _vp(out["probe"]) if cfg.num_probe else None))
        out["probe"] = out["probe"][:, :cfg.num_probe]
        return out

    def ladder_transient_device(self, cfg, seed, count, x, n, accepted, rejected, iterations, status, probe=None,
                                first: int = 0, stream: int = 0):
        """Device-buffer variant (torch CUDA tensors): x [count][max_sections+2] f64, n/accepted/rejected/
        iterations int32 [count], status uint8 [count], probe [count][num_probe] f64."""
        check(self._ptr, load().sp_ladder_transient_device(self._ptr, C.byref(cfg), seed, first, count, _vp(x), _vp(n),
                                                           _vp(accepted), _vp(rejected), _vp(iterations),
                                                           _vp(status), _vp(probe), stream))

    def ladder_transient_steps(self, cfg, seed: int, count: int, first: int = 0, max_steps: int = 4096) -> dict:
        """ladder_transient plus every instance's accepted step sizes
        (sp_ladder_transient_steps_device): adds steps [count][max_steps]
        (row i valid up to accepted[i]).  Runs on the device through torch
        buffers and copies the results back."""
        import torch
        dev = torch.device("cuda", self.device)
        ld = cfg.max_sections + 2
        t = dict(x=torch.zeros((count, ld), dtype=torch.float64, device=dev),
                 n=torch.zeros(count, dtype=torch.int32, device=dev),
                 accepted=torch.zeros(count, dtype=torch.int32, device=dev),
                 rejected=torch.zeros(count, dtype=torch.int32, device=dev),
                 iterations=torch.zeros(count, dtype=torch.int32, device=dev),
                 status=torch.zeros(count, dtype=torch.uint8, device=dev),
                 probe=torch.zeros((count, max(cfg.num_probe, 1)), dtype=torch.float64, device=dev),
                 steps=torch.zeros((count, max_steps), dtype=torch.float64, device=dev))
        stream = torch.cuda.current_stream(dev).cuda_stream
        check(self._ptr, load().sp_ladder_transient_steps_device(
            self._ptr, C.byref(cfg), seed, first, count, _vp(t["x"]), _vp(t["n"]), _vp(t["accepted"]),
            _vp(t["rejected"]), _vp(t["iterations"]), _vp(t["status"]), _vp(t["probe"]) if cfg.num_probe else None,
            _vp(t["steps"]), max_steps, stream))
        torch.cuda.synchronize(dev)
        out = {k: v.cpu().numpy() for k, v in t.items()}
        out["probe"] = out["probe"][:, :cfg.num_probe]
        return out

    # -- AC small-signal sweeps ------------------------------------------------
    @staticmethod
    def ac_frequencies(cfg: abi.SpAcConfig) -> np.ndarray:
        """The frequency grid of an AC sweep (generate_frequencies)."""
        n = load().sp_ac_frequencies(C.byref(cfg), None, 0)
        out = np.zeros(max(n, 1))
        load().sp_ac_frequencies(C.byref(cfg), _vp(out), n)
        return out[:n]

    def ac_sweep(self, circuit: Circuit, dc_cfg: abi.SpNewtonConfig, cfg: abi.SpAcConfig, seed: int, count: int,
                 first: int = 0, table=None):
        """Host-buffer batched AC sweep (sp_ac_sweep): (probe [count][nf][num_probe] complex, status [count])."""
        nf = len(self.ac_frequencies(cfg))
        out = np.zeros((count, nf, cfg.num_probe, 2))
        st = np.zeros(count, np.uint8)
        cols = 0
        if table is not None:
            table = np.ascontiguousarray(table, dtype=np.float64)
            cols = table.shape[1]
        cc = circuit.to_c()
        check(self._ptr, load().sp_ac_sweep(self._ptr, C.byref(cc), C.byref(dc_cfg), C.byref(cfg), seed, first, count,
                                            _vp(table), cols, _vp(out), _vp(st)))
        return out[..., 0] + 1j * out[..., 1], st

    def ac_sweep_device(self, topo: Topology, dc_cfg, cfg, seed, count, probe, status, first: int = 0, table=None,
                        stream: int = 0):
        """Device-buffer variant: probe [count][nf][num_probe][2] f64, status uint8 [count] (torch CUDA tensors)."""
        cols = 0 if table is None else int(table.shape[1])
        check(self._ptr, load().sp_ac_sweep_device(self._ptr, topo._ptr, C.byref(dc_cfg), C.byref(cfg), seed, first,
                                                   count, _vp(table), cols, _vp(probe), _vp(status), stream))

    # -- fixed-step linear transients -----------------------------------------
    def transient(self, circuit: Circuit, dc_cfg: abi.SpNewtonConfig, cfg: abi.SpTransientConfig, seed: int,
                  count: int, first: int = 0, table=None) -> dict:
        """Host-buffer batched fixed-step transients (sp_transient, solve_transient): dict of x (state at the
        last step, [count][nodes + V sources]), probe ([count][steps + 1] when cfg.probe >= 0), status."""
        nv = sum(1 for e in circuit.elements if e["kind"] == abi.SP_EL_V)
        nt = circuit.num_nodes + nv
        steps = int(np.ceil(cfg.tstop / cfg.tstep)) if cfg.tstep > 0 and cfg.tstop > 0 else 0  # the library rejects bad steps
        out = dict(x=np.zeros((count, nt)), status=np.zeros(count, np.uint8),
                   probe=np.zeros((count, steps + 1)) if cfg.probe >= 0 else None)
        cols = 0
        if table is not None:
            table = np.ascontiguousarray(table, dtype=np.float64)
            cols = table.shape[1]
        cc = circuit.to_c()
        check(self._ptr, load().sp_transient(self._ptr, C.byref(cc), C.byref(dc_cfg), C.byref(cfg), seed, first,
                                             count, _vp(table), cols, _vp(out["x"]), _vp(out["probe"]),
                                             _vp(out["status"])))
        return out

    def transient_device(self, topo: Topology, dc_cfg, cfg, seed, count, x, status, probe=None, first: int = 0,
                         table=None, stream: int = 0):
        """Device-buffer variant (torch CUDA tensors): x [count][nt] f64, status uint8 [count],
        probe [count][steps + 1] f64."""
        cols = 0 if table is None else int(table.shape[1])
        check(self._ptr, load().sp_transient_device(self._ptr, topo._ptr, C.byref(dc_cfg), C.byref(cfg), seed,
                                                    first, count, _vp(table), cols, _vp(x), _vp(probe),
                                                    _vp(status), stream))

    # -- power-grid corners ----------------------------------------------------
    def grid_solve(self, cfg, seed: int, count: int, first: int = 0) -> dict:
        """Host-buffer power-grid corner sweep (sp_grid_solve): dict of x [count][rows*cols+1],
        newton, krylov, status, resid."""
        n = cfg.rows * cfg.cols + 1
        out = dict(x=np.zeros((count, n)), newton=np.zeros(count, np.int32), krylov=np.zeros(count, np.int32),
                   status=np.zeros(count, np.uint8), resid=np.zeros(count))
        check(self._ptr, load().sp_grid_solve(self._ptr, C.byref(cfg), seed, first, count, _vp(out["x"]),
                                              _vp(out["newton"]), _vp(out["krylov"]), _vp(out["status"]),
                                              _vp(out["resid"])))
        return out

    def grid_solve_device(self, cfg, seed, count, x, newton, krylov, status, resid, first: int = 0, stream: int = 0):
        check(self._ptr, load().sp_grid_solve_device(self._ptr, C.byref(cfg), seed, first, count, _vp(x),
                                                     _vp(newton), _vp(krylov), _vp(status), _vp(resid), stream))

    # -- statistics ------------------------------------------------------------
    def bsim3_eval_device(self, pmos: bool, card, bias, out, region=None, stream: int = 0):
        """Batched BSIM3 DC evaluation (Bsim3Mosfet::evaluate) on CUDA float64 tensors: card[count][SP_B3_CARD],
        bias[count][3] = (vgs, vds, vbs) -> out[count][6] = (ids, gds, gm, gmbs, vth, vdsat), region[count] uint8."""
        count = int(bias.shape[0])
        if tuple(card.shape) != (count, abi.SP_B3_CARD) or tuple(bias.shape) != (count, 3) or tuple(out.shape) != (count, 6):
            raise ValueError("card [count][SP_B3_CARD], bias [count][3] and out [count][6] expected")
        for t in (card, bias, out):
            if not (t.is_cuda and t.is_contiguous()) or t.element_size() != 8:
                raise ValueError("contiguous CUDA float64 tensors expected")
        check(self._ptr, load().sp_bsim3_eval_device(self._ptr, int(pmos), _vp(card), _vp(bias), count, _vp(out),
                                                     _vp(region), stream))
        return out

    def histogram_device(self, values, col: int, num_bins: int, min: float = None, max: float = None, status=None,
                         stream: int = 0):
        """Histogram of column `col` of a [rows][ld] CUDA tensor (Histogram::new; with min/max None, the
        column's range as Histogram::from_sweep takes it, widened by 0.5 on each side if flat)."""
        import torch
        rows, ld = int(values.shape[0]), int(values.shape[1])
        if min is None or max is None:
            col_v = values[:, col] if status is None else values[:, col][(status & abi.SP_ST_MASK) == 0]
            lo, hi = float(col_v.min()), float(col_v.max())
            if abs(hi - lo) < np.finfo(float).eps:
                lo, hi = lo - 0.5, hi + 0.5
            min = lo if min is None else min
            max = hi if max is None else max
        bins = torch.empty(num_bins, dtype=torch.int64, device=values.device)
        check(self._ptr, load().sp_histogram_device(self._ptr, _vp(values), rows, ld, col, _vp(status), min, max,
                                                    num_bins, _vp(bins), stream))
        return bins, min, max

    def yield_device(self, values, specs, status=None, stream: int = 0):
        """Pass counts of [(col, lower, upper)] specs and of all together (YieldAnalysis)."""
        import torch
        rows, ld = int(values.shape[0]), int(values.shape[1])
        arr = (abi.SpYieldSpec * max(len(specs), 1))(*[abi.SpYieldSpec(c, 0, lo, hi) for c, lo, hi in specs])
        out = torch.empty(len(specs) + 1, dtype=torch.int64, device=values.device)
        check(self._ptr, load().sp_yield_device(self._ptr, _vp(values), rows, ld, _vp(status), C.addressof(arr),
                                                len(specs), _vp(out), stream))
        return out

    def profile_read(self) -> dict:
        """{kernel name: (launches, total_ms)} since the last read."""
        from ._lib import SpKernelTime
        buf = (SpKernelTime * 64)()
        cnt = C.c_int(0)
        check(self._ptr, load().sp_profile_read(self._ptr, buf, 64, C.byref(cnt)))
        return {buf[i].name.decode(): (int(buf[i].launches), float(buf[i].total_ms)) for i in range(cnt.value)}

    def moments_device(self, values, rows, ld, cols, status, out, stream: int = 0):
        check(self._ptr, load().sp_moments_device(self._ptr, _vp(values), rows, ld, cols, _vp(status), _vp(out),
                                                  stream))


class Mlp:
    """The BF16 warm-start network (sp_mlp)."""

    def __init__(self, ctx: Context, n_in: int, n_out: int, n_hidden: int = 256, n_layers: int = 3,
                 seed: int = 0):
        from ._lib import SpMlpDesc
        self.ctx = ctx
        self.n_in, self.n_out, self.n_hidden, self.n_layers = n_in, n_out, n_hidden, n_layers
        self._ptr = C.c_void_p()
        d = SpMlpDesc(n_in, n_hidden, n_layers, n_out, seed)
        check(ctx._ptr, load().sp_mlp_create(ctx._ptr, C.byref(d), C.byref(self._ptr)))

    def close(self):
        if self._ptr:
            load().sp_mlp_destroy(self._ptr)
            self._ptr = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def num_params(self) -> int:
        return load().sp_mlp_num_params(self._ptr)

    def get_params(self) -> np.ndarray:
        out = np.zeros(self.num_params, np.float32)
        check(self.ctx._ptr, load().sp_mlp_get_params(self._ptr, _vp(out)))
        return out

    def set_params(self, p):
        p = np.ascontiguousarray(p, dtype=np.float32)
        check(self.ctx._ptr, load().sp_mlp_set_params(self._ptr, _vp(p)))

    def set_io(self, in_slots, in_mean, in_scale, out_mean, out_scale):
        arrs = [np.ascontiguousarray(in_slots, dtype=np.int32)] + [
            np.ascontiguousarray(a, dtype=np.float32) for a in (in_mean, in_scale, out_mean, out_scale)]
        check(self.ctx._ptr, load().sp_mlp_set_io(self._ptr, *[_vp(a) for a in arrs]))

    def set_linear(self, lin):
        """FP64 linear term [n_out][n_in] of the warm start (None removes it)."""
        arr = None if lin is None else np.ascontiguousarray(lin, dtype=np.float64)
        check(self.ctx._ptr, load().sp_mlp_set_linear(self._ptr, _vp(arr)))

    def set_inference_kernel(self, kind: int):
        """abi.SP_MLP_KERNEL_{AUTO,TCGEN05,MMA_SYNC,LAYERED,LINEAR} for the warm start
        (LINEAR: the linear term alone, evaluated by the learned sweep's draw kernel)."""
        check(self.ctx._ptr, load().sp_mlp_set_inference_kernel(self._ptr, kind))

    def set_training_kernel(self, kind: int):
        """abi.SP_MLP_KERNEL_{AUTO,TCGEN05,MMA_SYNC} for the training GEMMs."""
        check(self.ctx._ptr, load().sp_mlp_set_training_kernel(self._ptr, kind))

    def fault(self) -> int:
        """Waits for the device; 1 if a tcgen05 training GEMM gave up a bounded
        wait, | 2 if the tcgen05 warm start did (sticky flags), else 0."""
        v = C.c_int(0)
        check(self.ctx._ptr, load().sp_mlp_fault(self._ptr, C.byref(v)))
        return v.value

    def warm_start_device(self, params_soa, stride, rows, x0, stream=0):
        """x0[rows][n_out] (FP64) from SoA parameters (slot s of sample i at s*stride+i)."""
        check(self.ctx._ptr, load().sp_mlp_warm_start_device(self._ptr, _vp(params_soa), stride, rows, _vp(x0),
                                                             stream))

    def forward_device(self, x, rows, y, stream=0):
        check(self.ctx._ptr, load().sp_mlp_forward_device(self._ptr, _vp(x), rows, _vp(y), stream))

    def gradients_device(self, x, t, rows, grads, loss=None, stream=0):
        check(self.ctx._ptr, load().sp_mlp_gradients_device(self._ptr, _vp(x), _vp(t), rows, _vp(grads),
                                                            _vp(loss), stream))

    def train_device(self, x, t, rows, batch, epochs, lr, epoch_loss=None, stream=0):
        check(self.ctx._ptr, load().sp_mlp_train_device(self._ptr, _vp(x), _vp(t), rows, batch, epochs,
                                                        C.c_float(lr), _vp(epoch_loss), stream))

    def layer_shapes(self):
        """[(out_pad, in_pad)] per layer of the flat parameter vector."""
        kin = (self.n_in + 31) // 32 * 32
        kout = (self.n_out + 31) // 32 * 32
        dims = [kin] + [self.n_hidden] * self.n_layers + [kout]
        return [(dims[i + 1], dims[i]) for i in range(len(dims) - 1)]

    def unflatten(self, flat):
        """[(Wt, b)] views of a flat parameter vector."""
        out, o = [], 0
        for (r, c) in self.layer_shapes():
            W = flat[o:o + r * c].reshape(r, c)
            o += r * c
            b = flat[o:o + r]
            o += r
            out.append((W, b))
        return out


def draw_params_host(circuit: Circuit, seed: int, count: int, first: int = 0, table=None,
                     threads: int = 0) -> np.ndarray:
    """Per-sample parameters [count][num_params] drawn on the host with the C
    library's ln/cos/exp (sp_draw_params_host): the reference's own draw bits
    on this host (crates/spicier-batched-sweep/src/rng.rs:120-150)."""
    npar = len(circuit.params)
    out = np.zeros((count, max(npar, 1)))
    cols = 0
    if table is not None:
        table = np.ascontiguousarray(table, dtype=np.float64)
        cols = table.shape[1]
    cc = circuit.to_c()
    rc = load().sp_draw_params_host(C.byref(cc), seed, first, count, _vp(table), cols, _vp(out), threads)
    if rc != 0:
        raise SpicierError(rc, "sp_draw_params_host")
    return out[:, :npar]


def table_circuit(circuit: Circuit) -> Circuit:
    """A copy of `circuit` whose parameter slot k reads column k of the sweep's
    table: run it with the table from draw_params_host to sweep on the host
    libm's draws (same elements, same slots, same nodeset)."""
    import copy
    c = copy.copy(circuit)
    c._c_keepalive = None  # the copy builds its own sp_circuit view
    c.node_index = dict(circuit.node_index)
    c.elements = copy.deepcopy(circuit.elements)
    c.param_labels = list(circuit.param_labels)
    c.pulses = list(circuit.pulses)
    c.nodeset = dict(circuit.nodeset)
    c.params = [(abi.SP_DRAW_TABLE, k, 0.0, 0.0) for k in range(len(circuit.params))]
    return c


def specialized_source(circuit: Circuit, precision: int = abi.SP_PREC_MIXED, compile: bool = False):
    """(source, jacobian_slots) of a circuit's specialised kernel; compiles it
    with NVRTC when asked (no device needed).  Raises on failure."""
    buf = C.create_string_buffer(1 << 21)
    nnz = C.c_int(0)
    rc = load().sp_specialize_source(C.byref(circuit.to_c()), precision, 1 if compile else 0, buf, len(buf),
                                     C.byref(nnz))
    if rc != 0:
        raise SpicierError(rc, buf.value.decode(errors="replace")[:2000])
    return buf.value.decode(errors="replace"), nnz.value


def newton_dc_learned_device(ctx: Context, topo: Topology, mlp: Mlp, cfg, seed, count, x, first=0, table=None,
                             iters=None, status=None, resid=None, moments=None, stream=0):
    cols = 0 if table is None else int(table.shape[1])
    check(ctx._ptr, load().sp_newton_dc_learned_device(ctx._ptr, topo._ptr, mlp._ptr, C.byref(cfg), seed, first,
                                                       count, _vp(table), cols, _vp(x), _vp(iters), _vp(status),
                                                       _vp(resid), _vp(moments), stream))


def newton_dc_learned(ctx: Context, circuit: Circuit, mlp: Mlp, cfg, seed: int, count: int, first: int = 0,
                      table=None) -> NewtonResult:
    """Host-buffer warm-started batched DC operating points (sp_newton_dc_learned)."""
    n = circuit.n
    x = np.zeros((count, n))
    iters = np.zeros(count, np.int32)
    status = np.zeros(count, np.uint8)
    r = np.zeros(count)
    cols = 0
    if table is not None:
        table = np.ascontiguousarray(table, dtype=np.float64)
        cols = table.shape[1]
    cc = circuit.to_c()
    check(ctx._ptr, load().sp_newton_dc_learned(ctx._ptr, C.byref(cc), mlp._ptr, C.byref(cfg), seed, first, count,
                                                _vp(table), cols, _vp(x), _vp(iters), _vp(status), _vp(r), None))
    return NewtonResult(x, iters, status, r, None, None)


# ---------------------------------------------------------------------------
# BatchedLuSolver mirror and the sweep API
# ---------------------------------------------------------------------------
class Gb300BatchedSolver:
    """BatchedLuSolver implementation backed by the GB300 kernels."""

    def __init__(self, config: Optional[GpuBatchConfig] = None, device: int = 0):
        self.ctx = Context(device)
        if config is not None:
            self.ctx.set_config(config)

    def solve_batch(self, matrices, rhs, n: int, batch_size: int) -> BatchedSolveResult:
        return self.ctx.solve_batch(matrices, rhs, n, batch_size)

    def should_use_gpu(self, matrix_size: int, batch_size: int) -> bool:
        return self.ctx.config().should_use_gpu(matrix_size, batch_size)

    def backend_type(self) -> BackendType:
        return BackendType(load().sp_backend_type())

    def config(self) -> GpuBatchConfig:
        return self.ctx.config()


class BackendSelector:
    """BackendSelector (solver.rs:137-312) reduced to the one backend here."""

    def __init__(self, device: int = 0, config: Optional[GpuBatchConfig] = None):
        self.device = device
        self.config = config or GpuBatchConfig()

    @staticmethod
    def auto():
        return BackendSelector()

    def create_solver(self) -> Gb300BatchedSolver:
        return Gb300BatchedSolver(self.config, self.device)


@dataclass
class ParameterVariation:
    """crates/spicier-solver/src/sweep.rs:15-54 (defaults +-10 %, sigma 5 %)."""
    name: str
    nominal: float
    min: float = math.nan
    max: float = math.nan
    sigma: float = 0.05

    def __post_init__(self):
        if math.isnan(self.min):
            self.min = self.nominal * 0.9
        if math.isnan(self.max):
            self.max = self.nominal * 1.1

    def with_bounds(self, lo, hi):
        self.min, self.max = lo, hi
        return self

    def with_sigma(self, s):
        self.sigma = s
        return self


@dataclass
class SweepPoint:
    parameters: List[float]


class MonteCarloGenerator:
    """LCG Monte Carlo generator (sweep.rs:145-200), seed default 12345."""

    def __init__(self, num_samples: int, seed: int = 12345):
        self.num_samples, self.seed = num_samples, seed

    def with_seed(self, seed):
        self.seed = seed
        return self

    def generate(self, variations: Sequence[ParameterVariation]) -> List[SweepPoint]:
        state = self.seed & 0xFFFFFFFFFFFFFFFF

        def nxt():
            nonlocal state
            state = (state * 6364136223846793005 + 1) & 0xFFFFFFFFFFFFFFFF
            return (state >> 33) / float(1 << 31)

        pts = []
        for _ in range(self.num_samples):
            vals = []
            for v in variations:
                u1 = max(nxt(), 1e-10)
                u2 = nxt()
                z = math.sqrt(-2.0 * math.log(u1)) * math.cos(2.0 * math.pi * u2)
                vals.append(min(max(v.nominal + z * v.sigma * v.nominal, v.min), v.max))
            pts.append(SweepPoint(vals))
        return pts


class CornerGenerator:
    """All 2^k min/max corners, bit j -> parameter j (sweep.rs:202-227)."""

    def generate(self, variations):
        if not variations:
            return [SweepPoint([])]
        k = len(variations)
        return [SweepPoint([v.max if (i >> j) & 1 else v.min for j, v in enumerate(variations)])
                for i in range(1 << k)]


class LinearSweepGenerator:
    """min..max in num_points steps, all parameters together (sweep.rs:229-266)."""

    def __init__(self, num_points: int):
        self.num_points = num_points

    def generate(self, variations):
        if not variations:
            return [SweepPoint([])]
        out = []
        for i in range(self.num_points):
            t = i / (self.num_points - 1) if self.num_points > 1 else 0.5
            out.append(SweepPoint([v.min + t * (v.max - v.min) for v in variations]))
        return out


@dataclass
class GpuBatchedSweepResult:
    """crates/spicier-batched-sweep/src/sweep.rs:15-55."""
    solutions: List[np.ndarray]
    points: List[SweepPoint]
    converged_count: int
    total_count: int
    singular_indices: List[int]
    used_gpu: bool
    backend_used: BackendType

    def node_voltages(self, node_index: int):
        return [s[node_index] for s in self.solutions]


def solve_batched_sweep_gpu(backend: BackendSelector, factory, generator, variations,
                            criteria=None, config: Optional[GpuBatchConfig] = None) -> GpuBatchedSweepResult:
    """Linear sweep through BatchedLuSolver::solve_batch (sweep.rs:101-217):
    generate points, let ``factory.create_stamper(params)`` stamp each
    point's dense system (stamp_linear(matrix, rhs) on numpy arrays), solve the
    batch on the GPU.  ``criteria`` is accepted and unused, as in the reference."""
    points = generator.generate(variations)
    total = len(points)
    if total == 0:
        return GpuBatchedSweepResult([], [], 0, 0, [], False, BackendType.Cpu)
    first = factory.create_stamper(points[0].parameters)
    size = first.num_nodes() + first.num_vsources()
    solver = backend.create_solver()
    mats = np.zeros((total, size, size))
    rhs = np.zeros((total, size))
    for i, p in enumerate(points):
        st = factory.create_stamper(p.parameters)
        m = np.zeros((size, size))
        b = np.zeros(size)
        st.stamp_linear(m, b)
        mats[i] = m.T  # column-major
        rhs[i] = b
    res = solver.solve_batch(mats.ravel(), rhs.ravel(), size, total)
    sols = [res.solution(i).copy() for i in range(total)]
    return GpuBatchedSweepResult(sols, points, total - len(res.singular_indices), total, res.singular_indices,
                                 True, solver.backend_type())


def solve_newton_sweep_gpu(ctx: Context, circuit: Circuit, seed: int, num_samples: int,
                           criteria: Optional[abi.SpNewtonConfig] = None, generator=None, variations=None,
                           x0=None) -> NewtonResult:
    """Nonlinear sweep: every point solved by batched Newton on the GPU.
    Parameters drawn by the hash RNG inside the kernel (seed), or — when a
    host ``generator`` is given — taken from its points as a table whose
    columns the circuit references with ``Table(col)``."""
    cfg = criteria or abi.newton_config()
    table = None
    if generator is not None:
        pts = generator.generate(variations or [])
        table = np.array([p.parameters for p in pts], dtype=np.float64)
        num_samples = len(pts)
    return ctx.newton_dc(circuit, cfg, seed, num_samples, table=table, x0=x0, resid=True)
