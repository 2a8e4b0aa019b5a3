"""Autotuner of the launch settings: a timed search per (setting, size
bucket), cached in a JSON file per GPU model.

The reference dispatches on fixed thresholds (DispatchConfig,
crates/spicier-solver/src/dispatch.rs:85-120; GpuBatchConfig,
crates/spicier-batched-sweep/src/solver.rs:15-40).  Here the library's
built-in heuristics pick threads per instance and tile shapes, and this
module times the alternatives on the caller's own workload and stores the
fastest with sp_tune_set (include/spicier_gb300.h lists the settings):

  lu.cta              thread-per-system or CTA-per-system batched LU (n <= 28)
  newton.block.<p>    threads per block of the thread-per-sample Newton kernels
  spec.bpsm.<p>       resident blocks per SM of the topology-specialised kernel
  ladder.bpsm         resident blocks per SM of the ladder transients
  mlp.teams           128-sample tiles in flight per SM of the warm-start network

No setting changes any result (each candidate runs the same arithmetic per
sample); the tuner only times.  A cache file holds, per GPU name, the chosen
value of every "<setting>@<bucket>" key and the timings that chose it;
Autotuner.apply() loads it into a context.  A value of 0 stands for the
built-in heuristic (the key is then absent from the library's table).
"""
from __future__ import annotations

import ctypes as C
import json
import os
from typing import Callable, Dict, Iterable, Optional

from . import _abi as abi
from ._lib import check, load

DEFAULT_CACHE = os.path.join(os.path.expanduser("~"), ".cache", "spicier_gb300", "tune.json")


def bucket(size: int) -> int:
    """Size bucket of a setting (sp_tune_bucket): the smallest power of two >= size, at least 4."""
    b = 4
    while b < size:
        b <<= 1
    return b


def key(setting: str, size: int) -> str:
    return f"{setting}@{bucket(size)}"


def device_name(device: int = 0) -> str:
    try:
        import torch
        return torch.cuda.get_device_name(device)
    except Exception:  # no GPU: cache entries stay addressable by name
        return "unknown"


class TuneCache:
    """{gpu name: {"settings": {key: value}, "timings": {key: {candidate: ms}}}} in a JSON file."""

    def __init__(self, path: Optional[str] = None):
        self.path = path or os.environ.get("SPICIER_GB300_TUNE_CACHE", DEFAULT_CACHE)
        self.data: Dict[str, dict] = {}
        if os.path.exists(self.path):
            with open(self.path) as f:
                self.data = json.load(f)

    def settings(self, gpu: str) -> Dict[str, int]:
        return dict(self.data.get(gpu, {}).get("settings", {}))

    def put(self, gpu: str, k: str, value: int, timings: Dict[int, float]):
        entry = self.data.setdefault(gpu, {"settings": {}, "timings": {}})
        entry["settings"][k] = int(value)
        entry["timings"][k] = {str(c): float(t) for c, t in timings.items()}

    def save(self):
        d = os.path.dirname(self.path)
        if d:
            os.makedirs(d, exist_ok=True)
        tmp = self.path + ".tmp"
        with open(tmp, "w") as f:
            json.dump(self.data, f, indent=1, sort_keys=True)
        os.replace(tmp, self.path)


class Autotuner:
    """Times candidate settings on a context's workload and keeps the fastest."""

    def __init__(self, ctx, cache: Optional[TuneCache] = None, reps: int = 5):
        self.ctx = ctx
        self.cache = cache or TuneCache()
        self.gpu = device_name(ctx.device)
        self.reps = reps

    # -- the library's table -------------------------------------------------------
    def set(self, k: str, value: int):
        check(self.ctx._ptr, load().sp_tune_set(self.ctx._ptr, k.encode(), int(value)))

    def get(self, k: str) -> Optional[int]:
        v = C.c_int(0)
        return v.value if load().sp_tune_get(self.ctx._ptr, k.encode(), C.byref(v)) == 1 else None

    def apply(self) -> Dict[str, int]:
        """Load this GPU's cached settings into the context."""
        s = self.cache.settings(self.gpu)
        for k, v in s.items():
            self.set(k, v)
        return s

    # -- timing ------------------------------------------------------------------
    def _time(self, run: Callable[[], None]) -> float:
        import torch
        run()  # warm-up (also compiles and allocates outside the timing)
        torch.cuda.synchronize()
        ts = []
        for _ in range(self.reps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            run()
            e1.record()
            e1.synchronize()
            ts.append(e0.elapsed_time(e1))
        ts.sort()
        return ts[len(ts) // 2]

    def search(self, setting: str, size: int, candidates: Iterable[int], run: Callable[[], None]) -> int:
        """Time run() under each candidate value of setting@bucket(size) (CUDA-
        event median) and keep the fastest."""
        k = key(setting, size)
        timings = {}
        for c in candidates:
            self.set(k, c)
            timings[c] = self._time(run)
        best = min(timings, key=timings.get)
        self.set(k, best)
        self.cache.put(self.gpu, k, best, timings)
        return best

    # -- the settings ----------------------------------------------------------------
    def tune_lu(self, sizes=(4, 8, 12, 16, 20, 24, 28), batch: int = 65536) -> Dict[int, int]:
        """Thread-per-system (0) or CTA-per-system (1) batched LU per size bucket."""
        import torch
        out = {}
        dev = torch.device("cuda", self.ctx.device)
        for n in sizes:
            A = torch.rand((batch, n, n), dtype=torch.float64, device=dev) + n * torch.eye(n, dtype=torch.float64,
                                                                                           device=dev)
            b = torch.rand((batch, n), dtype=torch.float64, device=dev)
            x = torch.empty_like(b)
            sing = torch.empty(batch, dtype=torch.uint8, device=dev)
            out[n] = self.search("lu.cta", n, (0, 1), lambda: self.ctx.solve_batch_device(A, b, n, batch, x, sing))
        return out

    def tune_newton(self, topo, precision: int, samples: int = 65536, seed: int = 1) -> Dict[str, int]:
        """Threads per block of the generic Newton kernels and, for FP64 and
        mixed precision, the resident blocks per SM of the topology-specialised
        kernel; both on `samples` samples of the topology's sweep."""
        import torch
        dev = torch.device("cuda", self.ctx.device)
        x = torch.empty((samples, topo.n), dtype=torch.float64, device=dev)
        st = torch.empty(samples, dtype=torch.uint8, device=dev)
        cfg = abi.newton_config(precision=precision)
        run = lambda: self.ctx.newton_dc_device(topo, cfg, seed, samples, x, status=st)
        pname = {abi.SP_PREC_FP64: "fp64", abi.SP_PREC_MIXED: "mixed", abi.SP_PREC_FP64_EXACT: "exact"}[precision]
        out = {}
        if precision != abi.SP_PREC_FP64_EXACT:
            try:
                self.ctx.specialize(topo, precision, True)
                out["spec.bpsm"] = self.search(f"spec.bpsm.{pname}", topo.n, (0, 1, 2, 3), run)
            finally:
                self.ctx.specialize(topo, precision, False)
        out["newton.block"] = self.search(f"newton.block.{pname}", topo.n, (0, 32, 64, 96, 128), run)
        return out

    def tune_ladder(self, cfg, count: int = 1024, seed: int = 1) -> int:
        """Resident blocks per SM of the ladder transients."""
        import torch
        dev = torch.device("cuda", self.ctx.device)
        ld = cfg.max_sections + 2
        x = torch.empty((count, ld), dtype=torch.float64, device=dev)
        ints = [torch.empty(count, dtype=torch.int32, device=dev) for _ in range(4)]
        st = torch.empty(count, dtype=torch.uint8, device=dev)
        probe = torch.empty((count, max(cfg.num_probe, 1)), dtype=torch.float64, device=dev)
        run = lambda: self.ctx.ladder_transient_device(cfg, seed, count, x, *ints, st, probe=probe)
        return self.search("ladder.bpsm", cfg.max_sections, (0, 1, 2), run)

    def tune_mlp(self, mlp, rows: int = 65536) -> int:
        """Tiles in flight per SM of the tcgen05 warm start (resident-weight
        shapes); `mlp` must have its I/O wiring set (sp_mlp_set_io)."""
        import numpy as np
        import torch
        dev = torch.device("cuda", self.ctx.device)
        P = torch.tensor(np.random.default_rng(0).normal(0, 1, (mlp.n_in, rows)), device=dev)
        x0 = torch.empty((rows, mlp.n_out), dtype=torch.float64, device=dev)
        run = lambda: mlp.warm_start_device(P, rows, rows, x0)
        return self.search("mlp.teams", mlp.n_hidden, (0, 2, 1), run)

    def save(self):
        self.cache.save()
