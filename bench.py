#!/usr/bin/env python3
"""Benchmark of the batched Newton sweep: converged DC operating points per
second on one GB300.

Workload (one "step"): Monte Carlo DC operating points of the two-stage Miller
op-amp buffer (spicier_gb300.configs.miller_opamp, MNA size 12), 65,536
samples, parameters drawn on the device by the stateless hash RNG (seed 1,
each step a fresh range of sweep indices), SPICE tolerances reltol 1e-3,
vntol 1e-6 V, abstol 1e-12 A.  Arms:
  * headline: mixed precision (FP32 LU, FP64 residual/update) with the
    learned MLP warm start when a trained network is present, else the
    circuit nodeset start;
  * plain FP64 on the GPU (same start rules as the reference API: nodeset);
  * --impl reference: the reference algorithm's CPU implementation (the C++
    restatement; Spicier's Rust cannot be built here) on all host cores.
One JSON line on stdout (rank 0).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

METRIC = "converged Newton solves/sec on 1 GB300: mixed+learned vs plain FP64, same tol"
UNIT = "solves/s"
SEED = 1
PROFILES = os.path.join(ROOT, "profiles")


def env_int(k, d):
    try:
        return int(os.environ.get(k, d))
    except ValueError:
        return d


def read_profile_number(fname, key):
    p = os.path.join(PROFILES, fname)
    if not os.path.exists(p):
        return None
    for line in open(p):
        if line.strip().startswith(key + ":"):
            try:
                return float(line.split(":", 1)[1].split()[0])
            except (ValueError, IndexError):
                return None
    return None


class Clocks:
    """nvidia-smi sampling during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "50"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        os.unlink(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def structural_nnz(circuit):
    """Structural nonzeros of the MNA matrix of a circuit (for the flop count)."""
    from spicier_gb300 import abi
    pos = set()
    nn = circuit.num_nodes

    def add(r, c):
        if r >= 0 and c >= 0:
            pos.add((r, c))

    for e in circuit.elements:
        a, b, c3 = e["node"]
        k = e["kind"]
        if k in (abi.SP_EL_R, abi.SP_EL_D):
            for r in (a, b):
                for c in (a, b):
                    add(r, c)
        elif k in (abi.SP_EL_V, abi.SP_EL_L):
            row = nn + e["branch"]
            for t in (a, b):
                add(t, row)
                add(row, t)
        elif k in (abi.SP_EL_NMOS, abi.SP_EL_PMOS, abi.SP_EL_NPN, abi.SP_EL_PNP):
            for r in (a, c3, b) if k >= abi.SP_EL_NPN else (a, c3):
                for c in (a, b, c3):
                    add(r, c)
    return len(pos)


def mosfet_count(circuit):
    from spicier_gb300 import abi
    return sum(1 for e in circuit.elements if e["kind"] in (abi.SP_EL_NMOS, abi.SP_EL_PMOS))


def cpu_baseline(circuit, samples, threads=0):
    """The oracle port (the reference algorithm restated in C++) timed on the
    host cores over one bounded sample of the workload."""
    import oracle
    from spicier_gb300 import abi
    oracle.lib()
    cfg = abi.newton_config(precision=abi.SP_PREC_FP64)
    t0 = time.perf_counter()
    _x, _it, st, _p = oracle.newton_dc(circuit, cfg, SEED, samples, threads=threads)
    dt = time.perf_counter() - t0
    conv = int(((st & 0x0F) == 0).sum())
    return conv / dt, dt, conv


def run_reference(args):
    """--impl reference: the reference algorithm's CPU implementation."""
    rank = env_int("RANK", 0)
    if rank != 0:
        return 0
    from spicier_gb300 import configs
    circ = configs.miller_opamp()
    cores = os.cpu_count() or 1
    sample = min(args.samples, 65536)
    for _ in range(max(args.warmup, 0)):
        cpu_baseline(circ, sample)
    rates, total_t, total_conv = [], 0.0, 0
    for _ in range(args.steps):
        r, dt, conv = cpu_baseline(circ, sample)
        rates.append(r)
        total_t += dt
        total_conv += conv
    value = total_conv / total_t if total_t > 0 else 0.0
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * total_t / max(args.steps, 1),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": "miller_opamp_mc_dc", "samples_per_step": sample, "mna_size": circ.n,
                   "precision": "fp64", "start": "nodeset", "seed": SEED, "parallelism": "host threads"},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": f"{sample} op-amp Monte Carlo samples per step, plain FP64 Newton from the nodeset"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=300)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--samples", type=int, default=65536)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    if args.impl == "reference":
        return run_reference(args)

    import numpy as np
    import torch

    import spicier_gb300 as sg
    from spicier_gb300 import abi, configs

    rank, world, local = env_int("RANK", 0), env_int("WORLD_SIZE", 1), env_int("LOCAL_RANK", 0)
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    def barrier():
        torch.cuda.synchronize()
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()

    ctx = sg.Context(local)
    circ = configs.miller_opamp()
    topo = ctx.topology(circ)
    N, n = args.samples, circ.n
    dev = torch.device("cuda", local)
    x = torch.empty((N, n), dtype=torch.float64, device=dev)
    iters = torch.empty(N, dtype=torch.int32, device=dev)
    status = torch.empty(N, dtype=torch.uint8, device=dev)
    resid = torch.empty(N, dtype=torch.float64, device=dev)
    moments = torch.empty((n, 5), dtype=torch.float64, device=dev)
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device=dev)  # 256 MiB > 129 MB L2
    stream = torch.cuda.current_stream().cuda_stream

    # sweep indices: each rank and each step take their own range (weak scaling)
    per_rank = N * (args.steps + args.warmup + 4)

    def sweep(cfg, first):
        ctx.newton_dc_device(topo, cfg, SEED, N, x, first=first, iters=iters, status=status, resid=resid,
                             moments=moments, stream=stream)

    def timed(cfg, base):
        for w in range(args.warmup):
            sweep(cfg, base + w * N)
        barrier()
        ctx.profile_enable(True)
        ctx.profile_read()
        total_ms, conv, it_sum, rmax = 0.0, 0, 0, 0.0
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        for k in range(args.steps):
            flush.fill_(float(k))  # L2 flush between timed steps (not timed)
            e0.record()
            sweep(cfg, base + (args.warmup + k) * N)
            e1.record()
            e1.synchronize()
            total_ms += e0.elapsed_time(e1)
            ok = (status & 0x0F) == 0
            conv += int(ok.sum().item())
            it_sum += int(iters.sum().item())
            rmax = max(rmax, float(resid[ok].max().item()) if conv else 0.0)
        barrier()
        prof = ctx.profile_read()
        ctx.profile_enable(False)
        t = torch.tensor([total_ms], dtype=torch.float64, device=dev)
        c = torch.tensor([conv], dtype=torch.float64, device=dev)
        if dist is not None:
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
            dist.all_reduce(c, op=dist.ReduceOp.SUM)
        return float(t.item()), int(c.item()), it_sum / (N * args.steps), rmax, prof

    base = rank * per_rank
    cfg_plain = abi.newton_config(precision=abi.SP_PREC_FP64)
    cfg_mixed = abi.newton_config(precision=abi.SP_PREC_MIXED)
    plain_ms, plain_conv, plain_it, plain_r, _ = timed(cfg_plain, base)
    clocks = Clocks(local)
    clocks.start()
    mix_ms, mix_conv, mix_it, mix_r, prof = timed(cfg_mixed, base)
    clk = clocks.stop()

    value = mix_conv / (mix_ms / 1e3)
    plain_value = plain_conv / (plain_ms / 1e3)

    # e2e through the public host-buffer API: pinned host outputs, the
    # circuit description uploaded by the call, outputs read back every step.
    pin_x = torch.empty((N, n), dtype=torch.float64, pin_memory=True)
    pin_it = torch.empty(N, dtype=torch.int32, pin_memory=True)
    pin_st = torch.empty(N, dtype=torch.uint8, pin_memory=True)
    pin_r = torch.empty(N, dtype=torch.float64, pin_memory=True)
    from spicier_gb300._lib import check, load
    import ctypes as C
    cc = circ.to_c()

    def host_call(first):
        check(ctx._ptr, load().sp_newton_dc(ctx._ptr, C.byref(cc), C.byref(cfg_mixed), SEED, first, N, None, 0,
                                            None, pin_x.data_ptr(), pin_it.data_ptr(), pin_st.data_ptr(),
                                            pin_r.data_ptr(), None, None))

    for w in range(args.warmup):
        host_call(base + w * N)
    barrier()
    e2e_s, e2e_conv = 0.0, 0
    for k in range(args.steps):
        flush.fill_(float(k))
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        host_call(base + (args.warmup + k) * N)
        e2e_s += time.perf_counter() - t0
        e2e_conv += int(((pin_st.numpy() & 0x0F) == 0).sum())
    h2d = (C.sizeof(sg.abi.SpElement) * len(circ.elements) + C.sizeof(sg.abi.SpParam) * len(circ.params)
           + 8 * n + 4 * len(circ.elements))
    d2h = N * (8 * n + 4 + 1 + 8)
    t = torch.tensor([e2e_s], dtype=torch.float64, device=dev)
    if dist is not None:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    e2e_value = e2e_conv * world / float(t.item())

    # roofline of the dominant kernel (the mixed primary Newton kernel)
    kname = "newton_primary_mixed"
    launches, kms = prof.get(kname, (0, 0.0))
    avg_ms = kms / max(launches, 1)
    m, nnz = mosfet_count(circ), structural_nnz(circ)
    fp64_per_iter = 30 * m + 4 * nnz + 3 * n          # device models, FP64 residual, update + test
    fp32_per_iter = (2 * n ** 3) // 3 + 2 * n * n     # FP32 LU factor + solve
    fp64_flops = fp64_per_iter * mix_it * N
    fp32_flops = fp32_per_iter * mix_it * N
    fp64_peak = read_profile_number("pipe_peaks_gb300.txt", "fp64_tflops") or 1.21
    fp32_peak = read_profile_number("pipe_peaks_gb300.txt", "fp32_tflops") or 70.5
    ach = fp64_flops / (avg_ms * 1e-3) / 1e12 if avg_ms > 0 else 0.0
    traffic = read_profile_number("newton_mixed_opamp.txt", "dram_bytes_per_launch")
    roofline = {"bound": "fp64", "achieved": ach, "peak": fp64_peak, "unit": "TFLOP/s",
                "frac": ach / fp64_peak, "traffic": traffic,
                "peak_source": "measured on this pool's GB300 by the FMA-chain probe (profiles/pipe_peaks_gb300.txt)",
                "fp32_achieved": fp32_flops / (avg_ms * 1e-3) / 1e12 if avg_ms > 0 else 0.0,
                "fp32_peak": fp32_peak, "kernel": kname, "avg_launch_ms": avg_ms,
                "fp64_flops_per_launch": fp64_flops, "fp32_flops_per_launch": fp32_flops}
    hbm_peak = 6770.8
    try:
        hbm_peak = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))["hbm_gbs"]
    except (OSError, KeyError, ValueError):
        pass
    per_sample_bytes = 8 * (topo_derived(circ) + n) + 4 + 1 + 8
    alg_bytes = per_sample_bytes * N
    roofline_hbm = {"bound": "hbm", "achieved": alg_bytes / (avg_ms * 1e-3) / 1e9 if avg_ms > 0 else 0.0,
                    "peak": hbm_peak, "unit": "GB/s",
                    "frac": alg_bytes / (avg_ms * 1e-3) / 1e9 / hbm_peak if avg_ms > 0 else 0.0,
                    "bytes_per_launch": alg_bytes}

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        r, dt, _ = cpu_baseline(circ, N)
        cpu = {"value": r, "unit": UNIT, "cores": os.cpu_count() or 1, "kind": "port",
               "sample": f"{N} op-amp Monte Carlo samples (one step), plain FP64 Newton from the nodeset, "
                         f"{dt:.2f} s on all host threads"}

    gpu_launches = sum(v[0] for v in prof.values())
    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": mix_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64/f32",
            "data": "synthetic (hash-RNG Monte Carlo draws on device, seed 1)",
            "config": {"workload": "miller_opamp_mc_dc", "samples_per_step": N, "mna_size": n,
                       "precision": "mixed (FP32 LU, FP64 residual/update/models)",
                       "warm_start": "nodeset", "tolerances": "reltol 1e-3, vntol 1e-6 V, abstol 1e-12 A",
                       "l2": "flushed between timed steps (256 MiB write)",
                       "parallelism": "replicas" if world > 1 else "single GPU"},
            "plain_fp64": {"value": plain_value, "unit": UNIT, "ms_per_step": plain_ms / args.steps,
                           "iters_per_solve": plain_it, "max_resid_A": plain_r},
            "speedup_vs_plain_fp64": value / plain_value if plain_value else None,
            "iters_per_solve": mix_it, "max_resid_A": mix_r,
            "converged_fraction": mix_conv / (N * args.steps * world),
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
            "roofline": roofline, "roofline_hbm": roofline_hbm,
            "kernel_ms": {k: v[1] / max(v[0], 1) for k, v in prof.items()},
            "gpu_launches": gpu_launches,
            "clocks": clk,
            "cpu_baseline": cpu,
        }
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()
    return 0


def topo_derived(circuit):
    from spicier_gb300 import abi
    cnt = 0
    for e in circuit.elements:
        k = e["kind"]
        cnt += 3 if k in (abi.SP_EL_D, abi.SP_EL_NMOS, abi.SP_EL_PMOS) else 8 if k in (abi.SP_EL_NPN, abi.SP_EL_PNP) else 1
    return cnt


if __name__ == "__main__":
    sys.exit(main())
