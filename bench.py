#!/usr/bin/env python3
"""Benchmark of the batched Newton sweep: converged DC operating points per
second on one GB300.

Workload (one "step"): Monte Carlo DC operating points of the two-stage Miller
op-amp buffer (spicier_gb300.configs.miller_opamp, MNA size 12), 65,536
samples, parameters drawn on the device by the stateless hash RNG (seed 1;
each step takes a fresh range of sweep indices), SPICE tolerances reltol 1e-3,
vntol 1e-6 V, abstol 1e-12 A.

Arms (all on the same sweep):
  * headline "mixed+learned": the BF16 warm-start network (trained before the
    timed region on 1,048,576 plain-FP64 solutions of seed 7; inputs: every
    swept parameter) predicts each sample's operating point, then the
    topology-specialised mixed-precision Newton kernel (FP32 sparse LU, FP64
    residual/update) converges it; misses fall back to the nodeset start and
    the gmin/source-stepping chain;
  * "plain FP64": the reference algorithm on the GPU — dense partial-pivot FP64
    LU in the companion form of solve_newton_raphson, started from the nodeset;
  * ablations: mixed precision from the nodeset; FP64 specialised kernel;
  * config 4 report: a 10-input network on 262,144 samples vs cold start;
  * --impl reference: the reference algorithm's CPU implementation (the C++
    restatement; Spicier's Rust cannot be built here) on all host cores.
One JSON line on stdout (rank 0).
"""
from __future__ import annotations

import argparse
import ctypes as C
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
TRAIN_SEED = 7
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
            return
        t0 = time.time()  # nvidia-smi takes a moment to start: wait for its first sample
        while time.time() - t0 < 10 and self.proc.poll() is None and os.path.getsize(self.path) == 0:
            time.sleep(0.05)

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
    """Structural nonzeros of the MNA matrix (for the flop counts)."""
    from spicier_gb300 import abi
    pos = set()
    nn = circuit.num_nodes

    def add(r, c):
        if r >= 0 and c >= 0:
            pos.add((r, c))

    for e in circuit.elements:
        a, b, c3 = e["node"][:3]
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
        elif k in (abi.SP_EL_BSIM3N, abi.SP_EL_BSIM3P):
            for r in (a, c3):
                for c in (a, b, c3, e["node"][3]):
                    add(r, c)
    return len(pos)


def derived_slots(circuit):
    from spicier_gb300 import abi
    cnt = 0
    for e in circuit.elements:
        k = e["kind"]
        cnt += 3 if k in (abi.SP_EL_D, abi.SP_EL_NMOS, abi.SP_EL_PMOS) else 8 if k in (abi.SP_EL_NPN,
                                                                                        abi.SP_EL_PNP) else 1
    return cnt


def cpu_baseline(circuit, samples, threads=0, min_seconds=0.0):
    """The oracle port (the reference algorithm restated in C++) timed on the
    host cores over a bounded sample of the workload: chunks of `samples`
    sweep indices, repeated until `min_seconds` have passed."""
    import oracle
    from spicier_gb300 import abi
    oracle.lib()
    cfg = abi.newton_config(precision=abi.SP_PREC_FP64)
    dt, conv, done = 0.0, 0, 0
    while True:
        t0 = time.perf_counter()
        _x, _it, st, _p = oracle.newton_dc(circuit, cfg, SEED, samples, first=done, threads=threads)
        dt += time.perf_counter() - t0
        conv += int(((st & 0x0F) == 0).sum())
        done += samples
        if dt >= min_seconds:
            break
    return conv / dt, dt, conv, done


def run_reference(args):
    """--impl reference: the reference algorithm's CPU implementation."""
    if env_int("RANK", 0) != 0:
        return 0
    from spicier_gb300 import configs
    circ = configs.miller_opamp()
    cores = os.cpu_count() or 1
    sample = min(args.samples, 65536)
    steps = max(1, args.steps)
    for _ in range(max(args.warmup, 0)):
        cpu_baseline(circ, sample)
    total_t, total_conv = 0.0, 0
    for _ in range(steps):
        _r, dt, conv, _done = cpu_baseline(circ, sample)
        total_t += dt
        total_conv += conv
    value = total_conv / total_t if total_t > 0 else 0.0
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": steps, "warmup": args.warmup, "ms_per_step": 1e3 * total_t / steps,
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
    ap.add_argument("--no-config4", action="store_true")
    ap.add_argument("--no-transient", action="store_true", help="skip the ladder-transient (workload 3) report")
    ap.add_argument("--no-grid", action="store_true", help="skip the power-grid (workload 5) report")
    ap.add_argument("--no-ac", action="store_true", help="skip the AC small-signal sweep report")
    ap.add_argument("--no-bsim3", action="store_true", help="skip the BSIM3 evaluation / sweep report")
    ap.add_argument("--train-samples", type=int, default=1 << 20)
    ap.add_argument("--no-ablations", action="store_true", help="skip the mixed-from-nodeset and FP64-specialised arms")
    ap.add_argument("--mlp-hidden", type=int, default=128, help="hidden width of the warm-start network")
    ap.add_argument("--mlp-layers", type=int, default=3, help="hidden layers of the warm-start network")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    if args.impl == "reference":
        return run_reference(args)

    import numpy as np
    import torch

    import spicier_gb300 as sg
    from spicier_gb300 import abi, configs
    from spicier_gb300._lib import check, load
    from spicier_gb300.learned import WarmStart, random_slots

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

    # set-up outside the timed regions: specialised kernel, warm-start network
    t0 = time.perf_counter()
    ctx.specialize(topo, abi.SP_PREC_MIXED, True)
    spec_s = time.perf_counter() - t0
    ws = WarmStart(ctx, circ, n_inputs=len(random_slots(circ)), n_hidden=args.mlp_hidden, n_layers=args.mlp_layers,
                   seed=3)
    rep = ws.train(topo, seed=TRAIN_SEED, samples=args.train_samples, epochs=16, batch=4096, lr=2e-3)

    cfg_plain = abi.newton_config(precision=abi.SP_PREC_FP64)
    cfg_mixed = abi.newton_config(precision=abi.SP_PREC_MIXED, warm_max_iterations=ws.WARM_MAX_ITERATIONS)
    base_index = rank * N * 100000

    # The timed sweeps return what the reference's solve returns (x, iterations,
    # status) plus the moments; the KCL residual is an extra output, computed
    # in an untimed re-run of the last timed sweep (the sweep is deterministic).
    def plain_step(first, r=None):
        ctx.newton_dc_device(topo, cfg_plain, SEED, N, x, first=first, iters=iters, status=status, resid=r,
                             moments=moments, stream=stream)

    def mixed_nodeset_step(first, r=None):
        ctx.newton_dc_device(topo, cfg_mixed, SEED, N, x, first=first, iters=iters, status=status, resid=r,
                             moments=moments, stream=stream)

    def learned_step(first, r=None):
        ws.sweep_device(topo, cfg_mixed, SEED, N, x, first=first, iters=iters, status=status, resid=r,
                        moments=moments, stream=stream)

    def timed(step, steps, clocks=None):
        for w in range(args.warmup):
            step(base_index + w * N)
        barrier()
        if clocks:
            clocks.start()
        total_ms, conv, it_sum, rmax, flags = 0.0, 0, 0, 0.0, {}
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        for k in range(steps):
            flush.fill_(float(k))  # L2 flush between timed steps (not timed)
            e0.record()
            step(base_index + (args.warmup + k) * N)
            e1.record()
            e1.synchronize()
            total_ms += e0.elapsed_time(e1)
            ok = (status & 0x0F) == 0
            conv += int(ok.sum().item())
            it_sum += int(iters.sum().item())
            for fl, cnt in zip(*np.unique(status.cpu().numpy(), return_counts=True)):
                flags[int(fl)] = flags.get(int(fl), 0) + int(cnt)
        clk = clocks.stop() if clocks else None
        barrier()
        # per-kernel times from a separate, untimed pass over the same sweeps: the
        # profiling events between kernels would keep the timed chain from
        # overlapping each kernel's launch with its predecessor's tail
        ctx.profile_enable(True)
        ctx.profile_read()
        for k in range(steps):
            flush.fill_(float(k))
            step(base_index + (args.warmup + k) * N)
        torch.cuda.synchronize()
        prof = ctx.profile_read()
        ctx.profile_enable(False)
        step(base_index + (args.warmup + steps - 1) * N, resid)  # untimed: residual of the last timed sweep
        ok = (status & 0x0F) == 0
        rmax = float(resid[ok].max().item()) if bool(ok.any()) else 0.0
        t = torch.tensor([total_ms], dtype=torch.float64, device=dev)
        c = torch.tensor([conv], dtype=torch.float64, device=dev)
        if dist is not None:
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
            dist.all_reduce(c, op=dist.ReduceOp.SUM)
        return dict(ms=float(t.item()), conv=int(c.item()), iters=it_sum / (N * steps), rmax=rmax, prof=prof,
                    clocks=clk, flags=flags, steps=steps)

    plain = timed(plain_step, args.steps)
    head = timed(learned_step, args.steps, clocks=Clocks(local))
    ablations = {}
    if not args.no_ablations:
        abl_steps = max(3, args.steps // 5)
        ablations["mixed_nodeset"] = timed(mixed_nodeset_step, abl_steps)
        ctx.specialize(topo, abi.SP_PREC_FP64, True)
        ablations["fp64_specialised_nodeset"] = timed(plain_step, abl_steps)
        ctx.specialize(topo, abi.SP_PREC_FP64, False)

    def rate(r):
        return r["conv"] / (r["ms"] / 1e3)

    value, plain_value = rate(head), rate(plain)

    # e2e through the public host-buffer API (pinned host outputs, the circuit
    # uploaded by the call, all outputs read back every step)
    pin_x = torch.empty((N, n), dtype=torch.float64, pin_memory=True)
    pin_it = torch.empty(N, dtype=torch.int32, pin_memory=True)
    pin_st = torch.empty(N, dtype=torch.uint8, pin_memory=True)
    cc = circ.to_c()

    def host_call(first):
        check(ctx._ptr, load().sp_newton_dc_learned(ctx._ptr, C.byref(cc), ws.mlp._ptr, C.byref(cfg_mixed), SEED,
                                                    first, N, None, 0, pin_x.data_ptr(), pin_it.data_ptr(),
                                                    pin_st.data_ptr(), None, None))

    for w in range(args.warmup):
        host_call(base_index + w * N)
    barrier()
    e2e_s, e2e_conv = 0.0, 0
    e2e_steps = min(args.steps, 100)
    for k in range(e2e_steps):
        flush.fill_(float(k))
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        host_call(base_index + (args.warmup + k) * N)
        e2e_s += time.perf_counter() - t0
        e2e_conv += int(((pin_st.numpy() & 0x0F) == 0).sum())
    h2d = (C.sizeof(abi.SpElement) * len(circ.elements) + C.sizeof(abi.SpParam) * len(circ.params) + 8 * n
           + 4 * len(circ.elements))
    d2h = N * (8 * n + 4 + 1)
    t = torch.tensor([e2e_s], dtype=torch.float64, device=dev)
    if dist is not None:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    e2e_value = e2e_conv * world / float(t.item())

    # rooflines of the headline's kernels (average launch durations, live)
    fp64_peak = read_profile_number("pipe_peaks_gb300.txt", "fp64_tflops") or 1.25
    fp32_peak = read_profile_number("pipe_peaks_gb300.txt", "fp32_tflops") or 73.3
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except (OSError, ValueError):
        peaks = {}
    hbm_peak = peaks.get("hbm_gbs", 6770.8)
    bf16_peak = peaks.get("bf16_tflops", 1892.9)
    kavg = {k: v[1] / max(v[0], 1) for k, v in head["prof"].items()}
    m_mos = sum(1 for e in circ.elements if e["kind"] in (abi.SP_EL_NMOS, abi.SP_EL_PMOS))
    nnz = structural_nnz(circ)
    rooflines = {}
    if "newton_primary_mixed_spec" in kavg:
        # FP64 instructions per sample-iteration of the mixed specialised kernel: per MOSFET the
        # drain current (8) and its two KCL terms, per resistor 4, per source 2-3, the update n
        ms = kavg["newton_primary_mixed_spec"]
        kinds = [e["kind"] for e in circ.elements]
        per_it = (10 * m_mos + 4 * kinds.count(abi.SP_EL_R) + 3 * kinds.count(abi.SP_EL_V)
                  + 2 * kinds.count(abi.SP_EL_I) + n)
        f64 = per_it * head["iters"] * N
        a = f64 / (ms * 1e-3) / 1e12
        pk = fp64_peak / 2  # FP64 instructions per second (an FMA counts two flops of the measured peak)
        rooflines["newton_primary_mixed_spec"] = {
            "bound": "fp64", "achieved": a, "peak": pk, "unit": "T FP64 instructions/s", "frac": a / pk,
            "traffic": read_profile_number("newton_spec_mixed_opamp.md", "dram_bytes_per_launch"),
            "avg_launch_ms": ms, "fp64_instructions_per_launch": f64,
            "peak_source": "FP64 pipe throughput measured on this pool's GB300 (profiles/pipe_peaks_gb300.txt)"}
    if "mlp_warm_start" in kavg:
        ms = kavg["mlp_warm_start"]
        ni, H, nl = ws.mlp.n_in, ws.mlp.n_hidden, ws.mlp.n_layers
        fl = 2.0 * (ni * H + (nl - 1) * H * H + H * n) * N
        a = fl / (ms * 1e-3) / 1e12
        rooflines["mlp_warm_start"] = {"bound": "tensor", "achieved": a, "peak": bf16_peak, "unit": "TFLOP/s",
                                       "frac": a / bf16_peak, "traffic": None, "avg_launch_ms": ms,
                                       "flops_per_launch": fl, "peak_source": "bf16_tflops of MEASURED_PEAKS.json"}
    if "draw_params" in kavg:
        ms = kavg["draw_params"]
        by = 8 * (len(circ.params) + derived_slots(circ)) * N
        a = by / (ms * 1e-3) / 1e9
        rooflines["draw_params"] = {"bound": "hbm", "achieved": a, "peak": hbm_peak, "unit": "GB/s",
                                    "frac": a / hbm_peak,
                                    "traffic": read_profile_number("draw_params_opamp.md", "dram_bytes_per_launch"),
                                    "avg_launch_ms": ms, "bytes_per_launch": by,
                                    "note": "integer-ALU bound (correctly rounded ln/cos in fixed point; ncu ALU pipe "
                                            "64 % busy), not HBM: its outputs stay in L2 for the next kernels"}
    dominant = max(kavg, key=kavg.get) if kavg else None
    roofline = rooflines.get(dominant) or next(iter(rooflines.values()), None)
    if roofline is not None:
        roofline = dict(roofline, kernel=dominant)

    def event_ms(fn):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        flush.fill_(0.5)
        e0.record()
        fn()
        e1.record()
        e1.synchronize()
        return e0.elapsed_time(e1)

    # workload 3: 4,096 RC-diode ladder transients (adaptive TR-BDF2), one run per precision
    config3 = None
    if not args.no_transient and rank == 0:
        import oracle
        count3 = 4096
        config3 = {"instances": count3, "sections": "8..512", "tstop_s": 100e-9}
        for name, prec in (("mixed", abi.SP_PREC_MIXED), ("plain_fp64", abi.SP_PREC_FP64)):
            lc = abi.ladder_config(precision=prec, num_probe=0)
            ld = lc.max_sections + 2
            lx = torch.empty((count3, ld), dtype=torch.float64, device=dev)
            li = [torch.empty(count3, dtype=torch.int32, device=dev) for _ in range(4)]
            lst = torch.empty(count3, dtype=torch.uint8, device=dev)
            ctx.ladder_transient_device(lc, SEED, 256, lx, *li, lst, stream=stream)  # warm-up
            torch.cuda.synchronize()
            ms = event_ms(lambda: ctx.ladder_transient_device(lc, SEED, count3, lx, *li, lst, stream=stream))
            acc = li[1].cpu().numpy()
            stages = 2.0 * float(acc.sum())
            config3[name] = {"ms": ms, "transients_per_s": count3 / (ms / 1e3), "stage_solves_per_s": stages / (ms / 1e3),
                             "newton_per_stage": float(li[3].cpu().numpy().sum()) / stages,
                             "accepted_steps_mean": float(acc.mean()), "rejected_steps_mean": float(li[2].float().mean()),
                             "converged_fraction": float((lst == 0).float().mean())}
        sample3 = 64
        with oracle.math_mode("cr"):
            t0 = time.perf_counter()
            o3 = oracle.ladder_transient(abi.ladder_config(num_probe=0), SEED, sample3)
            dt3 = time.perf_counter() - t0
        config3["cpu_oracle"] = {"transients_per_s": sample3 / dt3, "cores": os.cpu_count() or 1,
                                 "sample": f"{sample3} ladders (instances 0..{sample3 - 1}), FP64, all host threads"}
        config3["speedup_mixed_vs_plain_fp64"] = config3["mixed"]["transients_per_s"] / config3["plain_fp64"]["transients_per_s"]

    # AC small-signal sweep of the op-amp Monte Carlo (the next row after the DC sweep)
    ac_report = None
    if not args.no_ac and rank == 0:
        from spicier_gb300.api import Context as _Ctx
        acfg = {}
        for name, prec in (("mixed", abi.SP_PREC_MIXED), ("fp64", abi.SP_PREC_FP64)):
            cfg_ac = abi.ac_config(10.0, 1e9, 10, abi.SP_AC_DEC, [circ.node("out")], precision=prec)
            nf = len(_Ctx.ac_frequencies(cfg_ac))
            pd = torch.empty((N, nf, 1, 2), dtype=torch.float64, device=dev)
            sd = torch.empty(N, dtype=torch.uint8, device=dev)
            run_ac = lambda: ctx.ac_sweep_device(topo, cfg_mixed, cfg_ac, SEED, N, pd, sd, stream=stream)
            run_ac()
            ms = min(event_ms(run_ac) for _ in range(3))
            ok = float(((sd & 0x0F) == 0).float().mean().item())
            acfg[name] = {"ms": ms, "complex_solves_per_s": N * nf / (ms * 1e-3), "converged_fraction": ok}
        ac_report = {"samples": N, "frequencies": nf, "sweep": "10 Hz .. 1 GHz, 10 per decade",
                     "probe": "out", "dc": "mixed + nodeset, inside the timed call", **acfg}

    # BSIM3 (LEVEL=49) devices: batched evaluation, then a Monte Carlo DC sweep of a BSIM3 circuit
    b3_report = None
    if not args.no_bsim3 and rank == 0:
        from spicier_gb300 import configs as _cfgs
        from spicier_gb300.circuit import BSIM3_DEFAULTS
        nb = 1 << 22
        gen = torch.Generator(device=dev)
        gen.manual_seed(SEED)
        col = {k: i for i, k in enumerate(abi.BSIM3_CARD)}
        card = torch.tensor([BSIM3_DEFAULTS[False][k] for k in abi.BSIM3_CARD], dtype=torch.float64,
                            device=dev).repeat(nb, 1)
        u = lambda: torch.rand(nb, generator=gen, device=dev, dtype=torch.float64)
        card[:, col["vth0"]] = 0.3 + 0.3 * u()
        card[:, col["l"]] = 50e-9 + 950e-9 * u()
        card[:, col["u0"]] = 500.0 + 300.0 * u()
        bias = torch.stack([1.8 * u(), -0.5 + 2.3 * u(), -1.0 * u()], dim=1).contiguous()
        bout = torch.empty((nb, 6), dtype=torch.float64, device=dev)
        breg = torch.empty(nb, dtype=torch.uint8, device=dev)
        run_b3 = lambda: ctx.bsim3_eval_device(False, card, bias, bout, breg, stream=stream)
        run_b3()
        ms_b3 = min(event_ms(run_b3) for _ in range(5))
        bytes_b3 = nb * (abi.SP_B3_CARD * 8 + 3 * 8 + 6 * 8 + 1)
        gbs_b3 = bytes_b3 / (ms_b3 * 1e-3) / 1e9
        b3_report = {"evaluation": {"devices": nb, "ms": ms_b3, "devices_per_s": nb / (ms_b3 * 1e-3),
                                    "regions": [int((breg == k).sum()) for k in range(3)],
                                    "roofline": {"bound": "hbm", "achieved": gbs_b3, "peak": hbm_peak, "unit": "GB/s",
                                                 "frac": gbs_b3 / hbm_peak,
                                                 "bytes_per_device": bytes_b3 // nb,
                                                 "note": "FP64-pipe bound, not HBM: ~20 divides and 5 square "
                                                         "roots per device for its constants and evaluation"}}}
        bc = _cfgs.bsim3_cmos_chain()
        btopo = ctx.topology(bc)
        bx = torch.empty((N, bc.n), dtype=torch.float64, device=dev)
        bit = torch.empty(N, dtype=torch.int32, device=dev)
        bst = torch.empty(N, dtype=torch.uint8, device=dev)
        for name, prec in (("mixed", abi.SP_PREC_MIXED), ("plain_fp64", abi.SP_PREC_FP64)):
            bcfg = abi.newton_config(precision=prec)
            run_dc = lambda: ctx.newton_dc_device(btopo, bcfg, SEED, N, bx, iters=bit, status=bst, stream=stream)
            run_dc()
            ms = min(event_ms(run_dc) for _ in range(3))
            b3_report[name] = {"ms": ms, "solves_per_s": N / (ms * 1e-3),
                               "iters_per_solve": float(bit.double().mean()),
                               "converged_fraction": float(((bst & 0x0F) == 0).float().mean())}
        b3_report["sweep"] = {"circuit": "bsim3_cmos_chain (CMOS inverter + common-source stage, 3 BSIM3 devices)",
                              "samples": N, "mna_size": bc.n, "start": "nodeset"}
        b3_report["speedup_mixed_vs_plain_fp64"] = b3_report["mixed"]["solves_per_s"] / b3_report["plain_fp64"]["solves_per_s"]

    # workload 5: 256 power-grid corners (Newton + GMRES(30) + Jacobi)
    config5 = None
    if not args.no_grid and rank == 0:
        import oracle
        count5 = 256
        config5 = {"corners": count5, "mesh": "64x64 + VDD branch (4097 unknowns)", "sinks": 512}
        for name, prec in (("mixed", abi.SP_PREC_MIXED), ("plain_fp64", abi.SP_PREC_FP64)):
            gc = abi.grid_config(precision=prec)
            nG = gc.rows * gc.cols + 1
            gx = torch.empty((count5, nG), dtype=torch.float64, device=dev)
            gnw, gkr = (torch.empty(count5, dtype=torch.int32, device=dev) for _ in range(2))
            gst = torch.empty(count5, dtype=torch.uint8, device=dev)
            grs = torch.empty(count5, dtype=torch.float64, device=dev)
            ctx.grid_solve_device(gc, SEED, 8, gx, gnw, gkr, gst, grs, stream=stream)  # warm-up
            torch.cuda.synchronize()
            ms = event_ms(lambda: ctx.grid_solve_device(gc, SEED, count5, gx, gnw, gkr, gst, grs, stream=stream))
            nwt = gnw.cpu().numpy()
            config5[name] = {"ms": ms, "corners_per_s": count5 / (ms / 1e3),
                             "newton_solves_per_s": float(nwt.sum()) / (ms / 1e3), "newton_mean": float(nwt.mean()),
                             "krylov_mean": float(gkr.float().mean()), "max_kcl_residual_A": float(grs.max()),
                             "converged_fraction": float((gst == 0).float().mean())}
        sample5 = 4
        t0 = time.perf_counter()
        oracle.grid_solve(abi.grid_config(), SEED, sample5)
        dt5 = time.perf_counter() - t0
        config5["cpu_oracle"] = {"corners_per_s": sample5 / dt5, "cores": min(sample5, os.cpu_count() or 1),
                                 "sample": f"{sample5} corners (one per host thread), FP64"}

    # config 4: a 10-input network (the workload's stated MLP) on 262,144 samples
    config4 = None
    if not args.no_config4 and rank == 0:
        N4 = 262144
        ws10 = WarmStart(ctx, circ, n_inputs=10, seed=5)
        rep10 = ws10.train(topo, seed=TRAIN_SEED, samples=args.train_samples, epochs=16, batch=4096, lr=2e-3)
        x4 = torch.empty((N4, n), dtype=torch.float64, device=dev)
        it4 = torch.empty(N4, dtype=torch.int32, device=dev)
        st4 = torch.empty(N4, dtype=torch.uint8, device=dev)
        res4 = {}
        for name, run in (("learned", lambda f: ws10.sweep_device(topo, cfg_mixed, SEED, N4, x4, first=f, iters=it4,
                                                                  status=st4, stream=stream)),
                          ("cold_nodeset", lambda f: ctx.newton_dc_device(topo, cfg_mixed, SEED, N4, x4, first=f,
                                                                          iters=it4, status=st4, stream=stream))):
            for w in range(3):
                run(w * N4)
            torch.cuda.synchronize()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            tot, conv, its, fb = 0.0, 0, 0, 0
            for k in range(5):
                flush.fill_(float(k))
                e0.record()
                run((3 + k) * N4)
                e1.record()
                e1.synchronize()
                tot += e0.elapsed_time(e1)
                s = st4.cpu().numpy()
                conv += int(((s & 0x0F) == 0).sum())
                its += int(it4.sum().item())
                fb += int(((s & (abi.SP_ST_FLAG_COLD | abi.SP_ST_FLAG_GMIN | abi.SP_ST_FLAG_SOURCE)) != 0).sum())
            res4[name] = {"solves_per_s": conv / (tot / 1e3), "iters_per_solve": its / (5 * N4),
                          "fallback_rate": fb / (5 * N4), "converged_fraction": conv / (5 * N4)}
        config4 = {"samples": N4, "inputs": rep10.input_labels, "train_seconds": rep10.seconds, **res4,
                   "speedup_vs_cold": res4["learned"]["solves_per_s"] / res4["cold_nodeset"]["solves_per_s"]}

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        r, dt, _, done = cpu_baseline(circ, N, min_seconds=10.0)
        cpu = {"value": r, "unit": UNIT, "cores": os.cpu_count() or 1, "kind": "port",
               "sample": f"{done} op-amp Monte Carlo samples ({N}-sample chunks), plain FP64 Newton from the "
                         f"nodeset, {dt:.1f} s on all host threads"}

    if rank == 0:
        def arm(r):
            return {"value": rate(r), "unit": UNIT, "ms_per_step": r["ms"] / r["steps"],
                    "iters_per_solve": r["iters"], "max_resid_A": r["rmax"],
                    "kernel_ms": {k: v[1] / max(v[0], 1) for k, v in r["prof"].items()}}

        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": head["ms"] / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64/f32/bf16",
            "data": "synthetic (hash-RNG Monte Carlo draws on device, seed 1; network trained on seed 7)",
            "config": {"workload": "miller_opamp_mc_dc", "samples_per_step": N, "mna_size": n,
                       "precision": "mixed (FP32 sparse LU, FP64 residual/update/models) + BF16 warm start",
                       "warm_start": f"MLP {ws.mlp.n_in}->{ws.mlp.n_layers}x{ws.mlp.n_hidden} GELU->{n} "
                                     "(tcgen05, TMEM) + FP64-fitted linear term",
                       "tolerances": "reltol 1e-3, vntol 1e-6 V, abstol 1e-12 A",
                       "l2": "flushed between timed steps (256 MiB write)",
                       "parallelism": "replicas" if world > 1 else "single GPU"},
            "plain_fp64": arm(plain),
            "speedup_vs_plain_fp64": value / plain_value if plain_value else None,
            "iters_per_solve": head["iters"], "max_resid_A": head["rmax"],
            "converged_fraction": head["conv"] / (N * args.steps * world),
            "status_counts": {str(k): v for k, v in head["flags"].items()},
            "ablations": {k: arm(v) for k, v in ablations.items()},
            "setup": {"specialise_s": spec_s, "train_s": rep.seconds, "train_samples": rep.samples,
                      "train_loss_first_last": [rep.epoch_loss[0], rep.epoch_loss[-1]]},
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
            "roofline": roofline, "rooflines": rooflines,
            "kernel_ms": kavg,
            "gpu_launches": sum(v[0] for v in head["prof"].values()),
            "clocks": head["clocks"],
            "config4": config4,
            "config3_ladder_transient": config3,
            "config5_power_grid": config5,
            "ac_sweep": ac_report,
            "bsim3": b3_report,
            "cpu_baseline": cpu,
        }
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
