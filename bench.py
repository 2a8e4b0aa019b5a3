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
    and the same FP64 arithmetic in the topology-specialised kernel;
  * ablation: mixed precision from the nodeset;
  * workload 1 (1,024-sample common-source NMOS: latency, graph replay),
    workload 3 (4,096 RC-diode ladder transients), workload 4 (the stated
    10 -> 3x256 network on 262,144 samples against its linear term alone and a
    cold start), workload 5 (256 power-grid corners), AC and BSIM3 reports;
  * --impl reference: the reference algorithm's CPU implementation (the C++
    restatement; Spicier's Rust cannot be built here) on all host cores.
One JSON line on stdout (rank 0), ending with a compact "summary".
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
TOLERANCES = "reltol 1e-3, vntol 1e-6 V, abstol 1e-12 A"


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


def workload_config(samples, mna_size):
    """The workload both arms run (the line's `config`): what is solved, not how."""
    return {"workload": "miller_opamp_mc_dc", "circuit": "two-stage Miller op-amp, unity-gain buffer",
            "samples_per_step": samples, "mna_size": mna_size, "seed": SEED, "tolerances": TOLERANCES,
            "draws": "hash RNG (VIN uniform 1.0-2.3 V; per-device VTO, KP Gaussian)",
            "l2": "flushed between timed steps (256 MiB write)"}


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


# ---------------------------------------------------------------------------
# Pipe peaks: MEASURED_PEAKS.json holds HBM and BF16 tensor figures only.  The
# Newton kernels are bound by the FP64 pipe and the parameter draws by integer
# issue, so the bench measures those denominators itself with a small probe
# (independent dependency chains per thread) compiled for this GPU.
PIPE_PROBE = r"""
#include <cuda_runtime.h>
template <class T>
__global__ void fma_chain(T* out, int iters, T a, T b) {
    T x0 = threadIdx.x, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
    for (int i = 0; i < iters; ++i) {
        x0 = x0 * a + b; x1 = x1 * a + b; x2 = x2 * a + b; x3 = x3 * a + b;
        x4 = x4 * a + b; x5 = x5 * a + b; x6 = x6 * a + b; x7 = x7 * a + b;
    }
    out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}
// three-input logic operations mixing the eight values: the integer ALU
// pipe alone.  nvcc 13.0 emits four ALU instructions per iteration for these
// eight lines (ncu: smsp__inst_executed_pipe_alu.sum = 4 x iterations x
// threads / 32, with the ALU pipe at 99.98 % of its peak), so the rate below
// counts four instructions per iteration and thread
__global__ void alu_chain(unsigned* out, int iters, unsigned a, unsigned b) {
    unsigned x0 = threadIdx.x ^ b, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6,
             x7 = x0 + 7;
    for (int i = 0; i < iters; ++i) {
        x0 = (x0 ^ x1) | a; x1 = (x1 ^ x2) | a; x2 = (x2 ^ x3) | a; x3 = (x3 ^ x4) | a;
        x4 = (x4 ^ x5) | a; x5 = (x5 ^ x6) | a; x6 = (x6 ^ x7) | a; x7 = (x7 ^ x0) | a;
    }
    out[blockIdx.x * blockDim.x + threadIdx.x] = x0 ^ x1 ^ x2 ^ x3 ^ x4 ^ x5 ^ x6 ^ x7;
}
template <class K, class... A>
static float timed(K k, int blocks, A... a) {
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    k<<<blocks, 256>>>(a...);
    cudaEventRecord(e0);
    k<<<blocks, 256>>>(a...);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return ms;
}
// out: FP64 TFLOP/s, FP32 TFLOP/s (an FMA counts two), integer ALU T instructions/s (per thread)
extern "C" int pipe_peaks(double* out) {
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, 0);
    const int blocks = sms * 8, threads = 256;
    void* buf = nullptr;
    if (cudaMalloc(&buf, sizeof(double) * blocks * threads) != cudaSuccess) return 1;
    const int i64 = 2048, i32 = 65536, ialu = 65536;
    float ms = timed(fma_chain<double>, blocks, (double*)buf, i64, 0.999, 0.001);
    out[0] = 2.0 * 8 * (double)i64 * blocks * threads / (ms * 1e9);
    ms = timed(fma_chain<float>, blocks, (float*)buf, i32, 0.999f, 0.001f);
    out[1] = 2.0 * 8 * (double)i32 * blocks * threads / (ms * 1e9);
    ms = timed(alu_chain, blocks, (unsigned*)buf, ialu, 0x9e3779b9u, 0x7f4a7c15u);
    out[2] = 4.0 * (double)ialu * blocks * threads / (ms * 1e9);
    cudaFree(buf);
    return cudaGetLastError() == cudaSuccess ? 0 : 2;
}
"""


def measure_pipe_peaks():
    """Best of three probe runs: {"fp64_tflops", "fp32_tflops", "int_alu_tops"}, or {} without nvcc."""
    nvcc = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")
    d = tempfile.mkdtemp(prefix="pipe_peaks_")
    src, lib = os.path.join(d, "probe.cu"), os.path.join(d, "probe.so")
    open(src, "w").write(PIPE_PROBE)
    r = subprocess.run([nvcc, "-shared", "-Xcompiler", "-fPIC", "-O3", "-gencode", "arch=compute_103a,code=sm_103a",
                        "-o", lib, src], capture_output=True, text=True)
    if r.returncode != 0:
        return {}
    f = C.CDLL(lib).pipe_peaks
    f.restype, f.argtypes = C.c_int, [C.POINTER(C.c_double)]
    best = [0.0, 0.0, 0.0]
    for _ in range(3):
        out = (C.c_double * 3)()
        if f(out) == 0:
            best = [max(b, v) for b, v in zip(best, out)]
    return {"fp64_tflops": best[0], "fp32_tflops": best[1], "int_alu_tops": best[2],
            "probe": "independent FMA / logic-op chains, 8 per thread, 8 blocks of 256 per SM (bench.py PIPE_PROBE)"}


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
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": 0, "host_cores": cores,
        "steps": steps, "warmup": args.warmup, "ms_per_step": 1e3 * total_t / steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": workload_config(sample, circ.n),
        "arm": "plain FP64 Newton from the nodeset (solve_newton_raphson restated in C++), one task per sample on "
               "all host threads",
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": f"{sample} op-amp Monte Carlo samples per step, plain FP64 Newton from the nodeset"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def cublas_lu_comparator(ctx, sizes=(12, 50, 100), batch=65535, reps=5):
    """The reference's own GPU path for BatchedLuSolver::solve_batch: cuBLAS
    cublasDgetrfBatched + cublasDgetrsBatched over a pointer array
    (crates/spicier-backend-cuda/src/batched_lu.rs:411-470), against
    sp_solve_batch_device on the same column-major FP64 systems, device
    buffers only, CUDA events around each.  Returns {n: {...}} or a reason."""
    import torch
    cands = [os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "lib64", "libcublas.so"), "libcublas.so.13",
             "libcublas.so"]
    cb = None
    for c in cands:
        try:
            cb = C.CDLL(c)
            break
        except OSError:
            continue
    if cb is None:
        return {"unavailable": "libcublas not found"}
    vp = C.c_void_p
    handle = vp()
    if cb.cublasCreate_v2(C.byref(handle)) != 0:
        return {"unavailable": "cublasCreate failed"}
    stream = torch.cuda.current_stream()
    cb.cublasSetStream_v2(handle, vp(stream.cuda_stream))
    cb.cublasDgetrfBatched.argtypes = [vp, C.c_int, vp, C.c_int, vp, vp, C.c_int]
    cb.cublasDgetrsBatched.argtypes = [vp, C.c_int, C.c_int, C.c_int, vp, C.c_int, vp, vp, C.c_int,
                                       C.POINTER(C.c_int), C.c_int]
    dev = torch.device("cuda", ctx.device)
    gen = torch.Generator(device=dev)
    gen.manual_seed(SEED)
    out = {}

    def ev(fn):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        fn()
        e1.record()
        e1.synchronize()
        return e0.elapsed_time(e1)

    for n in sizes:
        # diagonally dominant random systems (column-major [batch][n][n] is the transposed row-major array)
        A = torch.rand((batch, n, n), dtype=torch.float64, device=dev, generator=gen) - 0.5
        A += n * torch.eye(n, dtype=torch.float64, device=dev)
        b = torch.rand((batch, n), dtype=torch.float64, device=dev, generator=gen)
        work = torch.empty_like(A)
        xb = torch.empty_like(b)
        ptr_a = (work.data_ptr() + torch.arange(batch, device=dev, dtype=torch.int64) * (n * n * 8)).contiguous()
        ptr_b = (xb.data_ptr() + torch.arange(batch, device=dev, dtype=torch.int64) * (n * 8)).contiguous()
        piv = torch.empty((batch, n), dtype=torch.int32, device=dev)
        info = torch.empty(batch, dtype=torch.int32, device=dev)
        hinfo = C.c_int(0)
        sol = torch.empty_like(b)
        sing = torch.empty(batch, dtype=torch.uint8, device=dev)

        def run_cublas():
            work.copy_(A)
            xb.copy_(b)
            cb.cublasDgetrfBatched(handle, n, vp(ptr_a.data_ptr()), n, vp(piv.data_ptr()), vp(info.data_ptr()), batch)
            cb.cublasDgetrsBatched(handle, 0, n, 1, vp(ptr_a.data_ptr()), n, vp(piv.data_ptr()), vp(ptr_b.data_ptr()),
                                   n, C.byref(hinfo), batch)

        def run_copy():
            work.copy_(A)
            xb.copy_(b)

        def run_ours():
            ctx.solve_batch_device(A, b, n, batch, sol, sing, stream=stream.cuda_stream)

        run_cublas()
        run_ours()
        torch.cuda.synchronize()
        t_copy = min(ev(run_copy) for _ in range(reps))
        t_cb = min(ev(run_cublas) for _ in range(reps)) - t_copy  # cuBLAS factors in place: copies excluded
        t_ours = min(ev(run_ours) for _ in range(reps))
        rel = float(((sol - xb).abs() / xb.abs().clamp_min(1e-300)).max())
        out[str(n)] = {"batch": batch, "ours_ms": t_ours, "cublas_getrf_getrs_ms": t_cb,
                       "speedup": t_cb / t_ours if t_ours > 0 else None, "max_rel_diff": rel,
                       "ours_systems_per_s": batch / (t_ours * 1e-3)}
        del A, b, work, xb, ptr_a, ptr_b, piv, info, sol, sing
    cb.cublasDestroy_v2(handle)
    return out


def launch_ranks(args):
    """--gpus N without a launcher: start N ranks of this script under
    torch.distributed.run on 127.0.0.1 and pass rank 0's line through."""
    import socket
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", f"--nproc-per-node={args.gpus}",
           "--master-addr", "127.0.0.1", f"--master-port={port}", os.path.abspath(__file__)] + sys.argv[1:]
    return subprocess.run(cmd).returncode


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=300)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--samples", type=int, default=65536)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-config1", action="store_true", help="skip the 1,024-sample CS-NMOS (workload 1) report")
    ap.add_argument("--no-config4", action="store_true")
    ap.add_argument("--no-transient", action="store_true", help="skip the ladder-transient (workload 3) report")
    ap.add_argument("--no-grid", action="store_true", help="skip the power-grid (workload 5) report")
    ap.add_argument("--no-ac", action="store_true", help="skip the AC small-signal sweep report")
    ap.add_argument("--no-bsim3", action="store_true", help="skip the BSIM3 evaluation / sweep report")
    ap.add_argument("--no-oracle-check", action="store_true", help="skip the error against the FP64 oracle")
    ap.add_argument("--no-lu-comparator", action="store_true",
                    help="skip the batched LU against the reference's cuBLAS getrf/getrs calls")
    ap.add_argument("--train-samples", type=int, default=1 << 20)
    ap.add_argument("--no-ablations", action="store_true", help="skip the mixed-from-nodeset and FP64-specialised arms")
    ap.add_argument("--mlp-hidden", type=int, default=128, help="hidden width of the headline warm-start network")
    ap.add_argument("--mlp-layers", type=int, default=3, help="hidden layers of the headline warm-start network")
    ap.add_argument("--pipe-peaks", action="store_true", help="only measure and print the FP64/FP32/ALU pipe peaks")
    ap.add_argument("--warm-start", default="auto", choices=["auto", "network", "linear"],
                    help="learned warm start of the headline: the network (tcgen05) with its linear term, the "
                         "linear term alone (evaluated in the draw kernel), or the faster of the two (both timed)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    if args.impl == "reference":
        return run_reference(args)
    if args.gpus > 1 and "WORLD_SIZE" not in os.environ:
        return launch_ranks(args)

    import numpy as np
    import torch

    import spicier_gb300 as sg
    from spicier_gb300 import abi, configs
    from spicier_gb300._lib import check, load
    from spicier_gb300.learned import WarmStart, random_slots

    rank, world, local = env_int("RANK", 0), env_int("WORLD_SIZE", 1), env_int("LOCAL_RANK", 0)
    torch.cuda.set_device(local)
    if args.pipe_peaks:
        print(json.dumps(measure_pipe_peaks()), flush=True)
        return 0
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    def barrier():
        torch.cuda.synchronize()
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()

    pipe = measure_pipe_peaks() if rank == 0 else {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
        peak_src = "MEASURED_PEAKS.json"
    except (OSError, ValueError):
        peaks, peak_src = {}, "fallback"
    hbm_peak = peaks.get("hbm_gbs", 6800.0)
    bf16_peak = peaks.get("bf16_tflops", 1900.0)
    fp64_peak = pipe.get("fp64_tflops") or 1.25
    alu_peak = pipe.get("int_alu_tops") or None

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
        total_ms, conv, it_sum, flags = 0.0, 0, 0, {}
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
        last_first = base_index + (args.warmup + steps - 1) * N
        step(last_first, resid)  # untimed: residual of the last timed sweep
        ok = (status & 0x0F) == 0
        rmax = float(resid[ok].max().item()) if bool(ok.any()) else 0.0
        t = torch.tensor([total_ms], dtype=torch.float64, device=dev)
        c = torch.tensor([conv], dtype=torch.float64, device=dev)
        if dist is not None:
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
            dist.all_reduce(c, op=dist.ReduceOp.SUM)
        return dict(ms=float(t.item()), conv=int(c.item()), iters=it_sum / (N * steps), rmax=rmax, prof=prof,
                    clocks=clk, flags=flags, steps=steps, last_first=last_first)

    def rate(r):
        return r["conv"] / (r["ms"] / 1e3)

    plain = timed(plain_step, args.steps)
    # both learned warm starts are timed (unless one is forced); the headline is the faster
    variants = {}
    for vname in ("network", "linear"):
        if args.warm_start in ("auto", vname):
            ws.use_network(vname == "network")
            variants[vname] = timed(learned_step, args.steps, clocks=Clocks(local))
    head_name = max(variants, key=lambda k: rate(variants[k]))
    head = variants[head_name]
    ws.use_network(head_name == "network")
    learned_step(head["last_first"])  # untimed: x holds the headline's last timed sweep again
    # error of the headline's last timed sweep against the FP64 oracle (same
    # draws: the oracle's correctly rounded mode), on a sample of it (untimed)
    oracle_err = None
    if rank == 0 and not args.no_oracle_check:
        import oracle
        S = min(N, 4096)
        xg = x[:S].cpu().numpy()
        stg = status[:S].cpu().numpy()
        with oracle.math_mode("cr"):
            xo, _io, so, _ = oracle.newton_dc(circ, abi.newton_config(), SEED, S, first=head["last_first"])
        nn = circ.num_nodes
        tol = np.empty_like(xo)
        tol[:, :nn] = 1e-3 * np.abs(xo[:, :nn]) + 1e-6
        tol[:, nn:] = 1e-3 * np.abs(xo[:, nn:]) + 1e-12
        both = ((stg & 0x0F) == 0) & ((so & 0x0F) == 0)
        units = np.abs(xg - xo)[both] / tol[both]
        rel = np.abs(xg - xo)[both] / np.maximum(np.abs(xo[both]), 1e-12)
        oracle_err = {"samples": S, "first_index": head["last_first"], "compared": int(both.sum()),
                      "max_tol_units": float(units.max()), "max_rel": float(rel.max()),
                      "oracle": "FP64 Newton (solve_newton_raphson restated), same device draws"}
    ablations = {}
    if not args.no_ablations:
        abl_steps = max(3, args.steps // 5)
        ablations["mixed_nodeset"] = timed(mixed_nodeset_step, abl_steps)
        ctx.specialize(topo, abi.SP_PREC_FP64, True)
        ablations["fp64_specialised_nodeset"] = timed(plain_step, max(3, args.steps // 2))
        ctx.specialize(topo, abi.SP_PREC_FP64, False)

    value, plain_value = rate(head), rate(plain)
    fp64_spec_value = rate(ablations["fp64_specialised_nodeset"]) if "fp64_specialised_nodeset" in ablations else None
    faster_fp64 = max(plain_value, fp64_spec_value or 0.0)

    # e2e through the public host-buffer API: the step's inputs are the circuit
    # (kept on the device after the first call, so nothing is copied), the seed
    # and the sweep range; its parameters are drawn on the device inside the
    # timed call; every output (x, iterations, status) is copied back to pinned
    # host memory and the call synchronises.
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
    d2h = N * (8 * n + 4 + 1)
    t = torch.tensor([e2e_s], dtype=torch.float64, device=dev)
    if dist is not None:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    e2e_value = e2e_conv * world / float(t.item())

    # rooflines of the headline's kernels (average launch durations, live)
    kavg = {k: v[1] / max(v[0], 1) for k, v in head["prof"].items()}
    rooflines = {}
    if "newton_primary_mixed_spec" in kavg:
        # the double-float kernel has no FP64 instruction in its iteration and is
        # latency-bound (one sample per thread at this size): its roofline is the
        # issue rate, warp instructions per launch (the committed ncu capture) over
        # the live launch time, against one instruction per clock per SM sub-partition
        ms = kavg["newton_primary_mixed_spec"]
        inst = read_profile_number("newton_spec_mixed_opamp.md", "warp_instructions_per_launch")
        sms = torch.cuda.get_device_properties(dev).multi_processor_count
        clk = (head.get("clocks") or {}).get("sm_max_mhz") or 2070.0
        pk = 4 * sms * clk * 1e6 / 1e12
        if inst:
            a = inst / (ms * 1e-3) / 1e12
            rooflines["newton_primary_mixed_spec"] = {
                "bound": "latency (issue)", "achieved": a, "peak": pk, "unit": "T warp instructions/s",
                "frac": a / pk,
                "traffic": read_profile_number("newton_spec_mixed_opamp.md", "dram_bytes_per_launch"),
                "avg_launch_ms": ms, "warp_instructions_per_launch": inst,
                "peak_source": "4 sub-partitions x SMs x the SM clock seen during the timed region"}
    if "mlp_warm_start" in kavg:
        ms = kavg["mlp_warm_start"]
        ni, H, nl = ws.mlp.n_in, ws.mlp.n_hidden, ws.mlp.n_layers
        fl = 2.0 * (ni * H + (nl - 1) * H * H + H * n) * N
        a = fl / (ms * 1e-3) / 1e12
        rooflines["mlp_warm_start"] = {"bound": "tensor", "achieved": a, "peak": bf16_peak, "unit": "TFLOP/s",
                                       "frac": a / bf16_peak, "traffic": None, "avg_launch_ms": ms,
                                       "flops_per_launch": fl, "peak_source": f"bf16_tflops of {peak_src}"}
    if "draw_params" in kavg:
        ms = kavg["draw_params"]
        # the headline's draw kernel writes the drawn parameters only (the
        # double-float Newton kernel derives its own constants and compiles the
        # fixed ones in)
        by = 8 * sum(1 for row in circ.params if row[0] != abi.SP_DRAW_FIXED) * N
        inst = read_profile_number("draw_params_opamp.md", "alu_warp_instructions_per_sample")
        entry = {"avg_launch_ms": ms, "bytes_per_launch": by,
                 "hbm_frac": by / (ms * 1e-3) / 1e9 / hbm_peak,
                 "traffic": read_profile_number("draw_params_opamp.md", "dram_bytes_per_launch")}
        f64i = read_profile_number("draw_params_opamp.md", "fp64_warp_instructions_per_sample")
        if f64i:
            entry["fp64_frac"] = f64i * 32 * N / (ms * 1e-3) / 1e12 / (fp64_peak / 2)
        if inst and alu_peak:
            a = inst * 32 * N / (ms * 1e-3) / 1e12
            entry.update({"bound": "int_alu", "achieved": a, "peak": alu_peak, "unit": "T ALU instructions/s",
                          "frac": a / alu_peak, "peak_source": "logic-op chains measured live by this bench (instruction count per iteration from ncu)",
                          "note": "integer ALU ops per sample from the committed ncu capture "
                                  "(sm__inst_executed_pipe_alu), times the live launch duration"})
        else:
            entry.update({"bound": "hbm", "achieved": by / (ms * 1e-3) / 1e9, "peak": hbm_peak, "unit": "GB/s",
                          "frac": entry["hbm_frac"]})
        rooflines["draw_params"] = entry
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

    # workload 1: 1,024-sample common-source NMOS, launch-latency bound
    config1 = None
    if not args.no_config1 and rank == 0:
        c1 = configs.cs_nmos_amp()
        t1 = ctx.topology(c1)
        N1 = 1024
        x1 = torch.empty((N1, c1.n), dtype=torch.float64, device=dev)
        i1 = torch.empty(N1, dtype=torch.int32, device=dev)
        s1 = torch.empty(N1, dtype=torch.uint8, device=dev)
        config1 = {"samples": N1, "mna_size": c1.n, "circuit": "common-source NMOS (cs_nmos_amp), 4 Gaussian draws"}
        for name, cfg1 in (("plain_fp64", abi.newton_config(precision=abi.SP_PREC_FP64)),
                           ("mixed", abi.newton_config(precision=abi.SP_PREC_MIXED))):
            run1 = lambda f=0: ctx.newton_dc_device(t1, cfg1, SEED, N1, x1, first=f, iters=i1, status=s1,
                                                    stream=stream)
            for w in range(5):
                run1(w * N1)
            torch.cuda.synchronize()
            lat = sorted(event_ms(lambda: run1(7 * N1)) for _ in range(50))
            med = lat[len(lat) // 2]
            conv1 = int(((s1 & 0x0F) == 0).sum())
            entry = {"latency_ms_median": med, "latency_ms_min": lat[0], "solves_per_s": conv1 / (med * 1e-3),
                     "converged": conv1, "iters_per_solve": float(i1.double().mean())}
            # the same call captured once in a CUDA graph and replayed
            try:
                g = torch.cuda.CUDAGraph()
                s = torch.cuda.Stream()
                with torch.cuda.graph(g, stream=s):  # ends the capture on every exit path
                    ctx.newton_dc_device(t1, cfg1, SEED, N1, x1, first=9 * N1, iters=i1, status=s1,
                                         stream=s.cuda_stream)
                g.replay()
                torch.cuda.synchronize()
                glat = sorted(event_ms(g.replay) for _ in range(50))
                entry["graph_replay_ms_median"] = glat[len(glat) // 2]
                entry["graph_solves_per_s"] = int(((s1 & 0x0F) == 0).sum()) / (glat[len(glat) // 2] * 1e-3)
            except Exception as exc:  # capture is an optimisation; report why it did not run
                entry["graph_replay"] = f"not captured: {type(exc).__name__}: {exc}"[:160]
            config1[name] = entry
        # the reference algorithm on all host cores, same 1,024 samples
        r1, dt1, _c, done1 = cpu_baseline(c1, N1, min_seconds=2.0)
        config1["cpu_oracle"] = {"solves_per_s": r1, "cores": os.cpu_count() or 1,
                                 "sample": f"{done1} samples in {N1}-sample chunks, plain FP64"}
        t1.close()

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
            ln = li[0].cpu().numpy().astype(np.float64) - 2  # sections N per instance
            acc = li[1].cpu().numpy()
            newton = float(li[3].cpu().numpy().sum())
            stages = 2.0 * float(acc.sum())
            # FP64 work per ladder node and Newton iteration (the workload's algorithmic count):
            # the diode exponential (~20) + 25 for the limiter, stamps, elimination and test
            node_its = float((li[3].cpu().numpy().astype(np.float64) * ln).sum())  # node x Newton iterations
            fl = 45.0 * node_its
            a = fl / (ms * 1e-3) / 1e12
            config3[name] = {"ms": ms, "transients_per_s": count3 / (ms / 1e3), "stage_solves_per_s": stages / (ms / 1e3),
                             "newton_per_stage": newton / stages,
                             "accepted_steps_mean": float(acc.mean()), "rejected_steps_mean": float(li[2].float().mean()),
                             "converged_fraction": float((lst == 0).float().mean()),
                             "roofline": {"bound": "fp64", "achieved": a, "peak": fp64_peak, "unit": "TFLOP/s",
                                          "frac": a / fp64_peak, "flops": fl,
                                          "per_unit": "45 FP64 flops per ladder node per Newton iteration",
                                          "note": "latency of the serial step chain (a warp per ladder) binds, "
                                                  "not the pipe"}}
        sample3 = 64
        with oracle.math_mode("cr"):
            t0 = time.perf_counter()
            oracle.ladder_transient(abi.ladder_config(num_probe=0), SEED, sample3)
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
            kry = float(gkr.cpu().numpy().astype(np.float64).sum())
            # algorithmic bytes per GMRES(30) iteration and instance: the 5-point stencil's
            # values + column indices (nnz 4-byte values and indices), the MGS reads of
            # k+1 basis vectors (k = 15 on average) and the new vector written, 4-byte
            # elements in the mixed mode and 8-byte in FP64
            eb = 4 if prec == abi.SP_PREC_MIXED else 8
            nnz = 5 * gc.rows * gc.cols + 2 * gc.num_sinks
            per_it = nnz * 8 + 2 * eb * nG * 16 + eb * nG * 2
            by = kry * per_it
            a = by / (ms * 1e-3) / 1e9
            config5[name] = {"ms": ms, "corners_per_s": count5 / (ms / 1e3),
                             "newton_solves_per_s": float(nwt.sum()) / (ms / 1e3), "newton_mean": float(nwt.mean()),
                             "krylov_mean": kry / count5, "max_kcl_residual_A": float(grs.max()),
                             "converged_fraction": float((gst == 0).float().mean()),
                             "roofline": {"bound": "hbm", "achieved": a, "peak": hbm_peak, "unit": "GB/s",
                                          "frac": a / hbm_peak, "bytes": by,
                                          "per_unit": f"{per_it} B per GMRES iteration and corner"}}
        sample5 = 4
        t0 = time.perf_counter()
        oracle.grid_solve(abi.grid_config(), SEED, sample5)
        dt5 = time.perf_counter() - t0
        config5["cpu_oracle"] = {"corners_per_s": sample5 / dt5, "cores": min(sample5, os.cpu_count() or 1),
                                 "sample": f"{sample5} corners (one per host thread), FP64"}

    # workload 4: the stated network (10 inputs -> 3 x 256 GELU -> 12) on 262,144 samples,
    # against its FP64 linear term alone and against a cold (nodeset) start
    config4 = None
    if not args.no_config4 and rank == 0:
        N4 = 262144
        ws10 = WarmStart(ctx, circ, n_inputs=10, n_hidden=256, n_layers=3, seed=5)
        rep10 = ws10.train(topo, seed=TRAIN_SEED, samples=args.train_samples, epochs=16, batch=4096, lr=2e-3)
        x4 = torch.empty((N4, n), dtype=torch.float64, device=dev)
        it4 = torch.empty(N4, dtype=torch.int32, device=dev)
        st4 = torch.empty(N4, dtype=torch.uint8, device=dev)
        res4 = {}
        learned4 = lambda f: ws10.sweep_device(topo, cfg_mixed, SEED, N4, x4, first=f, iters=it4, status=st4,
                                               stream=stream)
        arms4 = (("learned", learned4), ("linear_only", learned4),
                 ("cold_nodeset", lambda f: ctx.newton_dc_device(topo, cfg_mixed, SEED, N4, x4, first=f, iters=it4,
                                                                 status=st4, stream=stream)))
        ctx.profile_enable(True)
        for name, run in arms4:
            ws10.use_network(name != "linear_only")
            for w in range(3):
                run(w * N4)
            torch.cuda.synchronize()
            ctx.profile_read()
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
            prof4 = ctx.profile_read()
            res4[name] = {"solves_per_s": conv / (tot / 1e3), "ms_per_sweep": tot / 5, "iters_per_solve": its / (5 * N4),
                          "fallback_rate": fb / (5 * N4), "converged_fraction": conv / (5 * N4),
                          "kernel_ms": {k: v[1] / max(v[0], 1) for k, v in prof4.items()}}
        ctx.profile_enable(False)
        ws10.use_network(True)
        mlp_ms = res4["learned"]["kernel_ms"].get("mlp_warm_start")
        fl4 = 2.0 * (10 * 256 + 2 * 256 * 256 + 256 * n) * N4
        config4 = {"samples": N4, "network": "10->3x256 GELU->12 (tcgen05, weights streamed from L2)",
                   "inputs": rep10.input_labels, "train_seconds": rep10.seconds, "train_samples": rep10.samples,
                   **res4,
                   "speedup_vs_cold": res4["learned"]["solves_per_s"] / res4["cold_nodeset"]["solves_per_s"],
                   "speedup_vs_linear_only": res4["learned"]["solves_per_s"] / res4["linear_only"]["solves_per_s"]}
        if mlp_ms:
            a4 = fl4 / (mlp_ms * 1e-3) / 1e12
            config4["mlp_roofline"] = {"bound": "tensor", "achieved": a4, "peak": bf16_peak, "unit": "TFLOP/s",
                                       "frac": a4 / bf16_peak, "avg_launch_ms": mlp_ms, "flops_per_launch": fl4}

    # BatchedLuSolver::solve_batch against the reference's own GPU path (cuBLAS)
    lu_cmp = None
    if rank == 0 and not args.no_lu_comparator:
        lu_cmp = cublas_lu_comparator(ctx)

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        r, dt, _, done = cpu_baseline(circ, N, min_seconds=10.0)
        r1, dt1, _, done1 = cpu_baseline(circ, 4096, threads=1, min_seconds=2.0)
        cpu = {"value": r, "unit": UNIT, "cores": os.cpu_count() or 1, "kind": "port",
               "sample": f"{done} op-amp Monte Carlo samples ({N}-sample chunks), plain FP64 Newton from the "
                         f"nodeset, {dt:.1f} s on all host threads",
               "single_thread": {"value": r1, "sample": f"{done1} samples on one host thread, {dt1:.1f} s"}}

    if rank == 0:
        def arm(r):
            return {"value": rate(r), "unit": UNIT, "ms_per_step": r["ms"] / r["steps"],
                    "iters_per_solve": r["iters"], "max_resid_A": r["rmax"],
                    "kernel_ms": {k: v[1] / max(v[0], 1) for k, v in r["prof"].items()}}

        flagged = {str(k): v for k, v in head["flags"].items() if (k & 0x0F) != 0}
        summary = {
            "solves_per_s": value, "e2e_solves_per_s": e2e_value, "ms_per_step": head["ms"] / args.steps,
            "plain_fp64_generic": plain_value, "plain_fp64_specialised": fp64_spec_value,
            "speedup_vs_faster_fp64": value / faster_fp64 if faster_fp64 else None,
            "warm_start": head_name,
            "learned_variants": {k: {"solves_per_s": rate(v), "iters_per_solve": round(v["iters"], 4)}
                                 for k, v in variants.items()},
            "converged_fraction": head["conv"] / (N * args.steps * world), "flagged": flagged,
            "err_vs_fp64_oracle": None if oracle_err is None else
            {k: oracle_err[k] for k in ("samples", "max_tol_units", "max_rel")},
            "roofline": None if roofline is None else
            {k: roofline.get(k) for k in ("kernel", "bound", "frac", "achieved", "peak", "unit")},
            "config1": None if config1 is None else
            {k: {kk: config1[k].get(kk) for kk in ("latency_ms_median", "graph_replay_ms_median", "solves_per_s")}
             for k in ("plain_fp64", "mixed")},
            "config3_transients_per_s": None if config3 is None else
            {k: config3[k]["transients_per_s"] for k in ("mixed", "plain_fp64")},
            "config4": None if config4 is None else
            {"network": "10->3x256", "samples": config4["samples"],
             **{k: {kk: round(config4[k][kk], 4) if kk != "solves_per_s" else config4[k][kk]
                    for kk in ("solves_per_s", "iters_per_solve", "fallback_rate")}
                for k in ("learned", "linear_only", "cold_nodeset")},
             "mlp_tensor_frac": (config4.get("mlp_roofline") or {}).get("frac")},
            "config5_corners_per_s": None if config5 is None else
            {k: config5[k]["corners_per_s"] for k in ("mixed", "plain_fp64")},
            "lu_vs_cublas_speedup": None if not lu_cmp or "unavailable" in lu_cmp else
            {k: round(v["speedup"], 2) for k, v in lu_cmp.items()},
            "cpu_baseline_solves_per_s": None if cpu is None else cpu["value"],
            "cpu_single_thread_solves_per_s": None if cpu is None else cpu["single_thread"]["value"],
        }
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": head["ms"] / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64/f32/f16",
            "data": "synthetic (hash-RNG Monte Carlo draws on device, seed 1; network trained on seed 7)",
            "config": workload_config(N, n),
            "arm": {"parallelism": "replicas" if world > 1 else "single GPU",
                    "precision": "mixed (double-float residual, device currents and state; FP32 Jacobian and "
                                 "sparse LU) + learned warm start",
                    "warm_start": (f"MLP {ws.mlp.n_in}->{ws.mlp.n_layers}x{ws.mlp.n_hidden} GELU->{n} "
                                   "(tcgen05, FP16 operands, TMEM) + least-squares linear term")
                    if head_name == "network" else
                    f"least-squares linear term on {ws.mlp.n_in} drawn parameters, evaluated in FP32 in the "
                    "specialised Newton kernel's sample set-up (the network variant is timed beside it: "
                    "learned_variants)"},
            "learned_variants": {k: arm(v) for k, v in variants.items()},
            "plain_fp64": arm(plain),
            "iters_per_solve": head["iters"], "max_resid_A": head["rmax"],
            "status_counts": {str(k): v for k, v in head["flags"].items()},
            "oracle_error": oracle_err,
            "ablations": {k: arm(v) for k, v in ablations.items()},
            "setup": {"specialise_s": spec_s, "train_s": rep.seconds, "train_samples": rep.samples,
                      "train_loss_first_last": [rep.epoch_loss[0], rep.epoch_loss[-1]]},
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": d2h,
                    "inputs": "the circuit (kept on the device after the first call), seed and sweep range; the "
                              "parameters are drawn on the device inside the timed call",
                    "outputs": "x, iterations, status to pinned host memory"},
            "roofline": roofline, "rooflines": rooflines, "pipe_peaks": pipe,
            "kernel_ms": kavg,
            "gpu_launches": sum(v[0] for v in head["prof"].values()),
            "clocks": head["clocks"],
            "config1": config1,
            "config3_ladder_transient": config3,
            "config4": config4,
            "config5_power_grid": config5,
            "ac_sweep": ac_report,
            "bsim3": b3_report,
            "lu_vs_cublas": lu_cmp,
            "cpu_baseline": cpu,
            "summary": summary,
        }
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
