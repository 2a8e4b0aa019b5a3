"""Measure this GPU's FP64 and FP32 FMA-pipe throughput (roofline peaks).

MEASURED_PEAKS.json carries HBM and bf16 tensor peaks only; the batched
Newton kernels are bound by the FP64 pipe, so this probe (independent FMA
chains per thread, pipe_peak.cu) supplies that denominator.  Writes
profiles/pipe_peaks_gb300.txt.
"""
import os
import re
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))


def main():
    exe = os.path.join(HERE, "_pipe_peak")
    subprocess.run([os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc"),
                    "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-o", exe,
                    os.path.join(HERE, "pipe_peak.cu")], check=True)
    best = {}
    for _ in range(3):
        out = subprocess.run([exe], capture_output=True, text=True, check=True).stdout
        for name, tf in re.findall(r"(fp64|fp32): [\d.]+ ms\s+([\d.]+) TFLOP/s", out):
            best[name] = max(best.get(name, 0.0), float(tf))
    smi = subprocess.run(["nvidia-smi", "--query-gpu=name,clocks.sm,clocks.max.sm", "--format=csv,noheader"],
                         capture_output=True, text=True).stdout.strip()
    txt = (f"# FMA-pipe throughput, best of 3 runs of spicier_gb300/peaks/pipe_peak.cu\n"
           f"# command: python spicier_gb300/peaks/measure.py\n# gpu: {smi}\n"
           f"fp64_tflops: {best['fp64']:.3f}\nfp32_tflops: {best['fp32']:.3f}\n")
    os.makedirs(os.path.join(ROOT, "profiles"), exist_ok=True)
    open(os.path.join(ROOT, "profiles", "pipe_peaks_gb300.txt"), "w").write(txt)
    sys.stdout.write(txt)


if __name__ == "__main__":
    main()
