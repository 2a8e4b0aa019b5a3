"""Build libspicier_gb300.so in-tree with nvcc for sm_103a.

Each translation unit compiles in parallel to an object file under
spicier_gb300/_build/, then nvcc links the shared library next to this
file.  kernels_exact.cu is compiled with --fmad=false (the reference's
operation order, no a*b+c contraction); the others allow FMA.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libspicier_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
UNITS = {
    "api.cu": [],
    "kernels_exact.cu": ["--fmad=false"],
    "kernels_fast.cu": [],
    "newton_static.cu": [],
    "mlp.cu": [],
    "mlp_tc.cu": [],
    "spec.cu": [],
    "host_draw.cu": [],
}
EXTRA_UNITS: dict = {}


def _nvcc() -> str:
    cand = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")
    return cand if os.path.exists(cand) else "nvcc"


def _deps() -> list:
    out = []
    for d in (CSRC, os.path.join(HERE, "..", "include")):
        for f in os.listdir(d):
            if f.endswith((".cu", ".cuh", ".h", ".inc")):
                out.append(os.path.join(d, f))
    return out


def _compile(unit: str, flags: list, verbose: bool) -> str:
    src = os.path.join(CSRC, unit)
    obj = os.path.join(BUILD, unit.replace(".cu", ".o"))
    cmd = [_nvcc(), "-c", src, "-o", obj, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
           "-Xcompiler", "-ffp-contract=off", *ARCH, *flags]
    if verbose:
        cmd.append("-Xptxas=-v")
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"nvcc failed for {unit}:\n{res.stdout}\n{res.stderr}")
    if verbose:
        sys.stderr.write(res.stderr)
    return obj


def build(force: bool = False, verbose: bool = False) -> str:
    units = dict(UNITS)
    units.update(EXTRA_UNITS)
    deps = _deps()
    if not force and os.path.exists(LIB):
        mt = os.path.getmtime(LIB)
        if all(os.path.getmtime(d) <= mt for d in deps):
            return LIB
    os.makedirs(BUILD, exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=len(units)) as ex:
        objs = list(ex.map(lambda kv: _compile(kv[0], kv[1], verbose), units.items()))
    tmp = LIB + ".tmp"
    cuda_lib = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "lib64")
    cmd = [_nvcc(), "-shared", "-o", tmp, *objs, *ARCH, "-lnvrtc", f"-L{cuda_lib}", "-Xlinker", f"-rpath={cuda_lib}"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"link failed:\n{res.stdout}\n{res.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
