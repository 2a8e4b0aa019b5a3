"""The C-ABI library loads and exports every function the public header
declares; ctypes struct layouts match the header.  No GPU calls."""
import ctypes as C
import os
import subprocess
import tempfile

from spicier_gb300 import _abi as abi
from spicier_gb300 import _lib

HERE = os.path.dirname(os.path.abspath(__file__))
INCLUDE = os.path.join(HERE, "..", "include")

STRUCTS = {
    "sp_batch_config": (abi.SpBatchConfig, ["min_batch_size", "max_batch_per_launch"]),
    "sp_element": (abi.SpElement, ["kind", "node", "branch", "wave", "field"]),
    "sp_param": (abi.SpParam, ["kind", "rng_index", "a", "b"]),
    "sp_pulse": (abi.SpPulse, ["v1", "per"]),
    "sp_circuit": (abi.SpCircuit, ["num_nodes", "num_pulses", "elements", "params", "pulses", "nodeset"]),
    "sp_newton_config": (abi.SpNewtonConfig, ["v_abstol", "max_iterations", "precision", "fallback",
                                              "refine_steps", "gmin_initial", "gmin_max_attempts",
                                              "src_max_attempts", "src_initial", "src_min_step"]),
    "sp_moments": (abi.SpMoments, ["count", "sum", "sum_sq", "min", "max"]),
}


def test_every_declared_function_is_exported(product_lib):
    names = _lib.header_functions()
    assert len(names) >= 19
    missing = [n for n in names if not hasattr(product_lib, n)]
    assert not missing, f"declared but not exported: {missing}"


def test_version_and_backend_type(product_lib):
    assert product_lib.sp_version().decode().startswith("spicier-gb300")
    assert product_lib.sp_backend_type() == abi.SP_BACKEND_GB300


def test_default_config_matches_reference_defaults(product_lib):
    c = abi.SpNewtonConfig()
    product_lib.sp_newton_config_default(C.byref(c))
    ref = abi.newton_config()
    for name, _ in abi.SpNewtonConfig._fields_:
        assert getattr(c, name) == getattr(ref, name), name


def test_struct_layouts_match_header():
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "spicier_gb300.h"', "int main(void){"]
    for cname, (_, fields) in STRUCTS.items():
        lines.append(f'printf("{cname} %zu\\n", sizeof({cname}));')
        for f in fields:
            lines.append(f'printf("{cname}.{f} %zu\\n", offsetof({cname}, {f}));')
    lines.append("return 0;}")
    with tempfile.TemporaryDirectory() as td:
        src = os.path.join(td, "layout.c")
        exe = os.path.join(td, "layout")
        open(src, "w").write("\n".join(lines))
        subprocess.run(["gcc", "-std=c99", "-I", INCLUDE, src, "-o", exe], check=True)
        out = subprocess.run([exe], capture_output=True, text=True, check=True).stdout
    got = dict(line.rsplit(" ", 1) for line in out.strip().splitlines())
    for cname, (cls, fields) in STRUCTS.items():
        assert int(got[cname]) == C.sizeof(cls), cname
        for f in fields:
            assert int(got[f"{cname}.{f}"]) == getattr(cls, f).offset, f"{cname}.{f}"


def test_no_device_without_gpu_reports_error(product_lib):
    """sp_ctx_create fails with a status (never aborts) when no device is usable."""
    import torch
    if torch.cuda.is_available():
        return
    p = C.c_void_p()
    rc = product_lib.sp_ctx_create(0, C.byref(p))
    assert rc in (abi.SP_ERR_NO_BACKEND, abi.SP_ERR_BACKEND_INIT)
