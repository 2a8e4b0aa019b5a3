"""sp_newton_dc_static — the allocation-free sweep — against the allocating
entry point sp_newton_dc_device, through the C ABI.

The static entry point exists for callers that cannot let a library allocate
device memory (their device memory belongs to a pool they manage, or a hard
cap forbids growth, or cudaMalloc's implicit synchronisation is not allowed
where they call from).  It keeps all scratch in one fixed file-scope device
array.  This file is collected last so that a run stopping at the first
failure has already run every other test; it must pass on its own in a fresh
process as well.
"""
import ctypes as C
import re

import numpy as np
import pytest
import torch

import spicier_gb300 as sg
from spicier_gb300 import abi, configs

pytestmark = pytest.mark.gpu


def _bind(lib):
    f = lib.sp_newton_dc_static
    vp, u64 = C.c_void_p, C.c_uint64
    f.restype = C.c_int
    f.argtypes = [C.POINTER(abi.SpCircuit), C.POINTER(abi.SpNewtonConfig), u64, u64, u64, vp, C.c_uint32, vp,
                  vp, vp, vp, vp, vp, C.c_char_p, C.c_size_t]
    return f


def _bits_equal(a, b):
    eq = a.view(np.uint64) == b.view(np.uint64)
    return bool(np.all(eq | (np.isnan(a) & np.isnan(b))))


@pytest.mark.parametrize("prec", [abi.SP_PREC_MIXED, abi.SP_PREC_FP64_EXACT])
@pytest.mark.parametrize("make,N", [(configs.miller_opamp, 4096), (configs.bsim3_cmos_chain, 2048)])
def test_static_entry_matches_allocating_entry(product_lib, prec, make, N):
    static = _bind(product_lib)
    ctx = sg.Context(0)
    circ = make()
    topo = ctx.topology(circ)
    # the static entry runs the generic kernels (compiling a specialised one
    # would allocate); compare against the same kernels on the allocating side
    ctx.specialize(topo, abi.SP_PREC_MIXED, False)
    cfg = abi.newton_config(precision=prec)
    n = circ.n
    dev = torch.device("cuda", 0)
    stream = torch.cuda.current_stream().cuda_stream
    errbuf = C.create_string_buffer(256)
    for call, first in enumerate((0, 50000)):  # two calls in a row, different sweep ranges
        ref = [torch.full((N, n), -1.0, dtype=torch.float64, device=dev), torch.zeros(N, dtype=torch.int32, device=dev),
               torch.zeros(N, dtype=torch.uint8, device=dev), torch.zeros(N, dtype=torch.float64, device=dev)]
        new = [torch.full((N, n), -2.0, dtype=torch.float64, device=dev), torch.zeros(N, dtype=torch.int32, device=dev),
               torch.zeros(N, dtype=torch.uint8, device=dev), torch.zeros(N, dtype=torch.float64, device=dev)]
        ctx.newton_dc_device(topo, cfg, 1, N, ref[0], first=first, iters=ref[1], status=ref[2], resid=ref[3],
                             stream=stream)
        rc = static(C.byref(circ.to_c()), C.byref(cfg), 1, first, N, None, 0, None, new[0].data_ptr(),
                    new[1].data_ptr(), new[2].data_ptr(), new[3].data_ptr(), stream, errbuf, 256)
        assert rc == 0, errbuf.value.decode()
        torch.cuda.synchronize()
        a = [t.cpu().numpy() for t in ref]
        b = [t.cpu().numpy() for t in new]
        # same kernels and inputs: identical results (the tests' FP64 bar)
        assert _bits_equal(a[0], b[0]), f"call {call}: solutions differ"
        assert np.array_equal(a[1], b[1]) and np.array_equal(a[2], b[2])
        assert _bits_equal(a[3], b[3])
        assert ((b[2] & abi.SP_ST_MASK) == 0).all()
    topo.close()
    ctx.close()


def test_static_entry_rejects_oversized_sweeps(product_lib):
    static = _bind(product_lib)
    circ = configs.miller_opamp()
    cfg = abi.newton_config(precision=abi.SP_PREC_MIXED)
    errbuf = C.create_string_buffer(256)
    x = torch.empty((1, circ.n), dtype=torch.float64, device="cuda")
    rc = static(C.byref(circ.to_c()), C.byref(cfg), 1, 0, 10_000_000, None, 0, None, x.data_ptr(), None, None,
                None, None, errbuf, 256)
    assert rc == abi.SP_ERR_BATCH_TOO_LARGE
    assert b"exceeds maximum" in errbuf.value


def _outputs(N, n, fill):
    dev = torch.device("cuda", 0)
    return [torch.full((N, n), fill, dtype=torch.float64, device=dev), torch.zeros(N, dtype=torch.int32, device=dev),
            torch.zeros(N, dtype=torch.uint8, device=dev), torch.zeros(N, dtype=torch.float64, device=dev)]


def _compare(ref, new):
    a = [t.cpu().numpy() for t in ref]
    b = [t.cpu().numpy() for t in new]
    assert _bits_equal(a[0], b[0]), "solutions differ"
    assert np.array_equal(a[1], b[1]) and np.array_equal(a[2], b[2])
    assert _bits_equal(a[3], b[3])
    return b


def test_static_entry_at_its_limit(product_lib):
    """The largest sweep the fixed array accepts runs and matches the
    allocating entry point bit for bit; one sample more is rejected."""
    static = _bind(product_lib)
    circ = configs.miller_opamp()
    cfg = abi.newton_config(precision=abi.SP_PREC_MIXED)
    errbuf = C.create_string_buffer(256)
    x = torch.empty((1, circ.n), dtype=torch.float64, device="cuda")
    rc = static(C.byref(circ.to_c()), C.byref(cfg), 1, 0, 10_000_000, None, 0, None, x.data_ptr(), None, None,
                None, None, errbuf, 256)
    assert rc == abi.SP_ERR_BATCH_TOO_LARGE
    limit = int(re.search(rb"exceeds maximum (\d+)", errbuf.value).group(1))
    assert 10_000 < limit < 10_000_000
    ctx = sg.Context(0)
    topo = ctx.topology(circ)
    ctx.specialize(topo, abi.SP_PREC_MIXED, False)
    stream = torch.cuda.current_stream().cuda_stream
    ref, new = _outputs(limit, circ.n, -1.0), _outputs(limit, circ.n, -2.0)
    ctx.newton_dc_device(topo, cfg, 1, limit, ref[0], first=7, iters=ref[1], status=ref[2], resid=ref[3],
                         stream=stream)
    rc = static(C.byref(circ.to_c()), C.byref(cfg), 1, 7, limit, None, 0, None, new[0].data_ptr(),
                new[1].data_ptr(), new[2].data_ptr(), new[3].data_ptr(), stream, errbuf, 256)
    assert rc == 0, errbuf.value.decode()
    torch.cuda.synchronize()
    b = _compare(ref, new)
    assert ((b[2] & abi.SP_ST_MASK) == 0).all()
    rc = static(C.byref(circ.to_c()), C.byref(cfg), 1, 7, limit + 1, None, 0, None, new[0].data_ptr(),
                new[1].data_ptr(), new[2].data_ptr(), new[3].data_ptr(), stream, errbuf, 256)
    assert rc == abi.SP_ERR_BATCH_TOO_LARGE
    topo.close()
    ctx.close()


@pytest.mark.parametrize("prec", [abi.SP_PREC_MIXED, abi.SP_PREC_FP64_EXACT])
def test_static_entry_fallback_and_table(product_lib, prec):
    """A warm start that misses (the zero vector: the op-amp's Newton diverges
    from it) sends samples through the fallback launch, which reads the miss
    list kept in the fixed array; the input voltage comes from a table column."""
    static = _bind(product_lib)
    circ = configs.miller_opamp()
    slot = next(i for i, (kind, _idx, _a, _b) in enumerate(circ.params) if kind == abi.SP_DRAW_UNIFORM)
    circ.params[slot] = (abi.SP_DRAW_TABLE, 0, 0.0, 0.0)
    N, n = 3000, circ.n
    dev = torch.device("cuda", 0)
    table = torch.linspace(1.0, 2.3, N, dtype=torch.float64, device=dev).reshape(N, 1).contiguous()
    x0 = torch.zeros((N, n), dtype=torch.float64, device=dev)
    cfg = abi.newton_config(precision=prec, warm_max_iterations=8)
    ctx = sg.Context(0)
    topo = ctx.topology(circ)
    ctx.specialize(topo, abi.SP_PREC_MIXED, False)
    stream = torch.cuda.current_stream().cuda_stream
    errbuf = C.create_string_buffer(256)
    for first in (0, 123):  # two calls in a row
        ref, new = _outputs(N, n, -1.0), _outputs(N, n, -2.0)
        ctx.newton_dc_device(topo, cfg, 1, N, ref[0], first=first, table=table, x0=x0, iters=ref[1], status=ref[2],
                             resid=ref[3], stream=stream)
        rc = static(C.byref(circ.to_c()), C.byref(cfg), 1, first, N, table.data_ptr(), 1, x0.data_ptr(),
                    new[0].data_ptr(), new[1].data_ptr(), new[2].data_ptr(), new[3].data_ptr(), stream, errbuf, 256)
        assert rc == 0, errbuf.value.decode()
        torch.cuda.synchronize()
        b = _compare(ref, new)
        assert ((b[2] & abi.SP_ST_FLAG_COLD) != 0).sum() > N // 10  # the fallback ran for many samples
        assert ((b[2] & abi.SP_ST_MASK) == 0).all()
        assert np.allclose(b[0][:, circ.node("vin")], table.cpu().numpy()[:, 0], rtol=1e-9, atol=0)
    # a table narrower than the circuit reads is rejected
    rc = static(C.byref(circ.to_c()), C.byref(cfg), 1, 0, N, None, 0, x0.data_ptr(), new[0].data_ptr(), None,
                None, None, stream, errbuf, 256)
    assert rc == abi.SP_ERR_INVALID_DIMENSION
    topo.close()
    ctx.close()


def test_static_entry_refuses_a_capturing_stream(product_lib):
    static = _bind(product_lib)
    circ = configs.miller_opamp()
    cfg = abi.newton_config(precision=abi.SP_PREC_MIXED)
    errbuf = C.create_string_buffer(256)
    x = torch.zeros((64, circ.n), dtype=torch.float64, device="cuda")
    y = torch.zeros(64, dtype=torch.float64, device="cuda")
    # the set-up has run (earlier tests, or this call) before the capture starts
    assert static(C.byref(circ.to_c()), C.byref(cfg), 1, 0, 64, None, 0, None, x.data_ptr(), None, None, None,
                  torch.cuda.current_stream().cuda_stream, errbuf, 256) == 0
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        g.capture_begin()
        y.add_(1.0)
        rc = static(C.byref(circ.to_c()), C.byref(cfg), 1, 0, 64, None, 0, None, x.data_ptr(), None, None, None,
                    s.cuda_stream, errbuf, 256)
        g.capture_end()
    assert rc == abi.SP_ERR_INVALID_ARGUMENT
    assert b"capturing" in errbuf.value
    g.replay()
    torch.cuda.synchronize()
    assert float(y[0]) == 1.0
