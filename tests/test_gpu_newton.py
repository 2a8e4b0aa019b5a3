"""GPU parity of the batched Newton path against the CPU oracle.

Bars: FP64_EXACT is bit-identical to the oracle when both see the same
parameters (table mode); FP64 (FMA) within 1e-9 relative; MIXED within the
SPICE tolerances reltol 1e-3, vntol 1e-6 V, abstol 1e-12 A.  Iteration counts
and status bytes must match exactly wherever the trajectories are not chaotic.
"""
import numpy as np
import pytest

import oracle
from spicier_gb300 import Circuit, Table, abi, configs

pytestmark = pytest.mark.gpu

EXACT, FAST, MIXED = abi.SP_PREC_FP64_EXACT, abi.SP_PREC_FP64, abi.SP_PREC_MIXED


def tabled(circuit: Circuit, params: np.ndarray) -> Circuit:
    """Same circuit with every parameter read from a table column."""
    c = Circuit(circuit.title + "-table")
    c.node_index = dict(circuit.node_index)
    c.num_branches = circuit.num_branches
    c.nodeset = dict(circuit.nodeset)
    c.pulses = list(circuit.pulses)
    c.elements = [dict(e) for e in circuit.elements]
    c.params = [(abi.SP_DRAW_TABLE, k, 0.0, 0.0) for k in range(len(circuit.params))]
    c.param_labels = list(circuit.param_labels)
    return c


def same_bits(a, b):
    """Bitwise equality, NaN == NaN (payload bits of a NaN are not portable)."""
    eq = a.view(np.uint64) == b.view(np.uint64)
    return bool(np.all(eq | (np.isnan(a) & np.isnan(b))))


def spice_close(x, ref, num_nodes, reltol=1e-3, vntol=1e-6, abstol=1e-12):
    tol = np.empty_like(ref)
    tol[:, :num_nodes] = reltol * np.abs(ref[:, :num_nodes]) + vntol
    tol[:, num_nodes:] = reltol * np.abs(ref[:, num_nodes:]) + abstol
    return np.all(np.abs(x - ref) <= tol)


def zero_start_opamp():
    c = configs.miller_opamp()
    c.nodeset = {}
    return c


@pytest.mark.parametrize("name,make,N", [
    ("cs_nmos", configs.cs_nmos_amp, 1024),
    ("opamp", configs.miller_opamp, 4096),
    ("opamp_zero_start", zero_start_opamp, 1024),
])
def test_exact_mode_bitwise_with_shared_params(ctx, name, make, N):
    base = make()
    P = oracle.draw_params(base, seed=1, count=N)
    circ = tabled(base, P)
    cfg = abi.newton_config(precision=EXACT)
    r = ctx.newton_dc(circ, cfg, seed=1, count=N, table=P)
    xo, io, so, _ = oracle.newton_dc(circ, abi.newton_config(), seed=1, count=N, table=P)
    assert np.array_equal(r.status, so)
    assert np.array_equal(r.iters, io)
    assert same_bits(r.x, xo), "FP64_EXACT must be bit-identical"


@pytest.mark.parametrize("name,make,N", [("cs_nmos", configs.cs_nmos_amp, 4096),
                                         ("opamp", configs.miller_opamp, 8192)])
def test_exact_mode_bitwise_device_rng(ctx, name, make, N):
    """Parameters drawn on the device (correctly rounded Box-Muller) and the
    FP64_EXACT Newton chain: bit-identical to the oracle in "cr" mode."""
    circ = make()
    r = ctx.newton_dc(circ, abi.newton_config(precision=EXACT), seed=3, count=N, first=1000, params=True)
    with oracle.math_mode("cr"):
        xo, io, so, po = oracle.newton_dc(circ, abi.newton_config(), seed=3, count=N, first=1000)
    assert np.array_equal(r.params.view(np.uint64), po.view(np.uint64))
    assert np.array_equal(r.status, so) and np.array_equal(r.iters, io)
    assert same_bits(r.x, xo)


@pytest.mark.parametrize("prec", [FAST, EXACT])
def test_fp64_parity_device_rng(ctx, prec):
    circ = configs.miller_opamp()
    N = 8192
    r = ctx.newton_dc(circ, abi.newton_config(precision=prec), seed=1, count=N, params=True)
    xo, io, so, po = oracle.newton_dc(circ, abi.newton_config(), seed=1, count=N)
    assert np.max(np.abs(r.params - po) / np.abs(po).clip(1e-300)) <= 4.5e-16  # <= 2 ulp draws
    assert np.array_equal(r.iters, io) and np.array_equal(r.status, so)
    rel = np.abs(r.x - xo) / (np.abs(xo) + 1e-12)
    assert rel.max() < 1e-9
    assert r.converged.all() and np.nanmax(r.resid) < 1e-7


def test_mixed_within_spice_tolerance(ctx):
    circ = configs.miller_opamp()
    N = 16384
    r = ctx.newton_dc(circ, abi.newton_config(precision=MIXED), seed=3, count=N)
    xo, io, so, _ = oracle.newton_dc(circ, abi.newton_config(), seed=3, count=N)
    assert r.converged.all()
    assert spice_close(r.x, xo, circ.num_nodes)
    # same trajectories in practice: Newton is the FP64 refinement
    assert np.mean(r.iters == io) > 0.99


def test_cs_amp_all_modes(ctx):
    circ = configs.cs_nmos_amp()
    xo, io, so, _ = oracle.newton_dc(circ, abi.newton_config(), seed=1, count=1024)
    for prec in (EXACT, FAST, MIXED):
        r = ctx.newton_dc(circ, abi.newton_config(precision=prec), seed=1, count=1024)
        assert r.converged.all()
        assert spice_close(r.x, xo, circ.num_nodes)
        if prec != MIXED:
            assert np.max(np.abs(r.x - xo) / (np.abs(xo) + 1e-12)) < 1e-12


def diode_bjt_circuit():
    c = Circuit("diode_bjt")
    c.V("VCC", "vcc", "0", 5.0)
    c.R("RB", "vcc", "b", 430e3)
    c.R("RC", "vcc", "c", 2e3)
    c.Q("Q1", "c", "b", "e", is_=1e-15, bf=120.0, vaf=80.0)
    c.R("RE", "e", "0", 200.0)
    c.R("RD", "vcc", "d", 1e3)
    c.D("D1", "d", "0", is_=1e-14, n=1.0)
    c.params[c.param_labels.index("RC.r")] = (abi.SP_DRAW_GAUSS, 0, 2e3, 100.0)
    return c


def test_transcendental_models_parity(ctx):
    # diode + BJT use exp/log1p: the device libm differs from the host's in
    # the last bit, so parity is 1e-9 relative (not bitwise).
    circ = diode_bjt_circuit()
    N = 2048
    xo, io, so, _ = oracle.newton_dc(circ, abi.newton_config(), seed=5, count=N)
    assert ((so & abi.SP_ST_MASK) == 0).all()
    for prec in (EXACT, FAST):
        r = ctx.newton_dc(circ, abi.newton_config(precision=prec), seed=5, count=N)
        assert np.array_equal(r.status, so)
        assert np.max(np.abs(r.x - xo) / (np.abs(xo) + 1e-12)) < 1e-9
    r = ctx.newton_dc(circ, abi.newton_config(precision=MIXED), seed=5, count=N)
    assert r.converged.all() and spice_close(r.x, xo, circ.num_nodes)


def test_warm_start_and_cold_fallback(ctx):
    circ = configs.miller_opamp()
    N = 1024
    xo, io, so, _ = oracle.newton_dc(circ, abi.newton_config(), seed=2, count=N)
    # warm start at the answer: one iteration, WARM flag
    r = ctx.newton_dc(circ, abi.newton_config(precision=MIXED), seed=2, count=N, x0=xo)
    assert (r.status == abi.SP_ST_FLAG_WARM).all() and (r.iters == 1).all()
    # a far-off warm start misses and restarts cold from the nodeset; exact
    # mode with shared parameters follows the oracle's trajectory bit for bit
    P = oracle.draw_params(circ, seed=2, count=N)
    tc = tabled(circ, P)
    bad = np.tile(np.array(circ.nodeset_vector()), (N, 1))
    bad[:, circ.node_index["bias"]] = 3.3  # every NMOS current source hard on
    bad[:, circ.node_index["n2"]] = 0.0
    r2 = ctx.newton_dc(tc, abi.newton_config(precision=EXACT), seed=2, count=N, x0=bad, table=P)
    xo2, io2, so2, _ = oracle.newton_dc(tc, abi.newton_config(), seed=2, count=N, x0=bad, table=P)
    assert np.array_equal(r2.status, so2) and np.array_equal(r2.iters, io2)
    assert same_bits(r2.x, xo2)
    assert (r2.status & abi.SP_ST_FLAG_WARM).all()


def test_sweep_split_invariance(ctx):
    # draws are keyed by the global sweep index: two halves == one call
    circ = configs.miller_opamp()
    cfg = abi.newton_config(precision=FAST)
    a = ctx.newton_dc(circ, cfg, seed=9, count=2000, params=True)
    b1 = ctx.newton_dc(circ, cfg, seed=9, count=1000, first=0, params=True)
    b2 = ctx.newton_dc(circ, cfg, seed=9, count=1000, first=1000, params=True)
    assert np.array_equal(a.params, np.vstack([b1.params, b2.params]))
    assert np.array_equal(a.x, np.vstack([b1.x, b2.x]))


def test_moments_match_oracle(ctx):
    circ = configs.miller_opamp()
    N = 5000
    r = ctx.newton_dc(circ, abi.newton_config(precision=FAST), seed=4, count=N, moments=True)
    for col, m in enumerate(r.moments):
        v = r.x[r.converged, col]
        assert m["count"] == len(v)
        assert m["min"] == v.min() and m["max"] == v.max()
        assert abs(m["sum"] - v.sum()) <= 1e-12 * np.abs(v).sum() + 1e-300
        assert abs(m["sum_sq"] - (v * v).sum()) <= 1e-12 * (v * v).sum() + 1e-300


def test_errors_are_statuses(ctx):
    import spicier_gb300 as sg
    big = Circuit("too_big")
    for k in range(40):
        big.R(f"R{k}", f"n{k}", "0", 1.0)
    with pytest.raises(sg.SpicierError) as e:
        ctx.newton_dc(big, abi.newton_config(), seed=0, count=4)
    assert e.value.kind == "InvalidDimension"
    bad = configs.cs_nmos_amp()
    bad.elements[0]["node"][0] = 99
    bad._c_keepalive = None
    with pytest.raises(sg.SpicierError) as e:
        ctx.newton_dc(bad, abi.newton_config(), seed=0, count=4)
    assert e.value.kind == "InvalidDimension"
    tab = Circuit("table")
    tab.V("V", "a", "0", Table(3))
    tab.R("R", "a", "0", 1.0)
    with pytest.raises(sg.SpicierError):
        ctx.newton_dc(tab, abi.newton_config(), seed=0, count=4, table=np.zeros((4, 2)))
    # BatchTooLarge carries the reference variant's own text, "Batch size {size} exceeds
    # maximum {max}" (error.rs:28-30), so a binding recovers both fields from it
    cfg = ctx.config()
    small = type(cfg)(cfg.min_batch_size, cfg.min_matrix_size, 100)
    ctx.set_config(small)
    try:
        with pytest.raises(sg.SpicierError) as e:
            ctx.newton_dc(configs.cs_nmos_amp(), abi.newton_config(), seed=0, count=101)
        assert e.value.kind == "BatchTooLarge" and "Batch size 101 exceeds maximum 100" in str(e.value)
    finally:
        ctx.set_config(cfg)


@pytest.mark.parametrize("prec", [MIXED, EXACT])
def test_host_entry_mapped_output(ctx, prec):
    """sp_newton_dc with page-locked output buffers (the bench's end-to-end
    leg): results identical to those copied into pageable buffers."""
    import ctypes as C

    import torch
    from spicier_gb300._lib import check, load
    circ = configs.miller_opamp()
    N, n = 4096, circ.n
    cfg = abi.newton_config(precision=prec)
    r = ctx.newton_dc(circ, cfg, seed=2, count=N, first=777)
    x = torch.full((N, n), -1.0, dtype=torch.float64).pin_memory()
    it = torch.zeros(N, dtype=torch.int32).pin_memory()
    st = torch.zeros(N, dtype=torch.uint8).pin_memory()
    cc = circ.to_c()
    check(ctx._ptr, load().sp_newton_dc(ctx._ptr, C.byref(cc), C.byref(cfg), 2, 777, N, None, 0, None,
                                        x.data_ptr(), it.data_ptr(), st.data_ptr(), None, None, None))
    assert same_bits(x.numpy(), r.x)
    assert np.array_equal(it.numpy(), r.iters) and np.array_equal(st.numpy(), r.status)


def test_moments_with_fallback_samples(ctx):
    """Moments of the specialised kernel's sweeps (one sample per thread): the
    block partials merged when nothing misses, with or without a fallback
    launch; every converged row when the fallback changed samples (warm starts
    that miss, restarted cold from zero in the kernel, miss again and go to
    gmin / source stepping, which solve some of them).  Each equals numpy's
    moments over the final converged solutions."""
    import torch
    N = 6000
    dev = torch.device("cuda")
    for bad, fb in ((False, True), (True, True), (False, False)):
        circ = zero_start_opamp() if bad else configs.miller_opamp()
        n = circ.n
        topo = ctx.topology(circ)
        x = torch.empty((N, n), dtype=torch.float64, device=dev)
        st = torch.empty(N, dtype=torch.uint8, device=dev)
        mom = torch.full((n, 5), float("nan"), dtype=torch.float64, device=dev)
        cfg = abi.newton_config(precision=MIXED, warm_max_iterations=2,
                                fallback=abi.SP_FALLBACK_GMIN | abi.SP_FALLBACK_SOURCE if fb else 0)
        x0 = torch.full((N, n), 50.0, dtype=torch.float64, device=dev) if bad else None
        ctx.newton_dc_device(topo, cfg, 3, N, x, x0=x0, status=st, moments=mom)
        torch.cuda.synchronize()
        xs, ss, m = x.cpu().numpy(), st.cpu().numpy(), mom.cpu()
        ok = (ss & abi.SP_ST_MASK) == 0
        assert ok.mean() > (0.1 if bad else 0.99)
        if bad:  # the fallback kernel changed samples
            assert ((ss & (abi.SP_ST_FLAG_GMIN | abi.SP_ST_FLAG_SOURCE)) != 0).any()
        counts = m.view(torch.int64)[:, 0].numpy()
        for col in range(n):
            v = xs[ok, col]
            assert counts[col] == len(v)
            assert m[col, 3].item() == v.min() and m[col, 4].item() == v.max()
            assert abs(m[col, 1].item() - v.sum()) <= 1e-12 * np.abs(v).sum() + 1e-300
            assert abs(m[col, 2].item() - (v * v).sum()) <= 1e-12 * (v * v).sum() + 1e-300
        topo.close()
