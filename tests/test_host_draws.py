"""Parameter draws on the host with the C library's ln/cos/exp
(sp_draw_params_host): the reference's own draw bits on this host
(crates/spicier-batched-sweep/src/rng.rs:120-150), checked bit for bit
against the oracle in its host-libm mode; then a sweep run on those draws
against the oracle's sweep with the same draws."""
import numpy as np
import pytest

import oracle
from spicier_gb300 import abi, configs
from spicier_gb300.api import draw_params_host, table_circuit
from spicier_gb300.circuit import Circuit, Gauss, LogUniform, Table, Uniform


def mixed_draw_circuit():
    c = Circuit("draw_kinds")
    c.V("V1", "a", "0", Uniform(1.0, 2.0, 0))
    c.R("R1", "a", "b", LogUniform(100.0, 1e4, 1))
    c.R("R2", "b", "0", Gauss(1e3, 50.0, 2))
    c.R("R3", "b", "0", Table(0))
    c.I("I1", "b", "0", 1e-6)
    return c


@pytest.mark.parametrize("make", [configs.miller_opamp, configs.cs_nmos_amp, mixed_draw_circuit])
def test_host_draws_equal_reference_bits(product_lib, make):
    circ = make()
    n = 20000
    first = 123457
    table = np.random.default_rng(0).uniform(500, 1500, (n, 1)) if circ.table_cols() else None
    got = draw_params_host(circ, 1, n, first=first, table=table)
    with oracle.math_mode("libm"):
        ref = oracle.draw_params(circ, 1, n, first=first, table=table)
    assert np.array_equal(got.view(np.uint64), ref.view(np.uint64))
    # the same draws with one thread and with many
    one = draw_params_host(circ, 1, n, first=first, table=table, threads=1)
    assert np.array_equal(one.view(np.uint64), got.view(np.uint64))


def test_host_draws_differ_from_correctly_rounded_only_in_last_bits(product_lib):
    circ = configs.miller_opamp()
    n = 1 << 16
    libm = draw_params_host(circ, 1, n)
    with oracle.math_mode("cr"):
        cr = oracle.draw_params(circ, 1, n)
    diff = libm.view(np.int64) - cr.view(np.int64)
    assert np.abs(diff).max() <= 16
    assert (diff == 0).mean() > 0.98


def test_table_circuit_reads_every_slot_from_the_table():
    circ = configs.miller_opamp()
    t = table_circuit(circ)
    assert [p[0] for p in t.params] == [abi.SP_DRAW_TABLE] * len(circ.params)
    assert [p[1] for p in t.params] == list(range(len(circ.params)))
    assert t.table_cols() == len(circ.params) and circ.table_cols() == 0
    assert len(t.elements) == len(circ.elements) and t.nodeset == circ.nodeset


def test_host_draw_errors(product_lib):
    import ctypes as C
    circ = configs.miller_opamp()
    out = np.zeros((4, len(circ.params)))
    cc = circ.to_c()
    assert product_lib.sp_draw_params_host(C.byref(cc), 1, 0xFFFFFFFF, 4, None, 0,
                                           out.ctypes.data_as(C.c_void_p), 1) == abi.SP_ERR_INVALID_ARGUMENT
    assert product_lib.sp_draw_params_host(None, 1, 0, 4, None, 0, out.ctypes.data_as(C.c_void_p),
                                           1) == abi.SP_ERR_INVALID_ARGUMENT


@pytest.mark.gpu
@pytest.mark.parametrize("make", [configs.miller_opamp, configs.cs_nmos_amp])
def test_sweep_on_host_draws_is_bitwise_the_oracle(ctx, make):
    """FP64_EXACT on the host libm's draws: x, iterations and status equal the
    oracle's sweep with the reference's own draws (its libm mode), bit for bit."""
    circ = make()
    n = 8192
    table = draw_params_host(circ, 1, n, first=5000)
    r = ctx.newton_dc(table_circuit(circ), abi.newton_config(precision=abi.SP_PREC_FP64_EXACT), 1, n, first=5000,
                      table=table)
    with oracle.math_mode("libm"):
        xo, io, so, _ = oracle.newton_dc(circ, abi.newton_config(), 1, n, first=5000)
    assert np.array_equal(r.status, so) and np.array_equal(r.iters, io)
    assert np.array_equal(r.x.view(np.uint64), xo.view(np.uint64))
