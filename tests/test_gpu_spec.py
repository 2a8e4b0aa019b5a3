"""GPU parity of the topology-specialised Newton kernels against the oracle."""
import numpy as np
import pytest
import torch

import oracle
from spicier_gb300 import abi, configs
from test_gpu_newton import spice_close

pytestmark = pytest.mark.gpu


def run_device(ctx, circ, prec, seed, N, specialize):
    topo = ctx.topology(circ)
    if specialize:
        ctx.specialize(topo, prec, True)
    else:
        ctx.specialize(topo, abi.SP_PREC_MIXED, False)
    dev = torch.device("cuda")
    x = torch.empty((N, circ.n), dtype=torch.float64, device=dev)
    it = torch.empty(N, dtype=torch.int32, device=dev)
    st = torch.empty(N, dtype=torch.uint8, device=dev)
    res = torch.empty(N, dtype=torch.float64, device=dev)
    ctx.profile_enable(True)
    ctx.profile_read()
    ctx.newton_dc_device(topo, abi.newton_config(precision=prec), seed, N, x, iters=it, status=st, resid=res)
    torch.cuda.synchronize()
    prof = ctx.profile_read()
    ctx.profile_enable(False)
    topo.close()
    return x.cpu().numpy(), it.cpu().numpy(), st.cpu().numpy(), res.cpu().numpy(), prof


@pytest.mark.parametrize("make,N", [(configs.cs_nmos_amp, 1024), (configs.miller_opamp, 16384),
                                    (configs.bjt_diode_bias, 2048)])
def test_specialized_mixed_matches_oracle(ctx, make, N):
    circ = make()
    x, it, st, res, prof = run_device(ctx, circ, abi.SP_PREC_MIXED, 5, N, True)
    assert "newton_primary_mixed_spec" in prof, prof
    xo, io, so, _ = oracle.newton_dc(circ, abi.newton_config(), 5, N)
    assert ((st & abi.SP_ST_MASK) == 0).all()
    assert spice_close(x, xo, circ.num_nodes)
    assert np.mean(it == io) > 0.99
    if make is not configs.bjt_diode_bias:
        assert np.nanmax(res) < 1e-6
    # bjt_diode_bias: the diode and the B-E junction settle just above the
    # limiter's vcrit (0.730 V); the reference's discontinuous limiter
    # (diode.rs:138-148) stops Newton at a point that is not a KCL solution,
    # which the reported residual shows.  The oracle stops at the same point.


@pytest.mark.parametrize("make,N", [(configs.miller_opamp, 8192), (configs.bjt_diode_bias, 2048)])
def test_specialized_fp64_matches_oracle(ctx, make, N):
    circ = make()
    x, it, st, res, prof = run_device(ctx, circ, abi.SP_PREC_FP64, 6, N, True)
    assert "newton_primary_fp64_spec" in prof, prof
    xo, io, so, _ = oracle.newton_dc(circ, abi.newton_config(), 6, N)
    assert np.array_equal(st, so)
    assert np.max(np.abs(x - xo) / (np.abs(xo) + 1e-12)) < 1e-9
    assert np.mean(it == io) > 0.999


def test_specialized_and_generic_agree(ctx):
    circ = configs.miller_opamp()
    a = run_device(ctx, circ, abi.SP_PREC_MIXED, 8, 8192, True)
    b = run_device(ctx, circ, abi.SP_PREC_MIXED, 8, 8192, False)
    assert "newton_primary_mixed" in b[4] and "newton_primary_mixed_spec" not in b[4]
    assert spice_close(a[0], b[0], circ.num_nodes)
