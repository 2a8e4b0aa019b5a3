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


@pytest.mark.parametrize("prec", [abi.SP_PREC_MIXED, abi.SP_PREC_FP64])
@pytest.mark.parametrize("make", [configs.miller_opamp, configs.bjt_diode_bias])
def test_warm_miss_restarts_cold_in_kernel(ctx, prec, make):
    """A warm start that misses (its capped attempt does not converge) is
    restarted from the nodeset inside the specialised kernel, the fallback
    chain's first stage: the solution equals, bit for bit, that of a sweep
    started cold; the iterations add the capped attempt's; the status carries
    the warm and cold flags; none needs the fallback kernel's gmin stage."""
    circ = make()
    topo = ctx.topology(circ)
    ctx.specialize(topo, prec, True)
    N, n = 4096, circ.n
    dev = torch.device("cuda")
    outs = []
    for x0 in (None, torch.full((N, n), 50.0, dtype=torch.float64, device=dev)):
        x = torch.empty((N, n), dtype=torch.float64, device=dev)
        it = torch.empty(N, dtype=torch.int32, device=dev)
        st = torch.empty(N, dtype=torch.uint8, device=dev)
        cfg = abi.newton_config(precision=prec, warm_max_iterations=2)
        ctx.profile_enable(True)
        ctx.profile_read()
        ctx.newton_dc_device(topo, cfg, 9, N, x, x0=x0, iters=it, status=st)
        torch.cuda.synchronize()
        prof = ctx.profile_read()
        ctx.profile_enable(False)
        assert any(k.endswith("_spec") for k in prof), prof
        outs.append((x.cpu().numpy(), it.cpu().numpy(), st.cpu().numpy()))
    (xc, ic, sc), (xw, iw, sw) = outs
    assert ((sc & abi.SP_ST_MASK) == 0).all()
    missed = (sw & abi.SP_ST_FLAG_COLD) != 0
    assert missed.mean() > 0.9  # 50 V on every unknown: two iterations do not get there
    assert ((sw & abi.SP_ST_FLAG_GMIN) == 0).all() and ((sw & abi.SP_ST_MASK) == 0).all()
    assert (sw[missed] == (sc[missed] | abi.SP_ST_FLAG_WARM | abi.SP_ST_FLAG_COLD)).all()
    assert np.array_equal(xw[missed].view(np.uint64), xc[missed].view(np.uint64))
    # the capped attempt ran its two iterations, or stopped at the first on a
    # singular or non-finite iterate
    d = iw[missed] - ic[missed]
    assert ((d == 1) | (d == 2)).all() and (d == 2).mean() > 0.5
    topo.close()


def test_item_draws_match_group_draws(ctx):
    """The double-float kernel's sweeps draw their parameters as per-warp
    (group, slot) items when nothing else reads them in the draw kernel; a
    sweep that also returns the parameters draws them per 32-sample group.
    Both give the same solutions, iterations and status bit for bit, and the
    returned parameters are the oracle's draws (ragged last group)."""
    circ = configs.miller_opamp()
    topo = ctx.topology(circ)
    ctx.specialize(topo, abi.SP_PREC_MIXED, True)
    N, n = 5000, circ.n
    dev = torch.device("cuda")
    cfg = abi.newton_config(precision=abi.SP_PREC_MIXED)
    outs = []
    for with_params in (False, True):
        x = torch.empty((N, n), dtype=torch.float64, device=dev)
        it = torch.empty(N, dtype=torch.int32, device=dev)
        st = torch.empty(N, dtype=torch.uint8, device=dev)
        prm = torch.empty((N, len(circ.params)), dtype=torch.float64, device=dev) if with_params else None
        ctx.newton_dc_device(topo, cfg, 21, N, x, first=77, iters=it, status=st, params=prm)
        torch.cuda.synchronize()
        outs.append((x.cpu().numpy(), it.cpu().numpy(), st.cpu().numpy(), prm))
    assert np.array_equal(outs[0][0].view(np.uint64), outs[1][0].view(np.uint64))
    assert np.array_equal(outs[0][1], outs[1][1]) and np.array_equal(outs[0][2], outs[1][2])
    with oracle.math_mode("cr"):
        ref = np.asarray(oracle.draw_params(circ, 21, N, first=77)).reshape(N, -1)
    assert np.array_equal(outs[1][3].cpu().numpy().view(np.uint64), ref.view(np.uint64))
    topo.close()
