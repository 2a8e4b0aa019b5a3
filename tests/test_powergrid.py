"""Power-grid corner sweep (Newton + restarted GMRES with Jacobi): the oracle
on the CPU, and the GPU kernel against it in FP64 and mixed precision."""
import ctypes as C

import numpy as np
import pytest

import oracle
from spicier_gb300 import abi
from spicier_gb300._lib import load


def small_cfg(**kw):
    """A 24 x 24 mesh with 72 sinks: the workload's structure at a size the oracle finishes in seconds."""
    kw.setdefault("rows", 24)
    kw.setdefault("cols", 24)
    kw.setdefault("num_sinks", 72)
    return abi.grid_config(**kw)


def test_default_config_matches_library():
    c = abi.SpGridConfig()
    load().sp_grid_config_default(C.byref(c))
    assert bytes(c) == bytes(abi.grid_config())


def test_oracle_kcl_and_corners():
    cfg = small_cfg()
    r = oracle.grid_solve(cfg, 1, 8, threads=4)
    assert (r["status"] == 0).all()
    assert r["resid"].max() < 1e-7
    x = r["x"]
    n = cfg.rows * cfg.cols
    assert (x[:, :n] <= cfg.vdd + 1e-8).all() and (np.abs(x[:, 0] - cfg.vdd) < 1e-8).all()
    # the supply current equals the sum of the sink currents (KCL of the whole mesh)
    # and the heavier corner (resistances x 1.1, VTO - 50 mV) draws more
    assert (x[:, n] < 0).all()
    assert abs(x[1, n]) > 0 and abs(x[0, n]) > abs(x[2, n])  # corner 0 (VTO - 50 mV) > corner 2 (VTO + 50 mV)
    # IR drop grows with the resistance scale
    assert x[1, :n].min() < x[0, :n].min()


def test_oracle_math_modes_agree():
    cfg = small_cfg()
    a = oracle.grid_solve(cfg, 1, 4, threads=4)
    with oracle.math_mode("cr"):
        b = oracle.grid_solve(cfg, 1, 4, threads=4)
    assert np.abs(a["x"] - b["x"]).max() < 1e-9


@pytest.mark.gpu
def test_fp64_against_oracle(ctx):
    cfg = small_cfg(precision=abi.SP_PREC_FP64)
    g = ctx.grid_solve(cfg, 1, 16)
    with oracle.math_mode("cr"):
        o = oracle.grid_solve(cfg, 1, 16)
    assert (g["status"] == 0).all() and np.array_equal(g["newton"], o["newton"])
    # same iteration in exact arithmetic (the GPU orthogonalises by CGS2, the
    # oracle by MGS, and sums in other orders): agreement to the 1e-9 linear tolerance
    assert np.abs(g["x"] - o["x"]).max() < 2e-8
    assert np.abs(g["krylov"] - o["krylov"]).max() <= 0.1 * o["krylov"].max() + 30
    assert g["resid"].max() < 1e-7


@pytest.mark.gpu
def test_mixed_meets_residual_target(ctx):
    cfg = small_cfg(precision=abi.SP_PREC_MIXED)
    g = ctx.grid_solve(cfg, 1, 16)
    with oracle.math_mode("cr"):
        o = oracle.grid_solve(small_cfg(), 1, 16)
    assert (g["status"] == 0).all()
    assert g["resid"].max() <= cfg.resid_target
    n = cfg.rows * cfg.cols
    tol = 1e-3 * np.abs(o["x"][:, :n]) + 1e-6
    assert (np.abs(g["x"][:, :n] - o["x"][:, :n]) <= tol).all()


@pytest.fixture(scope="module")
def full_oracle():
    """Corners 0..3 of the workload's 64 x 64 mesh (4,097 unknowns, 512 sinks):
    one random layout under the four R x VTO corners."""
    with oracle.math_mode("cr"):
        return oracle.grid_solve(abi.grid_config(), 1, 4, threads=4)


@pytest.mark.gpu
@pytest.mark.parametrize("prec", [abi.SP_PREC_FP64, abi.SP_PREC_MIXED])
def test_full_size_mesh_against_oracle(ctx, full_oracle, prec):
    """The workload mesh against the oracle.  Each Newton step's linear solve
    stops at a relative residual of 1e-9, so two Krylov solvers (CGS2 here,
    MGS in the oracle) agree to about 1e-8 of the node voltages, not to the
    last bit: FP64 within 1e-7 V and the SPICE tolerance, MIXED within the
    SPICE tolerance (reltol 1e-3, vntol 1e-6 V; abstol 1e-12 A plus reltol
    for the supply current) and its 1e-9 A residual target."""
    cfg = abi.grid_config(precision=prec)
    g = ctx.grid_solve(cfg, 1, 4)
    o = full_oracle
    assert (g["status"] == 0).all() and (o["status"] == 0).all()
    n = cfg.rows * cfg.cols
    tol_v = 1e-3 * np.maximum(np.abs(g["x"][:, :n]), np.abs(o["x"][:, :n])) + 1e-6
    assert (np.abs(g["x"][:, :n] - o["x"][:, :n]) <= tol_v).all()
    tol_i = 1e-3 * np.abs(o["x"][:, n]) + 1e-12
    assert (np.abs(g["x"][:, n] - o["x"][:, n]) <= tol_i).all()
    if prec == abi.SP_PREC_FP64:
        assert np.array_equal(g["newton"], o["newton"])
        assert np.abs(g["x"][:, :n] - o["x"][:, :n]).max() < 1e-7
        assert g["resid"].max() < 1e-7
    else:
        assert g["resid"].max() <= cfg.resid_target


@pytest.mark.gpu
def test_full_size_mesh(ctx):
    cfg = abi.grid_config(precision=abi.SP_PREC_MIXED)
    g = ctx.grid_solve(cfg, 1, 8)
    assert (g["status"] == 0).all() and g["resid"].max() <= cfg.resid_target


@pytest.mark.gpu
def test_grid_errors(ctx):
    import spicier_gb300 as sg
    with pytest.raises(sg.SpicierError):
        ctx.grid_solve(abi.grid_config(rows=100, cols=100), 1, 1)
    with pytest.raises(sg.SpicierError):
        ctx.grid_solve(abi.grid_config(restart=64), 1, 1)
    with pytest.raises(sg.SpicierError):
        ctx.grid_solve(abi.grid_config(precision=abi.SP_PREC_FP64_EXACT), 1, 1)
