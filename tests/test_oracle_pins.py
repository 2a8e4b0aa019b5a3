"""Pin the CPU oracle to the reference's own known answers.

Each test restates a reference unit/integration test (cited) and checks the
oracle against it.  No GPU needed.
"""
import ctypes as C
import math

import numpy as np
import pytest

import oracle
from spicier_gb300 import Circuit, abi

L = oracle.lib()
dp = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))  # noqa: E731


# -- RNG (crates/spicier-batched-sweep/src/rng.rs) ----------------------------------
def test_splitmix64_published_first_output():
    # SplitMix64 from state 0: the generator's published first output.
    assert L.or_splitmix64(0) == 0xE220A8397B1DCDAF


def test_rng_determinism_and_ranges():
    # rng.rs:336-375 — same coordinates same value; uniform in [0, 1).
    assert L.or_uniform(42, 0, 0) == L.or_uniform(42, 0, 0)
    assert L.or_uniform(42, 0, 0) != L.or_uniform(42, 0, 1)
    u = np.array([L.or_uniform(7, i, 3) for i in range(20000)])
    assert u.min() >= 0.0 and u.max() < 1.0
    assert abs(u.mean() - 0.5) < 0.01
    f = np.array([L.or_uniform_f32(7, i, 3) for i in range(2000)])
    assert f.min() >= 0.0 and f.max() < 1.0


def test_rng_gaussian_moments():
    # rng.rs:376-486 — mean ~ 0, std ~ 1 over many sweep indices.
    g = np.array([L.or_gaussian(42, i, 0) for i in range(20000)])
    assert abs(g.mean()) < 0.05 and abs(g.std() - 1.0) < 0.05
    # u1 = uniform(seed, s, 2p), u2 = uniform(seed, s, 2p+1)
    s, p = 5, 3
    u1 = max(L.or_uniform(9, s, 2 * p), 1e-10)
    u2 = L.or_uniform(9, s, 2 * p + 1)
    assert L.or_gaussian(9, s, p) == math.sqrt(-2.0 * math.log(u1)) * math.cos(2.0 * math.pi * u2)


def test_uniform_is_top53_bits():
    h = L.or_splitmix64(L.or_combine_indices(3, 11, 2))
    assert L.or_uniform(3, 11, 2) == (h >> 11) * 2.0 ** -53


# -- Level-1 MOSFET (crates/spicier-devices/src/mosfet/level1.rs:342-538) ------------
NMOS_DEF = np.array([0.7, 2e-5, 0.0, 10e-6, 1e-6, 1.0])
PMOS_DEF = np.array([-0.7, 1e-5, 0.0, 10e-6, 1e-6, 1.0])


def mos(pmos, p, vgs, vds):
    out = np.zeros(3)
    region = L.or_mos_evaluate(pmos, dp(np.ascontiguousarray(p)), vgs, vds, dp(out))
    return region, out


def test_nmos_cutoff():
    region, (ids, gds, gm) = mos(0, NMOS_DEF, 0.3, 1.0)
    assert region == 0 and ids == 0.0 and gm == 0.0 and gds == 1e-12


def test_nmos_saturation():
    region, (ids, _, gm) = mos(0, NMOS_DEF, 2.0, 5.0)
    assert region == 2 and gm > 0
    assert abs(ids - 0.5 * (2e-5 * 10.0) * 1.3 * 1.3) < 1e-10


def test_nmos_linear():
    region, (ids, gds, gm) = mos(0, NMOS_DEF, 2.0, 0.5)
    assert region == 1 and gds > 0 and gm > 0
    assert abs(ids - 2e-4 * (1.3 * 0.5 - 0.5 * 0.5 * 0.5)) < 1e-10


def test_pmos_saturation_sign():
    region, (ids, _, _) = mos(1, PMOS_DEF, -2.0, -5.0)
    assert region == 2 and ids < 0


def test_pmos_stamping_entries():
    # level1.rs:452-538: PMOS d=1 g=2 s=3, vto -0.7, kp 50u, W/L 10.
    c = Circuit()
    for nm in ("d", "g", "s"):
        c.node(nm)
    c.M("M1", "d", "g", "s", pmos=True, vto=-0.7, kp=50e-6, lam=0.0, w=10e-6, l=1e-6)
    P = np.array([row[2] for row in c.params])
    x = np.array([0.0, 3.0, 5.0])
    A = np.zeros(9)
    b = np.zeros(3)
    L.or_stamp_dc(C.byref(c.to_c()), dp(P), dp(x), 0, 0.0, dp(A), dp(b))
    A = A.reshape(3, 3).T
    vgs, vds = -2.0, -5.0
    region, (ids, gds, gm) = mos(1, P[:6], vgs, vds)
    beta = 50e-6 * 10.0
    assert abs(ids - (-0.5 * beta * 1.3 * 1.3)) < 1e-10 and abs(gm - beta * 1.3) < 1e-10
    ieq = ids - gds * vds - gm * vgs
    eps = 1e-15
    assert abs(A[0, 0] - gds) < eps and abs(A[0, 1] - gm) < eps and abs(A[0, 2] - (-gds - gm)) < eps
    assert abs(A[2, 0] + gds) < eps and abs(A[2, 1] + gm) < eps and abs(A[2, 2] - (gds + gm)) < eps
    assert abs(b[0] + ieq) < eps and abs(b[2] - ieq) < eps


# -- Diode (crates/spicier-devices/src/diode.rs:231-301) ------------------------------
def diode(vd, is_=1e-14, n=1.0):
    out = np.zeros(2)
    L.or_diode_evaluate(is_, n, vd, dp(out))
    return out


def test_diode_bias_regions():
    idf, gdf = diode(0.7)
    assert idf > 0 and gdf > 0
    idr, _ = diode(-1.0)
    assert idr < 0 and abs(idr) < 1e-12
    assert abs(diode(0.0)[0]) < 1e-15


def test_thermal_voltage_and_limiter():
    vt = L.or_thermal_voltage(300.15)
    assert 0.0258 < vt < 0.0259
    lim = L.or_limit_voltage(100.0, vt)
    assert 0.0 < lim < 100.0
    # below vcrit the limiter is the identity
    assert L.or_limit_voltage(0.5, vt) == 0.5


# -- BJT (crates/spicier-devices/src/bjt.rs) ------------------------------------------
def test_bjt_forward_active_gain():
    p = np.array([1e-16, 100.0, 1.0, 1.0, 1.0, math.inf])
    out = np.zeros(6)
    L.or_bjt_evaluate(0, dp(p), 0.7, 5.0, dp(out))
    ic, ib, ie, gm, gpi, go = out
    assert ic > 0 and ib > 0 and abs(ic / ib - 100.0) < 1e-6
    assert abs(gpi - gm / 100.0) < 1e-18
    out2 = np.zeros(6)
    L.or_bjt_evaluate(1, dp(p), -0.7, -5.0, dp(out2))
    assert np.allclose(out2[:3], -out[:3]) and np.allclose(out2[3:], out[3:])


# -- Newton on reference circuits ----------------------------------------------------
def run(circuit, cfg=None, x0=None):
    cfg = cfg or abi.newton_config(fallback=0)
    x, it, st, _ = oracle.newton_dc(circuit, cfg, seed=0, count=1, x0=x0)
    return x[0], int(it[0]), int(st[0])


def test_newton_diode_low_voltage_ngspice():
    # crates/spicier-parser/tests/ngspice_validation.rs:771-829 (ngspice 0.641 V)
    c = Circuit()
    c.V("V1", "1", "0", 0.7)
    c.R("R1", "1", "2", 100.0)
    c.D("D1", "2", "0")
    x, it, st = run(c)
    assert st == abi.SP_ST_CONVERGED and it < 50
    vd = x[c.node_index["2"]]
    assert 0.55 < vd < 0.68
    assert 0.2e-3 < (0.7 - vd) / 100.0 < 1.5e-3


def test_newton_nmos_saturation_ngspice():
    # ngspice_validation.rs:834-890: VDD 5, VG 2, RD 1k, W/L 10u/1u, VTO 0.7, KP 110u.
    c = Circuit()
    c.V("VDD", "1", "0", 5.0)
    c.V("VG", "3", "0", 2.0)
    c.R("RD", "1", "2", 1e3)
    c.M("M1", "2", "3", "0", vto=0.7, kp=110e-6, lam=0.0, w=10e-6, l=1e-6)
    x, it, st = run(c)
    assert st == abi.SP_ST_CONVERGED
    vd = x[c.node_index["2"]]
    assert 3.0 < vd < 5.0
    assert abs(vd - (5.0 - 0.5 * 1.1e-3 * 1.3 ** 2 * 1e3)) < 1e-9  # square law, lambda = 0


def diode_5v():
    c = Circuit()
    c.V("V1", "a", "0", 5.0)
    c.R("R1", "a", "d", 1000.0)
    c.D("D1", "d", "0")
    return c


def test_newton_diode_5v_converges():
    # newton.rs:509-548 circuit (5 V, 1k, Is 1e-14): V(diode) in (0.5, 0.8).
    c = diode_5v()
    x, it, st = run(c)
    assert st == abi.SP_ST_CONVERGED and it < 50
    assert 0.5 < x[c.node_index["d"]] < 0.8
    assert abs(x[c.node_index["a"]] - 5.0) < 1e-6


@pytest.mark.parametrize("which", [0, 1])
def test_gmin_and_source_stepping_use_levels(which):
    # newton.rs:605-667: both aids converge and use more than one level.
    c = diode_5v()
    P = np.array([row[2] for row in c.params])
    cfg = abi.newton_config()
    x = np.zeros(c.n)
    out = (C.c_int * 3)()
    sing = L.or_stepping(C.byref(c.to_c()), dp(P), C.byref(cfg), which, dp(x), out)
    assert sing == 0 and out[0] == 1 and out[2] > 1
    assert 0.5 < x[c.node_index["d"]] < 0.8


def test_convergence_check_semantics():
    # newton.rs test_convergence_check: node tol = reltol*max + vntol.
    c = Circuit()
    c.V("V", "a", "0", 1.0)
    c.R("R", "a", "0", 1.0)
    cfg = abi.newton_config(max_iterations=1, fallback=0)
    # one iteration from the exact answer converges; from far away it does not
    x, it, st = run(c, cfg, x0=np.array([[1.0, -1.0]]))
    assert st & abi.SP_ST_MASK == abi.SP_ST_CONVERGED
    x, it, st = run(c, cfg, x0=np.array([[1.1, -1.0]]))
    assert st & abi.SP_ST_MASK == abi.SP_ST_FAILED


# -- Batched LU (crates/spicier-batched-sweep/src/solver.rs:408-459) ------------------
def test_lu_identity_and_singular():
    mats = np.array([1.0, 0.0, 0.0, 1.0, 1.0, 0.0, 0.0, 1.0])
    sol, sing = oracle.solve_batch(mats, np.array([1.0, 2.0, 3.0, 4.0]), 2, 2)
    assert np.allclose(sol, [1, 2, 3, 4], atol=1e-10) and not sing.any()
    mats = np.array([1.0, 0.0, 0.0, 1.0, 1.0, 1.0, 2.0, 2.0])
    sol, sing = oracle.solve_batch(mats, np.array([1.0, 2.0, 1.0, 2.0]), 2, 2)
    assert list(sing) == [0, 1] and np.all(sol[2:] == 0.0)


def test_lu_matches_numpy():
    rng = np.random.default_rng(0)
    n, B = 9, 64
    A = rng.standard_normal((B, n, n)) + 3 * np.eye(n)
    b = rng.standard_normal((B, n))
    sol, sing = oracle.solve_batch(np.ascontiguousarray(A.transpose(0, 2, 1)).ravel(), b.ravel(), n, B)
    ref = np.linalg.solve(A, b[..., None])[..., 0]
    assert not sing.any() and np.allclose(sol.reshape(B, n), ref, rtol=1e-10, atol=1e-12)


# -- Statistics (crates/spicier-batched-sweep/src/statistics.rs:54-160) ---------------
def test_moments_population_variance():
    v = np.array([1.0, 2.0, 3.0, 4.0])
    m = abi.SpMoments()
    L.or_moments(dp(v), 4, 1, 0, None, C.byref(m))
    assert (m.count, m.sum, m.sum_sq, m.min, m.max) == (4, 10.0, 30.0, 1.0, 4.0)
    mean = m.sum / m.count
    assert max(m.sum_sq / m.count - mean * mean, 0.0) == 1.25
