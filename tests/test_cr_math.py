"""The correctly rounded ln/cos of the Gaussian draw (host build of
cr_math.cuh) and the oracle's RNG against the golden vectors of
tests/golden/ (pure Python + 400/300-bit mpmath, make_golden.py)."""
import json
import os
import struct

import numpy as np
import pytest

import oracle

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def f(h):
    return struct.unpack(">d", bytes.fromhex(h))[0]


@pytest.fixture(scope="module")
def cr_gold():
    return json.load(open(os.path.join(GOLDEN, "cr_math_golden.json")))


@pytest.fixture(scope="module")
def rng_gold():
    return json.load(open(os.path.join(GOLDEN, "rng_golden.json")))


@pytest.mark.parametrize("fn", ["log", "cos", "exp"])
def test_cr_functions_match_golden(cr_gold, fn):
    x = np.array([f(a) for a, _ in cr_gold[fn]])
    want = np.array([f(b) for _, b in cr_gold[fn]])
    y, hard = oracle.cr_batch(fn, x)
    assert hard == 0
    bad = np.nonzero(y.view(np.uint64) != want.view(np.uint64))[0]
    assert bad.size == 0, [(x[i], y[i], want[i]) for i in bad[:5]]


def test_cr_functions_random_against_mpmath():
    mp = pytest.importorskip("mpmath")
    from mpmath.libmp import to_float
    mp.mp.prec = 300
    rng = np.random.default_rng(11)
    x = np.concatenate([rng.integers(1, 2 ** 53, 3000, dtype=np.uint64).astype(np.float64) * 2.0 ** -53,
                        np.exp(rng.uniform(-240, 240, 1000))])
    y, hard = oracle.cr_batch("log", x)
    assert hard == 0
    want = np.array([to_float(mp.log(mp.mpf(float(v)))._mpf_, rnd="n") for v in x])
    assert np.array_equal(y, want)
    t = rng.uniform(-7.99, 7.99, 3000)
    y, hard = oracle.cr_batch("cos", t)
    assert hard == 0
    want = np.array([to_float(mp.cos(mp.mpf(float(v)))._mpf_, rnd="n") for v in t])
    assert np.array_equal(y, want)


def test_cr_exp_random_against_mpmath():
    mp = pytest.importorskip("mpmath")
    from mpmath.libmp import to_float
    mp.mp.prec = 300
    x = np.random.default_rng(12).uniform(-700, 700, 3000)
    y, hard = oracle.cr_batch("exp", x)
    assert hard == 0
    assert np.array_equal(y, [to_float(mp.exp(mp.mpf(float(v)))._mpf_, rnd="n") for v in x])
    y, hard = oracle.cr_batch("exp", np.array([0.0, -0.0, 1e-300, 2.0 ** -55, -(2.0 ** -55)]))
    assert (y == 1.0).all() and hard == 0
    y, hard = oracle.cr_batch("exp", np.array([710.0, np.inf, -746.5, -np.inf]))
    assert list(y) == [np.inf, np.inf, 0.0, 0.0] and hard == 0
    y, hard = oracle.cr_batch("exp", np.array([np.nan]))
    assert np.isnan(y).all() and hard == 1
    # gradual underflow: round at 2^-1074 (exact rounding computed here; mpmath's
    # to_float rounds twice on subnormals)
    x = np.random.default_rng(13).uniform(-745.1, -708.5, 500)
    y, hard = oracle.cr_batch("exp", x)
    assert hard == 0
    for xi, yi in zip(x, y):
        m = mp.exp(mp.mpf(float(xi))) * mp.mpf(2) ** 1074
        r = int(mp.floor(m))
        f = m - r
        r += 1 if (f > 0.5 or (f == 0.5 and r % 2)) else 0
        assert yi == float(mp.mpf(r) * mp.mpf(2) ** -1074)


def test_cr_out_of_domain_is_nan_and_hard():
    y, hard = oracle.cr_batch("log", np.array([0.0, -1.0, np.inf, np.nan, 2.0 ** -400, 2.0 ** 400]))
    assert np.isnan(y).all() and hard == 6
    y, hard = oracle.cr_batch("cos", np.array([8.0, -9.0, np.inf, np.nan]))
    assert np.isnan(y).all() and hard == 4
    y, hard = oracle.cr_batch("log", np.array([1.0]))
    assert y[0] == 0.0 and hard == 0
    y, hard = oracle.cr_batch("cos", np.array([0.0, -0.0, 1e-300]))
    assert (y == 1.0).all() and hard == 0


def test_splitmix_and_uniform_golden(rng_gold):
    L = oracle.lib()
    for a, b in rng_gold["splitmix64"]:
        assert L.or_splitmix64(int(a, 16)) == int(b, 16)
    for seed, sweep, param, want in rng_gold["uniform"]:
        assert L.or_uniform(int(seed, 16), sweep, param) == f(want)


def test_gaussian_golden_cr_mode(rng_gold):
    L = oracle.lib()
    with oracle.math_mode("cr"):
        got = np.array([L.or_gaussian(int(s, 16), sw, p) for s, sw, p, _ in rng_gold["gaussian"]])
    want = np.array([f(w) for *_, w in rng_gold["gaussian"]])
    assert np.array_equal(got.view(np.uint64), want.view(np.uint64))


def test_gaussian_host_libm_agreement(rng_gold):
    """The reference's own draws (host libm) agree with the correctly rounded
    ones except where the libm's ln or cos rounds the wrong way."""
    L = oracle.lib()
    got = np.array([L.or_gaussian(int(s, 16), sw, p) for s, sw, p, _ in rng_gold["gaussian"]])
    want = np.array([f(w) for *_, w in rng_gold["gaussian"]])
    assert np.mean(got == want) > 0.98
    scale = np.spacing(np.maximum(np.abs(want), 1.0))
    assert np.all(np.abs(got - want) <= 8 * scale)


def _batch(fn, x):
    import ctypes as C
    x = np.ascontiguousarray(x, dtype=np.float64)
    y = np.empty_like(x)
    hard = C.c_uint(0)
    getattr(oracle.lib(), f"or_cr_{fn}_batch")(oracle._dp(x), x.size, oracle._dp(y), C.byref(hard))
    return y, hard.value


def test_fast_paths_equal_full_evaluation():
    """The 64-bit fast paths of ln and cos return the 128-bit evaluation's bits wherever they decide."""
    rng = np.random.default_rng(11)
    n = 1 << 19
    u = (rng.integers(1, 1 << 53, n, dtype=np.uint64) >> np.uint64(0)).astype(np.float64) * 2.0 ** -53
    x_cases = [np.maximum(u, 1e-10), np.exp(rng.uniform(-240, 240, n)),
               1.0 + rng.uniform(-2.0 ** -7, 2.0 ** -7, n // 4)]
    for x in x_cases:
        f, hf = _batch("log", x)
        g, hg = _batch("log_full", x)
        assert hf == hg == 0
        assert np.array_equal(f.view(np.uint64), g.view(np.uint64))
    miss = oracle.lib().or_cr_fast_misses(0, oracle._dp(x_cases[0]), x_cases[0].size)
    assert miss < n * 1e-4  # the fast path decides nearly every Box-Muller ln
    base = np.pi / 2 * np.arange(1, 5)
    near = np.concatenate([b * (1 + rng.uniform(-1e-9, 1e-9, 4000)) for b in base]
                          + [np.nextafter(base, base + 1), np.nextafter(base, base - 1)])
    for t in (6.283185307179586 * u, rng.uniform(-7.99, 7.99, n), near):
        f, hf = _batch("cos", t)
        g, hg = _batch("cos_full", t)
        assert hf == hg
        assert np.array_equal(f.view(np.uint64), g.view(np.uint64))


def test_integer_ieee_operations():
    """cr::mul_rn, div_pos and sqrt_pos (the device's integer-pipe IEEE operations) equal the host operators."""
    assert oracle.lib().or_ieee_int_mismatches(3, 1 << 20) == 0
