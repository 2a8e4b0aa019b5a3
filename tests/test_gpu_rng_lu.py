"""GPU hash RNG and BatchedLuSolver::solve_batch against the oracle."""
import numpy as np
import pytest
import torch

import oracle
import spicier_gb300 as sg
from spicier_gb300 import abi

pytestmark = pytest.mark.gpu


def rng_gpu(ctx, kind, seed, first, param, count):
    out = torch.empty(count, dtype=torch.float64, device="cuda")
    ctx.rng_fill_device(kind, seed, first, param, count, out)
    torch.cuda.synchronize()
    return out.cpu().numpy()


def rng_cpu(kind, seed, first, param, count):
    import ctypes as C
    out = np.zeros(count)
    oracle.lib().or_rng_fill(kind, seed, first, param, count, out.ctypes.data_as(C.POINTER(C.c_double)))
    return out


@pytest.mark.parametrize("seed,param", [(1, 0), (7, 13), (12345, 2 ** 31 - 1)])
def test_uniform_bit_exact(ctx, seed, param):
    n = 1 << 20
    g = rng_gpu(ctx, 0, seed, 5, param, n)
    c = rng_cpu(0, seed, 5, param, n)
    assert np.array_equal(g.view(np.uint64), c.view(np.uint64))


def test_gaussian_bit_exact_correctly_rounded(ctx):
    """Device Gaussian draws use correctly rounded ln/cos: bit-identical to
    the oracle in "cr" mode and to the mpmath golden vectors."""
    import json
    import os
    import struct
    n = 1 << 20
    g = rng_gpu(ctx, 1, 1, 0, 3, n)
    with oracle.math_mode("cr"):
        c = rng_cpu(1, 1, 0, 3, n)
    assert np.array_equal(g.view(np.uint64), c.view(np.uint64))
    gold = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "rng_golden.json")))["gaussian"]
    block = [w for s, sw, p, w in gold[:4096]]  # the file starts with sweeps 0..4095 of (seed 1, param 3)
    assert all(s == f"{1:016x}" and p == 3 and sw == i for i, (s, sw, p, _) in enumerate(gold[:4096]))
    want = np.array([struct.unpack(">d", bytes.fromhex(w))[0] for w in block])
    assert np.array_equal(g[:len(want)].view(np.uint64), want.view(np.uint64))
    # the reference's host-libm draws differ only where the libm misrounds
    h = rng_cpu(1, 1, 0, 3, n)
    assert np.mean(g == h) > 0.98
    assert np.all(np.abs(g - h) <= 8 * np.spacing(np.maximum(np.abs(h), 1.0)))


def test_f32_variants(ctx):
    n = 1 << 16
    g = rng_gpu(ctx, 2, 3, 0, 1, n)
    c = rng_cpu(2, 3, 0, 1, n)
    assert np.array_equal(g, c)
    g = rng_gpu(ctx, 3, 3, 0, 1, n)
    c = rng_cpu(3, 3, 0, 1, n)
    assert np.max(np.abs(g - c)) < 1e-5


@pytest.mark.parametrize("n,batch", [(1, 33), (2, 64), (6, 1000), (12, 4097), (28, 300), (29, 300), (64, 200),
                                     (100, 64), (165, 9), (200, 20)])
def test_solve_batch_matches_reference_lu(ctx, n, batch):
    rng = np.random.default_rng(n)
    A = rng.standard_normal((batch, n, n)) + 2.0 * np.eye(n)
    b = rng.standard_normal((batch, n))
    mats = np.ascontiguousarray(A.transpose(0, 2, 1)).ravel()  # column-major
    res = ctx.solve_batch(mats, b.ravel(), n, batch)
    sol, sing = oracle.solve_batch(mats, b.ravel(), n, batch)
    assert res.singular_indices == [int(i) for i in np.nonzero(sing)[0]]
    assert np.array_equal(res.solutions.view(np.uint64), sol.view(np.uint64))


@pytest.mark.parametrize("n", [20, 48, 180])
def test_solve_batch_pivot_edge_cases(ctx, n):
    """Ties, zero columns, NaN and Inf entries: the same pivots and the same bits as the reference's LU."""
    rng = np.random.default_rng(n)
    batch = 12
    A = rng.integers(-3, 4, (batch, n, n)).astype(float)  # many equal magnitudes (pivot ties)
    A[1, :, 3] = 0.0              # zero column: the step is skipped, the system singular
    A[2, 5, 5] = np.nan           # NaN on the diagonal: kept as the pivot
    A[3, 7, 2] = np.nan           # NaN below the diagonal: never chosen
    A[4, 9, 9] = np.inf
    A[5] = np.eye(n)              # identity
    A[6, :, :] = 0.0              # all zero
    b = rng.standard_normal((batch, n))
    mats = np.ascontiguousarray(A.transpose(0, 2, 1)).ravel()
    res = ctx.solve_batch(mats, b.ravel(), n, batch)
    sol, sing = oracle.solve_batch(mats, b.ravel(), n, batch)
    assert res.singular_indices == [int(i) for i in np.nonzero(sing)[0]]
    # NaN payloads and signs are not specified (the host and the GPU make different default NaNs)
    g = np.asarray(res.solutions).reshape(batch, n)
    sol = np.asarray(sol).reshape(batch, n)
    nan = np.isnan(g)
    assert np.array_equal(nan, np.isnan(sol))
    assert np.array_equal(g[~nan].view(np.uint64), sol[~nan].view(np.uint64))
    assert nan[2].any() and not nan[5].any()


def test_solve_batch_singular_zero_fill(ctx):
    mats = np.array([1.0, 0.0, 0.0, 1.0, 1.0, 1.0, 2.0, 2.0])
    res = ctx.solve_batch(mats, np.array([1.0, 2.0, 1.0, 2.0]), 2, 2)
    assert res.is_singular(1) and not res.is_singular(0)
    assert np.all(res.solution(1) == 0.0) and np.allclose(res.solution(0), [1.0, 2.0])


def test_solve_batch_mixed_refined(ctx):
    n, batch = 12, 4096
    rng = np.random.default_rng(1)
    A = rng.standard_normal((batch, n, n)) + 4.0 * np.eye(n)
    b = rng.standard_normal((batch, n))
    A[7] = 0.0  # singular system
    mats = torch.tensor(np.ascontiguousarray(A.transpose(0, 2, 1)), device="cuda")
    rhs = torch.tensor(b, device="cuda")
    sol = torch.empty((batch, n), dtype=torch.float64, device="cuda")
    flags = torch.empty(batch, dtype=torch.uint8, device="cuda")
    ctx.solve_batch_device(mats, rhs, n, batch, sol, flags, precision=abi.SP_PREC_MIXED, refine_steps=3)
    torch.cuda.synchronize()
    f = flags.cpu().numpy()
    x = sol.cpu().numpy()
    assert f[7] == 1 and np.all(x[7] == 0.0) and f.sum() == 1
    ok = np.arange(batch) != 7
    # backward error at FP64 level (refinement is backward stable; the forward
    # error additionally scales with each system's condition number)
    r = b[ok] - np.einsum("bij,bj->bi", A[ok], x[ok])
    back = np.max(np.abs(r), axis=1) / (np.max(np.abs(A[ok]), axis=(1, 2)) * np.max(np.abs(x[ok]), axis=1))
    assert back.max() < 64 * n * np.finfo(float).eps
    ref = np.linalg.solve(A[ok], b[ok][..., None])[..., 0]
    cond = np.linalg.cond(A[ok])
    forward = np.max(np.abs(x[ok] - ref), axis=1) / np.max(np.abs(ref), axis=1)
    assert np.all(forward <= 1e-14 * cond)


def test_solve_batch_errors(ctx):
    with pytest.raises(sg.SpicierError) as e:
        ctx.solve_batch(np.zeros(8), np.zeros(3), 2, 2)
    assert e.value.kind == "InvalidDimension"
    cfg = ctx.config()
    ctx.set_config(sg.GpuBatchConfig(cfg.min_batch_size, cfg.min_matrix_size, 4))
    try:
        with pytest.raises(sg.SpicierError) as e:
            ctx.solve_batch(np.tile(np.eye(2).ravel(), 5), np.ones(10), 2, 5)
        assert e.value.kind == "BatchTooLarge"
    finally:
        ctx.set_config(cfg)


def test_trait_mirror(ctx):
    s = sg.Gb300BatchedSolver()
    assert s.backend_type() == sg.BackendType.Gb300
    assert s.should_use_gpu(64, 32) and not s.should_use_gpu(64, 8)
