"""Histogram and yield (statistics.rs:243-428): the oracle's restatement
against the reference's own examples, and the GPU kernels against the oracle
(integer counts: exact)."""
import numpy as np
import pytest

import oracle


def test_histogram_oracle_semantics():
    # Histogram::new clamps values outside [min, max) into the end bins
    v = np.array([[-1.0], [0.0], [0.49], [0.5], [0.99], [1.0], [7.0], [np.nan]])
    b = oracle.histogram(v, 0, 0.0, 1.0, 2)
    assert list(b) == [4, 4]  # -1, 0, 0.49, NaN | 0.5, 0.99, 1.0, 7
    # uniform values fill the bins evenly (statistics.rs tests)
    u = ((np.arange(1000) + 0.5) / 1000.0)[:, None]
    assert list(oracle.histogram(u, 0, 0.0, 1.0, 10)) == [100] * 10


def test_yield_oracle_semantics():
    v = np.array([[0.9, 1.0], [1.1, 2.0], [1.0, 3.0], [0.95, 2.5]])
    # YieldSpec::passes is inclusive on both limits
    c = oracle.yield_counts(v, [(0, 0.95, 1.05), (1, 2.0, 3.0)])
    assert list(c) == [2, 3, 2]
    st = np.array([0, 0, 1, 0], np.uint8)  # a non-converged row passes nothing
    c = oracle.yield_counts(v, [(0, 0.95, 1.05), (1, 2.0, 3.0)], status=st)
    assert list(c) == [1, 2, 1]


@pytest.mark.gpu
def test_histogram_and_yield_on_gpu(ctx):
    import torch
    rng = np.random.default_rng(3)
    v = rng.normal(1.0, 0.1, (200_003, 7))
    v[::997, 3] = np.nan
    st = (rng.random(200_003) < 0.03).astype(np.uint8)
    dv = torch.tensor(v, device="cuda")
    ds = torch.tensor(st, device="cuda")
    for status in (None, ds):
        bins, lo, hi = ctx.histogram_device(dv, 3, 37, 0.7, 1.3, status=status)
        ref = oracle.histogram(v, 3, 0.7, 1.3, 37, status=None if status is None else st)
        assert np.array_equal(bins.cpu().numpy().astype(np.uint64), ref)
        specs = [(0, 0.9, 1.1), (3, 0.95, 1.2), (6, -1.0, 1.05)]
        y = ctx.yield_device(dv, specs, status=status)
        yo = oracle.yield_counts(v, specs, status=None if status is None else st)
        assert np.array_equal(y.cpu().numpy().astype(np.uint64), yo)


@pytest.mark.gpu
@pytest.mark.parametrize("rows,cols", [(0, 3), (1, 1), (63, 12), (64, 12), (65, 5), (5000, 12), (100_003, 17),
                                       (262_144, 12), (3000, 40)])
def test_moments_device_sizes(ctx, rows, cols):
    """StatisticsAccumulator over converged rows (statistics.rs:127-155): exact count/min/max, sums to 1e-12."""
    import torch
    rng = np.random.default_rng(rows + cols)
    v = rng.normal(0.0, 1.0, (rows, cols + 2)) * 10.0 ** rng.integers(-6, 3, cols + 2)
    st = (rng.random(rows) < 0.05).astype(np.uint8)
    dv = torch.tensor(v, device="cuda")
    ds = torch.tensor(st, device="cuda")
    out = torch.zeros(max(cols, 1) * 5, dtype=torch.float64, device="cuda")
    for status in (None, ds):
        ctx.moments_device(dv, rows, cols + 2, cols, status, out)
        m = out.cpu().numpy().reshape(-1, 5)[:cols]
        cnt = m[:, 0].copy().view(np.uint64)
        keep = np.ones(rows, bool) if status is None else st == 0
        for c in range(cols):
            x = v[keep, c]
            assert cnt[c] == x.size
            if x.size == 0:
                assert m[c, 1] == 0.0 and m[c, 3] == np.inf and m[c, 4] == -np.inf
                continue
            assert m[c, 3] == x.min() and m[c, 4] == x.max()
            assert abs(m[c, 1] - x.sum()) <= 1e-12 * np.abs(x).sum()
            assert abs(m[c, 2] - (x * x).sum()) <= 1e-12 * (x * x).sum()
