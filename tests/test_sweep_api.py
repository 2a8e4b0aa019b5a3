"""The host sweep API (crates/spicier-solver/src/sweep.rs:15-326 and
crates/spicier-batched-sweep/src/sweep.rs:101-217): the reference's own
generator tests restated against the Python mirror, and the reference's
voltage-divider sweep through the GPU batched solve."""
import math

import numpy as np
import pytest

from spicier_gb300.api import (BackendSelector, CornerGenerator, LinearSweepGenerator, MonteCarloGenerator,
                               ParameterVariation, solve_batched_sweep_gpu)
from spicier_gb300.statistics import SweepStatistics


def test_parameter_variation_defaults():
    v = ParameterVariation("R1", 1000.0)
    assert (v.min, v.max, v.sigma) == (900.0, 1100.0, 0.05)


def test_monte_carlo_generator():
    # sweep.rs:383-405
    gen = MonteCarloGenerator(100).with_seed(42)
    variations = [ParameterVariation("R1", 1000.0).with_sigma(0.1), ParameterVariation("R2", 2000.0).with_sigma(0.05)]
    points = gen.generate(variations)
    assert len(points) == 100
    for p in points:
        assert 900.0 <= p.parameters[0] <= 1100.0 and 1800.0 <= p.parameters[1] <= 2200.0
    assert MonteCarloGenerator(100).with_seed(42).generate(variations)[0].parameters == points[0].parameters
    assert MonteCarloGenerator(100).generate(variations)[0].parameters != points[0].parameters  # seed 12345


def test_monte_carlo_first_draw_by_hand():
    """The LCG (x' = 6364136223846793005 x + 1 mod 2^64, u = (x' >> 33) / 2^31)
    and Box-Muller with u1 clamped to 1e-10, spelled out for the first value."""
    m = (1 << 64) - 1
    s1 = (42 * 6364136223846793005 + 1) & m
    s2 = (s1 * 6364136223846793005 + 1) & m
    u1, u2 = max((s1 >> 33) / 2.0 ** 31, 1e-10), (s2 >> 33) / 2.0 ** 31
    z = math.sqrt(-2.0 * math.log(u1)) * math.cos(2.0 * math.pi * u2)
    want = min(max(1000.0 + z * 0.1 * 1000.0, 900.0), 1100.0)
    got = MonteCarloGenerator(1).with_seed(42).generate([ParameterVariation("R1", 1000.0).with_sigma(0.1)])
    assert got[0].parameters[0] == want


def test_corner_generator():
    # sweep.rs:407-433
    variations = [ParameterVariation("R1", 1000.0).with_bounds(900.0, 1100.0),
                  ParameterVariation("R2", 2000.0).with_bounds(1800.0, 2200.0)]
    points = CornerGenerator().generate(variations)
    assert len(points) == 4
    assert {tuple(int(v) for v in p.parameters) for p in points} == {(900, 1800), (900, 2200), (1100, 1800),
                                                                      (1100, 2200)}
    assert [p.parameters[0] for p in points] == [900.0, 1100.0, 900.0, 1100.0]  # bit j -> parameter j
    assert CornerGenerator().generate([])[0].parameters == []


def test_linear_sweep_generator():
    # sweep.rs:435-448
    points = LinearSweepGenerator(5).generate([ParameterVariation("V1", 5.0).with_bounds(0.0, 10.0)])
    assert len(points) == 5
    for p, want in zip(points, (0.0, 2.5, 5.0, 7.5, 10.0)):
        assert abs(p.parameters[0] - want) < 1e-10
    assert LinearSweepGenerator(1).generate([ParameterVariation("V1", 5.0).with_bounds(0.0, 10.0)])[0].parameters == [5.0]


def test_sweep_statistics_from_samples():
    # sweep.rs:450-460
    s = SweepStatistics.from_samples([1.0, 2.0, 3.0, 4.0, 5.0])
    assert abs(s.mean - 3.0) < 1e-10 and abs(s.min - 1.0) < 1e-10 and abs(s.max - 5.0) < 1e-10
    assert s.count == 5 and s.std_dev > 0.0


class DividerStamper:
    """sweep.rs:462-548: R1 between nodes 0 and 1, R2 from node 1 to ground,
    a 10 V source at node 0 (branch current at index 2)."""

    def __init__(self, r1, r2, v):
        self.r1, self.r2, self.v = r1, r2, v

    def stamp_linear(self, m, rhs):
        g1, g2 = 1.0 / self.r1, 1.0 / self.r2
        m[0, 0] += g1
        m[1, 1] += g1
        m[0, 1] -= g1
        m[1, 0] -= g1
        m[1, 1] += g2
        m[0, 2] += 1.0
        m[2, 0] += 1.0
        rhs[2] = self.v

    def num_nodes(self):
        return 2

    def num_vsources(self):
        return 1


class DividerFactory:
    def __init__(self, r2_nominal):
        self.r2 = r2_nominal

    def create_stamper(self, parameters):
        return DividerStamper(parameters[0] if parameters else 1000.0, self.r2, 10.0)


@pytest.mark.gpu
def test_batched_sweep_divider(product_lib):
    """The reference's divider sweep (R1 500..1500 ohm, R2 1 kohm, 10 V)
    solved as one batch on the GPU."""
    res = solve_batched_sweep_gpu(BackendSelector(), DividerFactory(1000.0), LinearSweepGenerator(5),
                                  [ParameterVariation("R1", 1000.0).with_bounds(500.0, 1500.0)])
    assert res.total_count == 5 and res.converged_count == 5 and res.used_gpu
    v1 = [s[1] for s in res.solutions]
    assert v1[0] > v1[-1] and abs(v1[2] - 5.0) < 0.01
    # exact divider values: V1 = 10 R2 / (R1 + R2), source current -10 / (R1 + R2)
    for p, s in zip(res.points, res.solutions):
        r1 = p.parameters[0]
        assert abs(s[1] - 10.0 * 1000.0 / (r1 + 1000.0)) < 1e-12 and abs(s[2] + 10.0 / (r1 + 1000.0)) < 1e-15
