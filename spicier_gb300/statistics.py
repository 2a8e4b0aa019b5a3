"""Sweep statistics: the reference's statistics types on top of the device
moment reductions.

Mirrors crates/spicier-batched-sweep/src/statistics.rs:
  SweepStatistics        :35-99   from_moments (population variance, clamped at 0)
  StatisticsAccumulator  :113-160 add / merge / finalize
  StreamingStatistics    :470-590 per-node accumulators over chunks, merge, finalize
Moments come either from host values (process_chunk, the reference's path)
or from a device sweep's sp_moments output (process_moments: the moments
kernel already reduced the chunk on the GPU), so a sweep split into chunks,
or into the sample ranges of several processes, combines into the statistics
of the whole sweep without moving its solutions.
"""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass
from typing import List, Optional

import numpy as np

from . import _abi as abi
from ._lib import load


@dataclass
class SweepStatistics:
    """Statistics of one unknown over the sweep (statistics.rs:35-99)."""
    count: int
    min: float
    max: float
    mean: float
    variance: float
    std_dev: float
    sum: float

    @staticmethod
    def from_moments(count: int, sum_: float, sum_sq: float, min_: float, max_: float) -> "SweepStatistics":
        mean = sum_ / count if count > 0 else 0.0
        variance = (sum_sq / count) - mean * mean if count > 0 else 0.0
        variance = max(variance, 0.0)
        return SweepStatistics(count, min_, max_, mean, variance, math.sqrt(variance), sum_)

    @staticmethod
    def from_samples(samples) -> "SweepStatistics":
        acc = StatisticsAccumulator()
        for v in samples:
            acc.add(float(v))
        return acc.finalize()

    def range(self) -> float:
        return self.max - self.min

    def coefficient_of_variation(self) -> Optional[float]:
        return self.std_dev / abs(self.mean) if abs(self.mean) > np.finfo(float).eps else None


def _fmin(a: float, b: float) -> float:  # f64::min: a NaN operand gives the other
    return b if math.isnan(a) else a if math.isnan(b) else min(a, b)


def _fmax(a: float, b: float) -> float:
    return b if math.isnan(a) else a if math.isnan(b) else max(a, b)


class StatisticsAccumulator:
    """Raw moments of one unknown (statistics.rs:113-160)."""

    def __init__(self, count=0, sum_=0.0, sum_sq=0.0, min_=math.inf, max_=-math.inf):
        self.count, self.sum, self.sum_sq, self.min, self.max = count, sum_, sum_sq, min_, max_

    def add(self, value: float):
        self.count += 1
        self.sum += value
        self.sum_sq += value * value
        self.min = _fmin(self.min, value)
        self.max = _fmax(self.max, value)

    def merge(self, other: "StatisticsAccumulator"):
        self.count += other.count
        self.sum += other.sum
        self.sum_sq += other.sum_sq
        self.min = _fmin(self.min, other.min)
        self.max = _fmax(self.max, other.max)

    def finalize(self) -> SweepStatistics:
        return SweepStatistics.from_moments(self.count, self.sum, self.sum_sq, self.min, self.max)

    def as_c(self) -> abi.SpMoments:
        return abi.SpMoments(self.count, self.sum, self.sum_sq, self.min, self.max)


class StreamingStatistics:
    """Per-node accumulators over chunks of solutions (statistics.rs:470-590)."""

    def __init__(self, num_nodes: int):
        self._num_nodes = num_nodes
        self.accumulators = [StatisticsAccumulator() for _ in range(num_nodes)]
        self._total = 0

    def num_nodes(self) -> int:
        return self._num_nodes

    def total_samples(self) -> int:
        return self._total

    def process_chunk(self, solutions, num_sweeps: int):
        """Add num_sweeps flattened solution vectors, value by value in sweep
        order, as the reference does."""
        v = np.asarray(solutions, dtype=np.float64).reshape(num_sweeps, self._num_nodes)
        for i in range(num_sweeps):
            for k, acc in enumerate(self.accumulators):
                acc.add(float(v[i, k]))
        self._total += num_sweeps

    def process_chunk_f32(self, solutions, num_sweeps: int):
        self.process_chunk(np.asarray(solutions, dtype=np.float32).astype(np.float64), num_sweeps)

    def process_moments(self, moments, num_sweeps: int):
        """Fold a device sweep's per-unknown moments (sp_moments[num_nodes],
        as a ctypes array, a list of dicts, or a [num_nodes][5] array of
        count, sum, sum_sq, min, max) into the accumulators; num_sweeps is
        the chunk's sample count (converged or not)."""
        for acc, m in zip(self.accumulators, _rows(moments)):
            acc.merge(StatisticsAccumulator(*m))
        self._total += num_sweeps

    def merge(self, other: "StreamingStatistics"):
        if other._num_nodes != self._num_nodes:
            raise ValueError("Cannot merge statistics with different num_nodes")
        for a, b in zip(self.accumulators, other.accumulators):
            a.merge(b)
        self._total += other._total

    def finalize(self) -> List[SweepStatistics]:
        return [a.finalize() for a in self.accumulators]

    def reset(self):
        self.accumulators = [StatisticsAccumulator() for _ in range(self._num_nodes)]
        self._total = 0

    def node_statistics(self, node_idx: int) -> SweepStatistics:
        return self.accumulators[node_idx].finalize()

    def moments_array(self) -> np.ndarray:
        """[num_nodes][5] float64: count, sum, sum_sq, min, max."""
        return np.array([[a.count, a.sum, a.sum_sq, a.min, a.max] for a in self.accumulators], dtype=np.float64)


def _rows(moments):
    if isinstance(moments, np.ndarray):
        return [(int(r[0]), float(r[1]), float(r[2]), float(r[3]), float(r[4])) for r in moments]
    out = []
    for m in moments:
        if isinstance(m, dict):
            out.append((int(m["count"]), m["sum"], m["sum_sq"], m["min"], m["max"]))
        else:
            out.append((int(m.count), m.sum, m.sum_sq, m.min, m.max))
    return out


def merge_moments(acc, other):
    """sp_moments_merge on two ctypes sp_moments arrays of equal length (acc updated)."""
    if len(acc) != len(other):
        raise ValueError("moment arrays of different lengths")
    rc = load().sp_moments_merge(C.cast(acc, C.c_void_p), C.cast(other, C.c_void_p), len(acc))
    if rc != 0:
        raise ValueError("sp_moments_merge failed")
    return acc


def allreduce_moments(moments: np.ndarray, group=None) -> np.ndarray:
    """Merge [num_nodes][5] moment arrays (count, sum, sum_sq, min, max) across
    the ranks of a torch.distributed group with StatisticsAccumulator::merge
    semantics: counts and sums added, min/max combined.  Works on CPU (gloo)
    and CUDA (nccl) tensors alike; returns the merged array on every rank.
    A moments array in the device layout (sp_moments, count as uint64) is
    taken as float64 here: counts are exact below 2^53."""
    import torch
    import torch.distributed as dist
    m = torch.as_tensor(np.ascontiguousarray(moments, dtype=np.float64))
    if dist.get_backend(group) == "nccl":
        m = m.cuda()
    sums = m[:, :3].contiguous()
    mins = m[:, 3].contiguous()
    maxs = m[:, 4].contiguous()
    # f64::min/max ignore a NaN operand; an empty accumulator holds +/-inf
    mins = torch.where(torch.isnan(mins), torch.full_like(mins, math.inf), mins)
    maxs = torch.where(torch.isnan(maxs), torch.full_like(maxs, -math.inf), maxs)
    dist.all_reduce(sums, op=dist.ReduceOp.SUM, group=group)
    dist.all_reduce(mins, op=dist.ReduceOp.MIN, group=group)
    dist.all_reduce(maxs, op=dist.ReduceOp.MAX, group=group)
    return torch.cat([sums, mins[:, None], maxs[:, None]], 1).cpu().numpy()


def moments_to_array(moments) -> np.ndarray:
    """ctypes sp_moments array (or list of dicts) -> [n][5] float64."""
    return np.array(_rows(moments), dtype=np.float64)
