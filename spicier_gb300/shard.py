"""A sweep split across processes (one per GPU) by contiguous sample ranges.

Every sample's draws are keyed by its global sweep index (the stateless hash
RNG, crates/spicier-batched-sweep/src/rng.rs:51-56), so a rank that solves
indices [first, first + count) produces exactly the samples a single process
would produce for them: the shards need no data-path exchange.  The one
exchange step is the merge of the per-unknown moments
(StatisticsAccumulator::merge, crates/spicier-batched-sweep/src/statistics.rs:
148-155), an all-reduce of count/sum/sum_sq (sum) and min/max.
"""
from __future__ import annotations

from typing import Callable, Optional, Tuple

import numpy as np

from .statistics import StreamingStatistics, allreduce_moments


def shard_range(total: int, rank: int, world: int, first: int = 0) -> Tuple[int, int]:
    """(first index, count) of rank's contiguous share of `total` samples
    starting at `first`; the first total % world ranks take one extra."""
    if world < 1 or not 0 <= rank < world or total < 0:
        raise ValueError("bad shard request")
    base, extra = divmod(total, world)
    start = rank * base + min(rank, extra)
    return first + start, base + (1 if rank < extra else 0)


def sharded_sweep(run_shard: Callable[[int, int], tuple], total: int, rank: int, world: int, num_nodes: int,
                  first: int = 0, group=None):
    """Run this rank's share of a sweep and merge the moments across ranks.

    run_shard(first_index, count) -> (x [count][n], status [count], moments
    [n][5]) solves the shard (on this rank's GPU).  Returns (first_index,
    x, status, merged StreamingStatistics of the whole sweep)."""
    f, c = shard_range(total, rank, world, first)
    x, st, mom = run_shard(f, c)
    merged = allreduce_moments(np.asarray(mom, dtype=np.float64), group=group) if world > 1 else \
        np.asarray(mom, dtype=np.float64)
    stats = StreamingStatistics(num_nodes)
    stats.process_moments(merged, total)
    return f, x, st, stats


def newton_dc_shard(ctx, topo, cfg, seed: int, total: int, rank: int, world: int, first: int = 0, group=None,
                    stream: Optional[int] = None):
    """sharded_sweep of a DC operating-point sweep on this rank's GPU
    (sp_newton_dc_device with device moments over the converged samples)."""
    import torch
    nn = topo.n
    dev = torch.device("cuda", ctx.device)

    def run(f, c):
        x = torch.empty((c, nn), dtype=torch.float64, device=dev)
        st = torch.empty(c, dtype=torch.uint8, device=dev)
        m = torch.empty((nn, 5), dtype=torch.float64, device=dev)
        ctx.newton_dc_device(topo, cfg, seed, c, x, first=f, status=st, moments=m,
                             stream=stream if stream is not None else torch.cuda.current_stream(dev).cuda_stream)
        torch.cuda.synchronize(dev)
        mom = m.cpu().numpy().copy()
        mom[:, 0] = m.cpu().view(torch.int64)[:, 0].numpy().astype(np.float64)  # count is a uint64 field
        return x, st, mom

    return sharded_sweep(run, total, rank, world, nn, first=first, group=group)
