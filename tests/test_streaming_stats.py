"""Streaming statistics and the moments merge (statistics.rs:54-160, 470-590):
the reference's examples, chunked equals whole, the C merge against the
Python accumulator, and a sweep split across two gloo ranks whose merged
moments equal one process's."""
import ctypes as C
import math
import os

import numpy as np
import pytest

from spicier_gb300 import abi
from spicier_gb300.shard import shard_range, sharded_sweep
from spicier_gb300.statistics import (StatisticsAccumulator, StreamingStatistics, SweepStatistics, merge_moments,
                                      moments_to_array)


def test_from_moments_population_variance():
    s = SweepStatistics.from_moments(4, 10.0, 30.0, 1.0, 4.0)  # values 1, 2, 3, 4
    assert s.mean == 2.5 and s.variance == 30.0 / 4 - 6.25 and s.std_dev == math.sqrt(1.25)
    assert s.range() == 3.0
    e = SweepStatistics.from_moments(0, 0.0, 0.0, math.inf, -math.inf)
    assert e.mean == 0.0 and e.variance == 0.0
    # clamped at zero when rounding makes E[x^2] - mean^2 negative
    assert SweepStatistics.from_moments(3, 3.0, 3.0 - 1e-14, 1.0, 1.0).variance == 0.0


def test_streaming_example_of_the_reference():
    # StreamingStatistics doc example (statistics.rs:440-465): two chunks of two 5-node points
    st = StreamingStatistics(5)
    st.process_chunk([1.0, 2.0, 3.0, 4.0, 5.0, 1.1, 2.1, 3.1, 4.1, 5.1], 2)
    st.process_chunk([0.9, 1.9, 2.9, 3.9, 4.9, 1.2, 2.2, 3.2, 4.2, 5.2], 2)
    stats = st.finalize()
    assert len(stats) == 5 and st.total_samples() == 4
    assert abs(stats[0].mean - 1.05) < 1e-12 and stats[0].min == 0.9 and stats[0].max == 1.2


def test_chunked_equals_whole_and_merge_commutes():
    rng = np.random.default_rng(0)
    v = rng.normal(1.0, 0.2, (1000, 3))
    whole = StreamingStatistics(3)
    whole.process_chunk(v, 1000)
    a, b = StreamingStatistics(3), StreamingStatistics(3)
    a.process_chunk(v[:400], 400)
    b.process_chunk(v[400:], 600)
    a.merge(b)
    for x, y in zip(a.finalize(), whole.finalize()):
        assert x.count == y.count and x.min == y.min and x.max == y.max
        assert abs(x.sum - y.sum) <= 1e-12 * abs(y.sum) and abs(x.variance - y.variance) <= 1e-9 * y.variance
    with pytest.raises(ValueError):
        a.merge(StreamingStatistics(4))


def test_c_merge_matches_accumulator(product_lib):
    rng = np.random.default_rng(1)
    vals = rng.normal(size=(2, 50, 4))
    vals[1, 3, 2] = np.nan  # f64::min/max ignore a NaN operand
    accs = [[StatisticsAccumulator() for _ in range(4)] for _ in range(2)]
    for h in range(2):
        for row in vals[h]:
            for k in range(4):
                if not np.isnan(row[k]):
                    accs[h][k].add(float(row[k]))
    ca = (abi.SpMoments * 4)(*[a.as_c() for a in accs[0]])
    cb = (abi.SpMoments * 4)(*[a.as_c() for a in accs[1]])
    merge_moments(ca, cb)
    for k in range(4):
        accs[0][k].merge(accs[1][k])
    assert np.array_equal(moments_to_array(ca), np.array([[a.count, a.sum, a.sum_sq, a.min, a.max]
                                                          for a in accs[0]]))
    nan = (abi.SpMoments * 1)(abi.SpMoments(0, 0.0, 0.0, math.nan, math.nan))
    one = (abi.SpMoments * 1)(abi.SpMoments(1, 2.0, 4.0, 2.0, 2.0))
    merge_moments(nan, one)
    assert nan[0].min == 2.0 and nan[0].max == 2.0


def test_shard_ranges_cover_the_sweep():
    for total in (0, 1, 7, 1000, 65537):
        for world in (1, 2, 3, 8):
            spans = [shard_range(total, r, world, first=11) for r in range(world)]
            assert spans[0][0] == 11 and sum(c for _, c in spans) == total
            for (f0, c0), (f1, _c1) in zip(spans, spans[1:]):
                assert f0 + c0 == f1
            assert max(c for _, c in spans) - min(c for _, c in spans) <= 1


def _oracle_shard(circ, seed):
    """A rank's shard solved by the oracle (the CPU stand-in for its GPU):
    (x, status, moments over the converged samples)."""
    import oracle

    def run(first, count):
        x, _it, st, _p = oracle.newton_dc(circ, abi.newton_config(), seed, count, first=first, threads=2)
        ok = (st & 0x0F) == 0
        acc = StreamingStatistics(circ.n)
        acc.process_chunk(x[ok], int(ok.sum()))
        return x, st, acc.moments_array()

    return run


def _rank_main(rank, world, port, total, out_dir):
    import torch.distributed as dist
    from spicier_gb300 import configs
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    circ = configs.miller_opamp()
    first, x, st, stats = sharded_sweep(_oracle_shard(circ, 1), total, rank, world, circ.n, first=100)
    np.savez(os.path.join(out_dir, f"rank{rank}.npz"), first=first, x=x, st=st,
             mom=np.array([[s.count, s.sum, s.min, s.max, s.variance] for s in stats.finalize()]))
    dist.destroy_process_group()


def test_two_gloo_ranks_merge_to_one_process(tmp_path):
    """Two processes take disjoint sample ranges of one 3,001-sample sweep and
    all-reduce their moments: each rank ends with the moments of the whole
    sweep, equal to one process's (counts, min, max exactly; sums to
    rounding), and the shards' solutions are the single process's rows."""
    import multiprocessing as mp
    import socket

    import oracle
    from spicier_gb300 import configs
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    total = 3001
    ctx = mp.get_context("spawn")
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, total, str(tmp_path))) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=300)
        assert p.exitcode == 0
    circ = configs.miller_opamp()
    x, st, mom = _oracle_shard(circ, 1)(100, total)
    single = StreamingStatistics(circ.n)
    single.process_moments(mom, total)
    ref = np.array([[s.count, s.sum, s.min, s.max, s.variance] for s in single.finalize()])
    r0, r1 = (np.load(tmp_path / f"rank{r}.npz") for r in range(2))
    assert int(r0["first"]) == 100 and int(r1["first"]) == 100 + len(r0["x"])
    assert np.array_equal(np.vstack([r0["x"], r1["x"]]).view(np.uint64), x.view(np.uint64))
    for r in (r0, r1):
        m = r["mom"]
        assert np.array_equal(m[:, [0, 2, 3]], ref[:, [0, 2, 3]])
        assert np.allclose(m[:, 1], ref[:, 1], rtol=1e-13, atol=0)
        assert np.allclose(m[:, 4], ref[:, 4], rtol=1e-6, atol=1e-18)


@pytest.mark.gpu
def test_device_chunks_merge_to_the_whole_sweep(ctx):
    """Moments of a sweep run in three device chunks, merged on the device,
    equal the moments of the same sweep in one call (counts, min, max
    exactly; sums to rounding)."""
    import torch
    from spicier_gb300 import configs
    circ = configs.miller_opamp()
    topo = ctx.topology(circ)
    n, total = circ.n, 30000
    cfg = abi.newton_config(precision=abi.SP_PREC_MIXED)
    dev = torch.device("cuda", 0)
    x = torch.empty((total, n), dtype=torch.float64, device=dev)
    whole = torch.empty((n, 5), dtype=torch.float64, device=dev)
    ctx.newton_dc_device(topo, cfg, 1, total, x, first=500, moments=whole)
    acc = torch.empty((n, 5), dtype=torch.float64, device=dev)
    part = torch.empty((n, 5), dtype=torch.float64, device=dev)
    from spicier_gb300._lib import check, load
    f = 500
    for k, c in enumerate((10000, 7000, 13000)):
        ctx.newton_dc_device(topo, cfg, 1, c, x[:c], first=f, moments=acc if k == 0 else part)
        if k:
            check(ctx._ptr, load().sp_moments_merge_device(ctx._ptr, acc.data_ptr(), part.data_ptr(), n, 0))
        f += c
    torch.cuda.synchronize()
    a, w = acc.cpu(), whole.cpu()
    assert torch.equal(a.view(torch.int64)[:, 0], w.view(torch.int64)[:, 0])
    assert torch.equal(a[:, 3:], w[:, 3:])
    assert torch.allclose(a[:, 1:3], w[:, 1:3], rtol=1e-12, atol=0)
    topo.close()
