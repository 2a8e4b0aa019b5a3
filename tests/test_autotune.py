"""The autotuner (spicier_gb300/autotune.py) and the library's tuning table
(sp_tune_set / sp_tune_get): bucket keys and the JSON cache on the CPU; on the
GPU, that every setting leaves results bit for bit unchanged while the tuner
picks the fastest candidate and records it."""
import numpy as np
import pytest

from spicier_gb300 import abi, configs
from spicier_gb300.autotune import Autotuner, TuneCache, bucket, key


def test_buckets_match_the_library(product_lib):
    for n in (1, 3, 4, 5, 8, 12, 16, 17, 100, 513, 4097):
        assert bucket(n) == product_lib.sp_tune_bucket(n)
    assert key("lu.cta", 12) == "lu.cta@16" and key("ladder.bpsm", 512) == "ladder.bpsm@512"


def test_cache_round_trip(tmp_path):
    c = TuneCache(str(tmp_path / "t.json"))
    c.put("NVIDIA GB300", "lu.cta@16", 1, {0: 0.5, 1: 0.25})
    c.save()
    d = TuneCache(str(tmp_path / "t.json"))
    assert d.settings("NVIDIA GB300") == {"lu.cta@16": 1}
    assert d.data["NVIDIA GB300"]["timings"]["lu.cta@16"] == {"0": 0.5, "1": 0.25}
    assert d.settings("other") == {}


@pytest.mark.gpu
def test_tune_table_set_get(ctx, tmp_path):
    t = Autotuner(ctx, TuneCache(str(tmp_path / "none.json")))
    assert t.get("lu.cta@16") is None
    t.set("lu.cta@16", 1)
    assert t.get("lu.cta@16") == 1
    t.set("lu.cta@16", 0)  # 0 removes the key: the built-in heuristic
    assert t.get("lu.cta@16") is None


@pytest.mark.gpu
def test_lu_setting_keeps_results_and_is_tuned(ctx, tmp_path):
    import torch
    t = Autotuner(ctx, TuneCache(str(tmp_path / "t.json")), reps=3)
    n, batch = 12, 20000
    A = torch.rand((batch, n, n), dtype=torch.float64, device="cuda") + n * torch.eye(n, dtype=torch.float64,
                                                                                      device="cuda")
    b = torch.rand((batch, n), dtype=torch.float64, device="cuda")
    outs = []
    for v in (0, 1):
        t.set(key("lu.cta", n), v)
        x = torch.empty_like(b)
        s = torch.empty(batch, dtype=torch.uint8, device="cuda")
        ctx.solve_batch_device(A, b, n, batch, x, s)
        torch.cuda.synchronize()
        outs.append(x.cpu().numpy())
    assert np.array_equal(outs[0].view(np.uint64), outs[1].view(np.uint64))
    best = t.tune_lu(sizes=(n,), batch=batch)[n]
    assert best in (0, 1) and t.get(key("lu.cta", n)) == (best or None)
    t.save()
    t.set(key("lu.cta", n), 0)
    t2 = Autotuner(ctx, TuneCache(str(tmp_path / "t.json")))
    assert t2.apply()[key("lu.cta", n)] == best and t2.get(key("lu.cta", n)) == (best or None)
    t2.set(key("lu.cta", n), 0)


@pytest.mark.gpu
def test_newton_settings_keep_results(ctx, tmp_path):
    import torch
    circ = configs.miller_opamp()
    topo = ctx.topology(circ)
    t = Autotuner(ctx, TuneCache(str(tmp_path / "t.json")), reps=2)
    N = 8192
    for prec, spec, setting, values in ((abi.SP_PREC_MIXED, False, "newton.block.mixed", (0, 32, 64, 128)),
                                        (abi.SP_PREC_MIXED, True, "spec.bpsm.mixed", (0, 1, 2))):
        ctx.specialize(topo, prec, spec)
        outs = []
        for v in values:
            t.set(key(setting, circ.n), v)
            x = torch.empty((N, circ.n), dtype=torch.float64, device="cuda")
            it = torch.empty(N, dtype=torch.int32, device="cuda")
            ctx.newton_dc_device(topo, abi.newton_config(precision=prec), 1, N, x, iters=it)
            torch.cuda.synchronize()
            outs.append((x.cpu().numpy(), it.cpu().numpy()))
        for xo, io in outs[1:]:
            assert np.array_equal(xo.view(np.uint64), outs[0][0].view(np.uint64)) and np.array_equal(io, outs[0][1])
        t.set(key(setting, circ.n), 0)
    ctx.specialize(topo, abi.SP_PREC_MIXED, False)
    chosen = t.tune_newton(topo, abi.SP_PREC_MIXED, samples=N)
    assert set(chosen) == {"spec.bpsm", "newton.block"}
    for k in ("spec.bpsm.mixed", "newton.block.mixed"):
        t.set(key(k, circ.n), 0)
    topo.close()


@pytest.mark.gpu
def test_ladder_and_mlp_settings_keep_results(ctx, tmp_path):
    import torch
    from spicier_gb300.api import Mlp
    t = Autotuner(ctx, TuneCache(str(tmp_path / "t.json")), reps=2)
    cfg = abi.ladder_config(max_sections=64, num_probe=5, precision=abi.SP_PREC_FP64)
    outs = []
    for v in (0, 1):
        t.set(key("ladder.bpsm", cfg.max_sections), v)
        outs.append(ctx.ladder_transient(cfg, 1, 300))
    assert np.array_equal(outs[0]["x"].view(np.uint64), outs[1]["x"].view(np.uint64))
    assert np.array_equal(outs[0]["accepted"], outs[1]["accepted"])
    assert t.tune_ladder(cfg, count=300) in (0, 1, 2)
    t.set(key("ladder.bpsm", cfg.max_sections), 0)
    m = Mlp(ctx, 17, 12, 128, 3, seed=3)
    m.set_io(np.arange(17, dtype=np.int32), np.zeros(17, np.float32), np.ones(17, np.float32),
             np.zeros(12, np.float32), np.ones(12, np.float32))
    m.set_inference_kernel(abi.SP_MLP_KERNEL_TCGEN05)
    P = torch.tensor(np.random.default_rng(1).normal(0, 1, (17, 5000)), device="cuda")
    res = []
    for v in (0, 2, 1):
        t.set(key("mlp.teams", 128), v)
        x0 = torch.empty((5000, 12), dtype=torch.float64, device="cuda")
        m.warm_start_device(P, 5000, 5000, x0)
        torch.cuda.synchronize()
        res.append(x0.cpu().numpy())
    for r in res[1:]:
        assert np.array_equal(res[0].view(np.uint64), r.view(np.uint64))
    assert t.tune_mlp(m, rows=5000) in (0, 1, 2)
    t.set(key("mlp.teams", 128), 0)
    m.close()
