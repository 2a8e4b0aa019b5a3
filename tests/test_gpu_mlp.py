"""The BF16 tensor-core MLP (forward, gradients, training) against the CPU
oracle, and the learned Newton warm start against the nodeset start."""
import numpy as np
import pytest
import torch

import oracle
from oracle import mlp_oracle as mo
import spicier_gb300 as sg
from spicier_gb300 import abi, configs
from spicier_gb300.api import Mlp, newton_dc_learned
from spicier_gb300.learned import WarmStart
from test_gpu_newton import spice_close

pytestmark = pytest.mark.gpu


def rel(a, b):
    return np.linalg.norm(np.ravel(a - b)) / max(np.linalg.norm(np.ravel(b)), 1e-30)


@pytest.fixture(scope="module")
def net(ctx):
    m = Mlp(ctx, n_in=10, n_out=12, n_hidden=256, n_layers=3, seed=11)
    yield m
    m.close()


TRAIN_KINDS = [abi.SP_MLP_KERNEL_TCGEN05, abi.SP_MLP_KERNEL_MMA_SYNC]


@pytest.mark.parametrize("kind", TRAIN_KINDS)
def test_forward_matches_oracle(ctx, net, kind):
    rng = np.random.default_rng(0)
    rows = 200
    X = rng.standard_normal((rows, 10)).astype(np.float32)
    y = torch.empty((rows, 12), dtype=torch.float32, device="cuda")
    net.set_training_kernel(kind)
    try:
        net.forward_device(torch.tensor(X, device="cuda"), rows, y)
        torch.cuda.synchronize()
    finally:
        net.set_training_kernel(abi.SP_MLP_KERNEL_AUTO)
    layers = net.unflatten(net.get_params())
    Yo, _, _ = mo.forward_backward(layers, X, np.zeros((rows, 12), np.float32), 12)
    assert rel(y.cpu().numpy(), Yo[:, :12]) < 1e-2


def gradients(m, X, T, rows):
    g = torch.empty(m.num_params, dtype=torch.float32, device="cuda")
    loss = torch.zeros(1, dtype=torch.float32, device="cuda")
    m.gradients_device(torch.tensor(X, device="cuda"), torch.tensor(T, device="cuda"), rows, g, loss)
    torch.cuda.synchronize()
    return m.unflatten(g.cpu().numpy()), loss.item()


@pytest.mark.parametrize("kind", TRAIN_KINDS)
def test_gradients_match_oracle(ctx, net, kind):
    rng = np.random.default_rng(1)
    rows = 512
    X = rng.standard_normal((rows, 10)).astype(np.float32)
    T = rng.standard_normal((rows, 12)).astype(np.float32)
    net.set_training_kernel(kind)
    try:
        gpu, loss = gradients(net, X, T, rows)
    finally:
        net.set_training_kernel(abi.SP_MLP_KERNEL_AUTO)
    layers = net.unflatten(net.get_params())
    _, lo, go = mo.forward_backward(layers, X, T, 12)
    assert abs(loss - lo) <= 1e-2 * lo
    for l, ((dW, db), (oW, ob)) in enumerate(zip(gpu, go)):
        assert rel(dW, oW) < 3e-2, f"layer {l} weight gradient"
        assert rel(db, ob) < 3e-2, f"layer {l} bias gradient"
    assert net.fault() == 0


@pytest.mark.parametrize("H,nl,rows", [(128, 3, 576), (64, 2, 64), (256, 1, 1088), (96, 2, 320)])
def test_tcgen05_training_gemms_against_mma_sync(ctx, H, nl, rows):
    """The tcgen05 training GEMMs (every epilogue: bias + GELU with the
    transposed copy, bias only, split-K weight gradients, GELU backward)
    against the mma.sync kernel and the numpy oracle, on widths 64..256 and
    row counts that leave partial 128-row tiles and single split-K chunks."""
    n_in, n_out = 17, 12
    m = Mlp(ctx, n_in, n_out, H, nl, seed=H + nl)
    rng = np.random.default_rng(rows)
    X = rng.standard_normal((rows, n_in)).astype(np.float32)
    T = rng.standard_normal((rows, n_out)).astype(np.float32)
    out = {}
    for kind in TRAIN_KINDS:
        m.set_training_kernel(kind)
        out[kind] = gradients(m, X, T, rows)
    layers = m.unflatten(m.get_params())
    _, lo, go = mo.forward_backward(layers, X, T, n_out)
    (gt, lt), (gm, lm) = out[TRAIN_KINDS[0]], out[TRAIN_KINDS[1]]
    assert abs(lt - lo) <= 1e-2 * lo and abs(lm - lo) <= 1e-2 * lo
    for l in range(len(go)):
        for a, b, o in ((gt[l][0], gm[l][0], go[l][0]), (gt[l][1], gm[l][1], go[l][1])):
            assert rel(a, o) < 3e-2 and rel(b, o) < 3e-2, l
            assert rel(a, b) < 3e-2, l
    assert m.fault() == 0
    m.close()


def test_training_kernel_selector_rejects_bad_kinds(ctx, net):
    with pytest.raises(sg.SpicierError):
        net.set_training_kernel(abi.SP_MLP_KERNEL_LAYERED)


def test_training_is_deterministic_and_learns(ctx):
    rng = np.random.default_rng(2)
    rows = 8192
    X = rng.standard_normal((rows, 10)).astype(np.float32)
    W = rng.standard_normal((10, 12)).astype(np.float32) * 0.5
    T = np.tanh(X @ W).astype(np.float32)
    xs, ts = torch.tensor(X, device="cuda"), torch.tensor(T, device="cuda")
    finals = []
    for _ in range(2):
        m = Mlp(ctx, 10, 12, 256, 3, seed=5)
        ep = torch.zeros(6, dtype=torch.float32, device="cuda")
        m.train_device(xs, ts, rows, 1024, 6, 2e-3, ep)
        torch.cuda.synchronize()
        e = ep.cpu().numpy() / (rows // 1024)
        assert e[-1] < 0.2 * e[0]
        finals.append(m.get_params())
        m.close()
    assert np.array_equal(finals[0], finals[1])


def test_learned_warm_start_cuts_iterations(ctx):
    circ = configs.miller_opamp()
    topo = ctx.topology(circ)
    ws = WarmStart(ctx, circ, n_inputs=10, seed=3)
    rep = ws.train(topo, seed=7, samples=1 << 17, epochs=12, batch=2048)
    assert len(rep.inputs) == 10 and rep.epoch_loss[-1] < rep.epoch_loss[0]
    N = 8192
    dev = torch.device("cuda")
    x = torch.empty((N, circ.n), dtype=torch.float64, device=dev)
    it = torch.empty(N, dtype=torch.int32, device=dev)
    st = torch.empty(N, dtype=torch.uint8, device=dev)
    cfg = abi.newton_config(precision=abi.SP_PREC_MIXED)
    ws.sweep_device(topo, cfg, 1, N, x, iters=it, status=st)
    torch.cuda.synchronize()
    xl, il, sl = x.cpu().numpy(), it.cpu().numpy(), st.cpu().numpy()
    base = ctx.newton_dc(circ, cfg, 1, N)
    assert ((sl & abi.SP_ST_MASK) == 0).all()
    assert (sl & abi.SP_ST_FLAG_WARM).all()
    assert il.mean() < base.iters.mean() - 0.5, (il.mean(), base.iters.mean())
    xo, _io, _so, _ = oracle.newton_dc(circ, abi.newton_config(), 1, N)
    tol = np.empty_like(xo)
    nn = circ.num_nodes
    tol[:, :nn] = 1e-3 * np.abs(xo[:, :nn]) + 1e-6
    tol[:, nn:] = 1e-3 * np.abs(xo[:, nn:]) + 1e-12
    assert np.all(np.abs(xl - xo) <= tol)
    # the host-buffer entry point runs the same kernels on the same draws
    cfg8 = abi.newton_config(precision=abi.SP_PREC_MIXED, warm_max_iterations=ws.WARM_MAX_ITERATIONS)
    h = newton_dc_learned(ctx, circ, ws.mlp, cfg8, 1, N)
    assert np.array_equal(h.x.view(np.uint64), xl.view(np.uint64))
    assert np.array_equal(h.iters, il) and np.array_equal(h.status, sl)


@pytest.mark.parametrize("H,nl", [(128, 3), (64, 2), (128, 1), (256, 3), (256, 1)])
def test_inference_kernels_match_oracle(ctx, H, nl):
    """The tcgen05 warm-start kernel, the fused mma.sync kernel and the
    layer-by-layer GEMMs against the numpy oracle (same BF16 rounding points),
    including the I/O mapping and the linear term, on a ragged row count."""
    n_in, n_out, nslots, rows = 17, 12, 24, 70001
    m = Mlp(ctx, n_in, n_out, H, nl, seed=21)
    rng = np.random.default_rng(H + nl)
    slots = rng.choice(nslots, n_in, replace=False).astype(np.int32)
    in_mean = rng.normal(0, 1, n_in).astype(np.float32)
    in_scale = rng.uniform(0.5, 2, n_in).astype(np.float32)
    out_mean = rng.normal(0, 1, n_out).astype(np.float32)
    out_scale = rng.uniform(0.1, 1, n_out).astype(np.float32)
    lin = rng.normal(0, 0.1, (n_out, n_in))
    m.set_io(slots, in_mean, in_scale, out_mean, out_scale)
    m.set_linear(lin)
    P = rng.normal(0, 1, (nslots, rows))
    dP = torch.tensor(P, device="cuda")
    layers = m.unflatten(m.get_params())
    pc = (P[slots].T - in_mean.astype(np.float64)).astype(np.float32)
    refs = {}
    for rounding in ("bf16", "f16"):  # the mma.sync kernels round like the trainer; tcgen05 runs in FP16
        Y, _, _ = mo.forward_backward(layers, pc / in_scale, np.zeros((rows, n_out), np.float32), n_out,
                                      rounding=rounding)
        refs[rounding] = out_mean + out_scale * Y[:, :n_out].astype(np.float64) + pc.astype(np.float64) @ lin.T
    for kind in (abi.SP_MLP_KERNEL_TCGEN05, abi.SP_MLP_KERNEL_MMA_SYNC, abi.SP_MLP_KERNEL_LAYERED):
        ref = refs["f16" if kind == abi.SP_MLP_KERNEL_TCGEN05 else "bf16"]
        m.set_inference_kernel(kind)
        x0 = torch.full((rows, n_out), float("nan"), dtype=torch.float64, device="cuda")
        m.warm_start_device(dP, rows, rows, x0)
        torch.cuda.synchronize()
        err = np.abs(x0.cpu().numpy() - ref) / out_scale
        assert np.isfinite(err).all(), kind
        # FP32 accumulation order and the SFU tanh flip an occasional BF16
        # rounding of an activation against the oracle; a layout or indexing
        # error would be O(1) everywhere
        assert err.mean() < 2e-3 and np.quantile(err, 0.999) < 3e-2 and err.max() < 0.1, \
            (kind, err.max(), err.mean(), np.quantile(err, 0.999))
    m.close()


def test_tcgen05_rejects_unsupported_shape(ctx):
    for H in (192, 512):
        m = Mlp(ctx, 17, 12, H, 3, seed=1)
        with pytest.raises(sg.SpicierError):
            m.set_inference_kernel(abi.SP_MLP_KERNEL_TCGEN05)
        m.close()


@pytest.mark.parametrize("rows", [1, 127, 129, 300, 128 * 152 * 3 + 5, 262144])
def test_tcgen05_hidden256_row_counts(ctx, rows):
    """The streaming kernel (hidden 256) on the workload's 10 -> 3x256 -> 12
    network over row counts that leave a CTA with no tile, one tile, an odd
    number of tiles (team 1 idle in the last pair) and many tiles: equal to
    the layer-by-layer GEMMs up to the BF16 rounding points."""
    n_in, n_out = 10, 12
    m = Mlp(ctx, n_in, n_out, 256, 3, seed=7)
    rng = np.random.default_rng(rows)
    slots = np.arange(n_in, dtype=np.int32)
    m.set_io(slots, np.zeros(n_in, np.float32), np.ones(n_in, np.float32), np.zeros(n_out, np.float32),
             np.ones(n_out, np.float32))
    P = torch.tensor(rng.normal(0, 1, (n_in, rows)), device="cuda")
    outs = {}
    for kind in (abi.SP_MLP_KERNEL_TCGEN05, abi.SP_MLP_KERNEL_LAYERED):
        m.set_inference_kernel(kind)
        x0 = torch.full((rows, n_out), float("nan"), dtype=torch.float64, device="cuda")
        m.warm_start_device(P, rows, rows, x0)
        torch.cuda.synchronize()
        outs[kind] = x0.cpu().numpy()
    a, b = outs[abi.SP_MLP_KERNEL_TCGEN05], outs[abi.SP_MLP_KERNEL_LAYERED]
    assert np.isfinite(a).all()
    # against the FP16 oracle on the first and last rows (every tile position,
    # the ragged end included), and against the BF16 layer-by-layer GEMMs
    idx = np.unique(np.r_[np.arange(min(rows, 2048)), np.arange(max(0, rows - 2048), rows)])
    layers = m.unflatten(m.get_params())
    Y, _, _ = mo.forward_backward(layers, P.cpu().numpy()[:, idx].T.astype(np.float32),
                                  np.zeros((len(idx), n_out), np.float32), n_out, rounding="f16")
    err = np.abs(a[idx] - Y[:, :n_out])
    assert err.mean() < 2e-3 and err.max() < 0.1, (err.mean(), err.max())
    err = np.abs(a - b)
    assert err.mean() < 1e-2 and err.max() < 0.2, (err.mean(), err.max())
    m.close()


def test_linear_warm_start(ctx):
    """SP_MLP_KERNEL_LINEAR: the fitted linear term alone, evaluated by the
    topology-specialised Newton kernel from each sample's parameters (or by
    the draw kernel for the generic kernels); no inference kernel runs.  The
    standalone warm start equals the formula; the learned sweep equals, bit
    for bit, a sweep started from that standalone warm start, and converges
    every sample in fewer iterations than the nodeset start, within SPICE
    tolerance of the oracle."""
    circ = configs.miller_opamp()
    topo = ctx.topology(circ)
    ws = WarmStart(ctx, circ, n_inputs=10, seed=3)
    ws.train(topo, seed=7, samples=1 << 16, epochs=4, batch=2048)
    ws.use_network(False)
    # standalone: x0 = out_mean + lin (p - in_mean) in FP32
    rows, m = 4099, ws.mlp
    rng = np.random.default_rng(5)
    nslots = len(circ.params)
    in_mean, in_scale = ws._in
    out_mean, _ = ws._io
    P = rng.normal(1.0, 0.1, (nslots, rows))
    P[ws.inputs] = np.asarray(in_mean, np.float64)[:, None] + \
        np.asarray(in_scale, np.float64)[:, None] * rng.normal(0.0, 1.0, (len(ws.inputs), rows))
    x0 = torch.empty((rows, circ.n), dtype=torch.float64, device="cuda")
    m.warm_start_device(torch.tensor(P, device="cuda"), rows, rows, x0)
    torch.cuda.synchronize()
    pc = P[ws.inputs].T.astype(np.float32) - np.asarray(in_mean, np.float32)
    lin = np.asarray(ws._lin, np.float32).astype(np.float64)
    ref = np.asarray(out_mean, np.float64) + pc.astype(np.float64) @ lin.T
    # FP32 evaluation: a few roundings of the largest term
    scale = np.abs(np.asarray(out_mean, np.float64)) + np.abs(pc.astype(np.float64)) @ np.abs(lin).T
    assert np.all(np.abs(x0.cpu().numpy() - ref) <= 1e-6 * scale + 1e-12)
    # the learned sweep
    N = 8192
    dev = torch.device("cuda")
    x = torch.empty((N, circ.n), dtype=torch.float64, device=dev)
    it = torch.empty(N, dtype=torch.int32, device=dev)
    st = torch.empty(N, dtype=torch.uint8, device=dev)
    cfg = abi.newton_config(precision=abi.SP_PREC_MIXED)
    ctx.profile_enable(True)
    ctx.profile_read()
    ws.sweep_device(topo, cfg, 1, N, x, iters=it, status=st)
    torch.cuda.synchronize()
    prof = ctx.profile_read()
    ctx.profile_enable(False)
    assert "mlp_warm_start" not in prof, prof
    xl, il, sl = x.cpu().numpy(), it.cpu().numpy(), st.cpu().numpy()
    assert ((sl & abi.SP_ST_MASK) == 0).all() and (sl & abi.SP_ST_FLAG_WARM).all()
    base = ctx.newton_dc(circ, cfg, 1, N)
    assert il.mean() < base.iters.mean() - 0.5, (il.mean(), base.iters.mean())
    xo, _io, _so, _ = oracle.newton_dc(circ, abi.newton_config(), 1, N)
    assert spice_close(xl, xo, circ.num_nodes)
    # the same sweep from the standalone linear warm start of the same draws
    prm = torch.empty((N, nslots), dtype=torch.float64, device=dev)
    ctx.newton_dc_device(topo, cfg, 1, N, torch.empty_like(x), params=prm)
    x0 = torch.empty((N, circ.n), dtype=torch.float64, device=dev)
    m.warm_start_device(prm.t().contiguous(), N, N, x0)
    cfg8 = abi.newton_config(precision=abi.SP_PREC_MIXED, warm_max_iterations=ws.WARM_MAX_ITERATIONS)
    x2, it2, st2 = torch.empty_like(x), torch.empty_like(it), torch.empty_like(st)
    ctx.newton_dc_device(topo, cfg8, 1, N, x2, x0=x0, iters=it2, status=st2)
    torch.cuda.synchronize()
    assert np.array_equal(x2.cpu().numpy().view(np.uint64), xl.view(np.uint64))
    assert np.array_equal(it2.cpu().numpy(), il) and np.array_equal(st2.cpu().numpy(), sl)
    # the same term with its inputs in descending slot order: the specialised
    # kernel then reads it from memory (its launch-parameter form needs
    # ascending slots); again bit for bit a sweep from the standalone warm start
    assert list(ws.inputs) == sorted(ws.inputs)
    rev = list(range(len(ws.inputs)))[::-1]
    out_mean, out_scale = ws._io
    m.set_io([ws.inputs[j] for j in rev], np.asarray(in_mean)[rev], np.asarray(in_scale)[rev], out_mean, out_scale)
    m.set_linear(np.asarray(ws._lin)[:, rev])
    xr, itr, str_ = torch.empty_like(x), torch.empty_like(it), torch.empty_like(st)
    ws.sweep_device(topo, cfg, 1, N, xr, iters=itr, status=str_)
    m.warm_start_device(prm.t().contiguous(), N, N, x0)
    ctx.newton_dc_device(topo, cfg8, 1, N, x2, x0=x0, iters=it2, status=st2)
    torch.cuda.synchronize()
    assert np.array_equal(x2.cpu().numpy().view(np.uint64), xr.cpu().numpy().view(np.uint64))
    assert np.array_equal(it2.cpu().numpy(), itr.cpu().numpy())
    assert spice_close(xr.cpu().numpy(), xo, circ.num_nodes)
    ws.use_network(True)
    ws.mlp.close()
