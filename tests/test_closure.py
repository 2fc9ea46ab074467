"""The learned closure's tensor-core convolutions against a PyTorch FP32
reference of the same network (BF16-rounded weights, inputs and hidden
activations, circular padding), its gradients against autograd, Adam, and
the q_parameterization plug-in."""
import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu


def _torch_net(channels, params, slices, x, round_hidden=True):
    import torch
    import torch.nn.functional as F
    h = x.to(torch.bfloat16).float()
    nl = len(channels) - 1
    for i, (ws, shape, bs) in enumerate(slices):
        w = torch.from_numpy(params[ws].reshape(shape)).cuda().permute(0, 3, 1, 2).contiguous()
        w = w.to(torch.bfloat16).float()
        b = torch.from_numpy(params[bs]).cuda()
        h = F.conv2d(F.pad(h, (2, 2, 2, 2), mode="circular"), w, b)
        if i < nl - 1:
            h = torch.relu(h)
            if round_hidden:
                h = h.to(torch.bfloat16).float()
    return h


def _he_params(net, seed):
    """He-uniform weights and small biases: a well-conditioned network for
    checking kernels (independent of the training initialisation)."""
    rng = np.random.default_rng(seed)
    p = np.zeros(net.nparams, dtype=np.float32)
    for ws, shape, bs in net.layer_slices():
        fan_in = shape[1] * shape[2] * shape[3]
        b = np.sqrt(6.0 / fan_in)
        p[ws] = rng.uniform(-b, b, size=ws.stop - ws.start)
        p[bs] = rng.uniform(-0.05, 0.05, size=bs.stop - bs.start)
    return p


def _reference_grads(channels, params, slices, x, t):
    import torch
    import torch.nn.functional as F
    ws_t = []
    h = x.to(torch.bfloat16).float()
    nl = len(channels) - 1
    for i, (ws, shape, bs) in enumerate(slices):
        w = torch.from_numpy(params[ws].reshape(shape)).cuda().permute(0, 3, 1, 2).contiguous()
        w = w.to(torch.bfloat16).float().requires_grad_(True)
        b = torch.from_numpy(params[bs]).cuda().requires_grad_(True)
        ws_t.append((w, b))
        h = F.conv2d(F.pad(h, (2, 2, 2, 2), mode="circular"), w, b)
        if i < nl - 1:
            h = torch.relu(h)
    loss = ((h - t) ** 2).mean()
    loss.backward()
    out = []
    for w, b in ws_t:
        out.append((w.grad.permute(0, 2, 3, 1).contiguous().cpu().numpy(), b.grad.cpu().numpy()))
    return float(loss.detach()), out


@pytest.mark.parametrize("channels,batch", [((2, 16, 8, 2), 2), ((2, 128, 64, 32, 32, 32, 32, 32, 2), 4)])
def test_forward_matches_torch(channels, batch):
    import torch
    from pyqg_gb300.closure import ConvNet
    net = ConvNet(channels, max_batch=batch, seed=3)
    p = net.params
    rng = np.random.default_rng(0)
    p += (0.05 * rng.standard_normal(p.shape)).astype(np.float32)  # nonzero biases too
    net.params = p
    x = torch.from_numpy(rng.standard_normal((batch, channels[0], 64, 64)).astype(np.float32)).cuda()
    y = net.forward(x)
    torch.cuda.synchronize()
    ref = _torch_net(channels, p, net.layer_slices(), x)
    err = rel_l2(y.cpu().numpy(), ref.cpu().numpy())
    assert err < 1e-2, err
    # FP64 in / out through the same kernels
    y64 = net.forward(x.double())
    assert y64.dtype == torch.float64
    assert rel_l2(y64.cpu().numpy(), y.cpu().numpy()) < 1e-6


def test_forward_standardisation():
    import torch
    from pyqg_gb300.closure import ConvNet
    net = ConvNet((2, 16, 2), max_batch=1, seed=1)
    rng = np.random.default_rng(5)
    x = torch.from_numpy(rng.standard_normal((1, 2, 64, 64))).cuda()
    y0 = net.forward(x).cpu().numpy()
    net.set_norm([0.5, -1.0], [2.0, 4.0], [3.0, -2.0], [10.0, 0.5])
    xs = x.clone()
    xs[:, 0] = x[:, 0] * 2.0 + 0.5
    xs[:, 1] = x[:, 1] * 4.0 - 1.0
    y1 = net.forward(xs).cpu().numpy()
    expect = np.stack([y0[:, 0] * 10.0 + 3.0, y0[:, 1] * 0.5 - 2.0], axis=1)
    assert rel_l2(y1, expect) < 1e-2


@pytest.mark.parametrize("channels,batch", [((2, 16, 8, 2), 2), ((2, 128, 64, 32, 32, 32, 32, 32, 2), 2)])
def test_gradients_match_autograd(channels, batch):
    import torch
    from pyqg_gb300.closure import ConvNet
    net = ConvNet(channels, max_batch=batch, seed=4)
    p = _he_params(net, 4)
    rng = np.random.default_rng(1)
    p += (0.02 * rng.standard_normal(p.shape)).astype(np.float32)
    net.params = p
    x = torch.from_numpy(rng.standard_normal((batch, channels[0], 64, 64)).astype(np.float32)).cuda()
    t = torch.from_numpy(rng.standard_normal((batch, channels[-1], 64, 64)).astype(np.float32)).cuda()
    loss = net.backward(x, t)
    g = net.grads
    ref_loss, ref = _reference_grads(channels, p, net.layer_slices(), x, t)
    assert abs(loss - ref_loss) / ref_loss < 1e-2
    for (ws, shape, bs), (gw, gb) in zip(net.layer_slices(), ref):
        assert rel_l2(g[ws].reshape(shape), gw) < 5e-2
        assert rel_l2(g[bs], gb) < 5e-2


def test_adam_reduces_loss():
    import torch
    from pyqg_gb300.closure import ConvNet
    net = ConvNet((2, 32, 32, 2), max_batch=4, seed=2)
    rng = np.random.default_rng(2)
    x = torch.from_numpy(rng.standard_normal((4, 2, 64, 64)).astype(np.float32)).cuda()
    # a target the net can represent: a fixed smoothing of the input
    t = 0.5 * (x + torch.roll(x, 1, dims=2) + torch.roll(x, -1, dims=3)) / 1.5
    losses = [net.train_step(x, t, lr=3e-3) for _ in range(60)]
    assert np.all(np.isfinite(losses))
    assert losses[-1] < 0.5 * losses[0], (losses[0], losses[-1])


def test_adam_update_matches_formula():
    import torch
    from pyqg_gb300.closure import ConvNet
    net = ConvNet((2, 16, 2), max_batch=1, seed=6)
    rng = np.random.default_rng(3)
    x = torch.from_numpy(rng.standard_normal((1, 2, 64, 64)).astype(np.float32)).cuda()
    t = torch.from_numpy(rng.standard_normal((1, 2, 64, 64)).astype(np.float32)).cuda()
    p0 = net.params
    net.backward(x, t)
    g = net.grads
    net.adam(lr=1e-2)
    p1 = net.params
    # first Adam step: m_hat = g, v_hat = g^2 -> step = lr * g / (|g| + eps)
    expect = p0 - 1e-2 * g / (np.abs(g) + 1e-8)
    np.testing.assert_allclose(p1, expect, rtol=1e-5, atol=1e-6)


def test_cnn_parameterization_in_model(quiet):
    import torch
    import pyqg_gb300 as P
    from pyqg_gb300.closure import ConvNet, CNNParameterization
    net = ConvNet(max_batch=1, seed=7)
    stats = ([0.0, 0.0], [1e-6, 1e-7], [0.0, 0.0], [1e-12, 1e-13])
    param = CNNParameterization(net, stats)
    m = P.QGModel(nx=64, dt=7200.0, q_parameterization=param, **quiet)
    rng = np.random.default_rng(0)
    m.q = 1e-7 * rng.standard_normal((2, 64, 64))
    q_dev = m.device_field("q").clone()
    dq = param(m)
    assert isinstance(dq, torch.Tensor) and dq.dtype == torch.float64 and dq.shape == (2, 64, 64)
    direct = net.forward(q_dev)
    assert torch.equal(dq, direct)
    for _ in range(5):
        m._step_forward()
    assert np.all(np.isfinite(m.q))
    assert m.tc == 5


def test_ensemble_closure_matches_single_models(quiet):
    """FP64 ensemble members with the closure attached step like single
    FP64-engine models with the same net as q_parameterization."""
    import pyqg_gb300 as P
    from pyqg_gb300.closure import ConvNet, CNNParameterization
    from pyqg_gb300.coarsen import PHYSICS
    net = ConvNet(max_batch=2, seed=11)
    stats = ([0.0, 0.0], [3e-7, 3e-8], [0.0, 0.0], [3e-13, 3e-14])
    param = CNNParameterization(net, stats)
    rng = np.random.default_rng(9)
    qs = [1e-7 * rng.standard_normal((2, 64, 64)) for _ in range(2)]
    ens = P.Ensemble([("qg", dict(nx=64, dt=7200.0, **PHYSICS))] * 2, precision="fp64")
    ens.set_q(qs)
    assert ens.set_closure(net) == 1
    ens.step(6)
    for i in range(2):
        m = P.QGModel(nx=64, dt=7200.0, q_parameterization=param, **PHYSICS, **quiet)
        m.engine = "fp64"
        m.q = qs[i]
        for _ in range(6):
            m._step_forward()
        assert rel_l2(ens.q(i), m.q) < 1e-13
    # the closure changes the trajectory
    ens2 = P.Ensemble([("qg", dict(nx=64, dt=7200.0, **PHYSICS))] * 2, precision="fp64")
    ens2.set_q(qs)
    ens2.step(6)
    assert rel_l2(ens2.q(0), ens.q(0)) > 1e-8


def test_ensemble_closure_fp32_runs():
    import torch
    import pyqg_gb300 as P
    from pyqg_gb300.closure import ConvNet, CNNParameterization
    from pyqg_gb300.coarsen import PHYSICS
    net = ConvNet(max_batch=8, seed=12)
    CNNParameterization(net, ([0.0, 0.0], [3e-7, 3e-8], [0.0, 0.0], [3e-13, 3e-14]))
    rng = np.random.default_rng(10)
    ens = P.Ensemble([("qg", dict(nx=64, dt=7200.0, **PHYSICS))] * 8, precision="fp32")
    ens.set_q([1e-7 * rng.standard_normal((2, 64, 64)) for _ in range(8)])
    ens.set_closure(net)
    ens.step(20)
    torch.cuda.synchronize()
    assert all(np.all(np.isfinite(ens.q(i))) for i in range(8))


def test_ensemble_closure_fp32_warp_kernels(monkeypatch):
    """The FP32 closure ensemble on the warp-owned kernels (the subgrid
    forcing transformed inside the column kernel) against the block-wide
    FP32 kernels: the same trajectory up to FP32 rounding, amplified only by
    the network's BF16 inputs; the closure's own effect is far larger."""
    import pyqg_gb300 as P
    from pyqg_gb300.closure import ConvNet, CNNParameterization
    from pyqg_gb300.coarsen import PHYSICS
    net = ConvNet(max_batch=4, seed=13)
    CNNParameterization(net, ([0.0, 0.0], [3e-7, 3e-8], [0.0, 0.0], [3e-13, 3e-14]))
    rng = np.random.default_rng(14)
    qs = [1e-7 * rng.standard_normal((2, 64, 64)) for _ in range(4)]
    out = {}
    for name, warp, closure in (("warp", "1", True), ("block", "0", True), ("none", "1", False)):
        monkeypatch.setenv("PQG_ENS_WARP", warp)
        ens = P.Ensemble([("qg", dict(nx=64, dt=7200.0, **PHYSICS))] * 4, precision="fp32")
        ens.set_q(qs)
        if closure:
            ens.set_closure(net)
        ens.step(8)
        out[name] = [ens.q(i) for i in range(4)]
    for i in range(4):
        d = rel_l2(out["warp"][i], out["block"][i])
        assert d < 1e-3, (i, d)
        assert rel_l2(out["none"][i], out["warp"][i]) > 30 * d


@pytest.mark.parametrize("batch", [48, 160])
def test_forward_many_tiles_per_cta(batch):
    """Batches large enough that every persistent CTA processes several tiles
    (buffer and accumulator reuse across tiles)."""
    import torch
    from pyqg_gb300.closure import ConvNet
    channels = (2, 128, 64, 32, 32, 32, 32, 32, 2)
    net = ConvNet(channels, max_batch=batch, seed=5)
    p = net.params
    rng = np.random.default_rng(4)
    p += (0.05 * rng.standard_normal(p.shape)).astype(np.float32)
    net.params = p
    x = torch.from_numpy(rng.standard_normal((batch, 2, 64, 64)).astype(np.float32)).cuda()
    y = net.forward(x)
    torch.cuda.synchronize()
    ref = _torch_net(channels, p, net.layer_slices(), x)
    err = rel_l2(y.cpu().numpy(), ref.cpu().numpy())
    assert err < 1e-2, err
    # every image separately: no tile of any image may be wrong
    for b in range(batch):
        assert rel_l2(y[b].cpu().numpy(), ref[b].cpu().numpy()) < 2e-2, b


def test_gradients_many_tiles_per_cta():
    import torch
    from pyqg_gb300.closure import ConvNet
    channels = (2, 128, 64, 32, 32, 32, 32, 32, 2)
    batch = 48
    net = ConvNet(channels, max_batch=batch, seed=8)
    p = _he_params(net, 8)
    rng = np.random.default_rng(6)
    p += (0.02 * rng.standard_normal(p.shape)).astype(np.float32)
    net.params = p
    x = torch.from_numpy(rng.standard_normal((batch, 2, 64, 64)).astype(np.float32)).cuda()
    t = torch.from_numpy(rng.standard_normal((batch, 2, 64, 64)).astype(np.float32)).cuda()
    loss = net.backward(x, t)
    g = net.grads
    ref_loss, ref = _reference_grads(channels, p, net.layer_slices(), x, t)
    assert abs(loss - ref_loss) / ref_loss < 1e-2
    for (ws, shape, bs), (gw, gb) in zip(net.layer_slices(), ref):
        assert rel_l2(g[ws].reshape(shape), gw) < 5e-2
        assert rel_l2(g[bs], gb) < 5e-2


def test_default_net_learns():
    """The 8-layer network fits a fixed local linear map of its input."""
    import torch
    from pyqg_gb300.closure import ConvNet
    net = ConvNet(max_batch=32, seed=9)
    rng = np.random.default_rng(7)
    x = torch.from_numpy(rng.standard_normal((32, 2, 64, 64)).astype(np.float32)).cuda()
    lap = (torch.roll(x, 1, 2) + torch.roll(x, -1, 2) + torch.roll(x, 1, 3) + torch.roll(x, -1, 3) - 4 * x)
    t = (lap / lap.std()).contiguous()
    losses = [net.train_step(x, t, lr=1e-3) for _ in range(150)]
    assert np.all(np.isfinite(losses))
    assert losses[-1] < 0.3 * losses[0], (losses[0], losses[-1])


@pytest.mark.parametrize("channels,batch", [((2, 24, 40, 32, 2), 3), ((2, 128, 64, 32, 32, 2), 40)])
def test_row_tile_and_halo_kernels_agree(channels, batch, monkeypatch):
    """The row-tile kernel (horizontal taps folded into N) on every layer it
    takes and on the 64 -> 32 layer only, and the halo kernel (one MMA per
    tap, the default) on every layer with 64- and with 32-channel input
    units, on the same network: forward and gradients."""
    import torch
    from pyqg_gb300.closure import ConvNet
    nets = []
    for rows, unit in (("2", "64"), ("1", "64"), ("0", "64"), ("0", "32")):
        monkeypatch.setenv("PQG_CNN_ROWS", rows)
        monkeypatch.setenv("PQG_CNN_UNIT", unit)   # halo kernel: input channels per unit
        nets.append(ConvNet(channels, max_batch=batch, seed=13))
    p = _he_params(nets[0], 13)
    rng = np.random.default_rng(13)
    p += (0.02 * rng.standard_normal(p.shape)).astype(np.float32)
    for n in nets:
        n.params = p
    x = torch.from_numpy(rng.standard_normal((batch, 2, 64, 64)).astype(np.float32)).cuda()
    t = torch.from_numpy(rng.standard_normal((batch, 2, 64, 64)).astype(np.float32)).cuda()
    ys = [n.forward(x).cpu().numpy() for n in nets]
    ref = _torch_net(channels, p, nets[0].layer_slices(), x).cpu().numpy()
    for y in ys:
        assert rel_l2(y, ref) < 1e-2
        for b in range(batch):
            assert rel_l2(y[b], ref[b]) < 2e-2, b
    for y in ys[1:]:
        assert rel_l2(ys[0], y) < 1e-2
    gs = []
    for n in nets:
        n.backward(x, t)
        gs.append(n.grads)
    for ws, shape, bs in nets[0].layer_slices():
        for g in gs[1:]:
            assert rel_l2(gs[0][ws], g[ws]) < 2e-2
            assert rel_l2(gs[0][bs], g[bs]) < 2e-2


def test_pipeline_timeout_reports_and_recovers(monkeypatch):
    """The failure path of the halo-tile convolution, made to run without a
    GPU fault: the producer stops issuing copies from pipeline unit 1 on,
    so the MMA issuers' and epilogue warps' bounded waits (2 ms here) run
    out.  The kernel waits for its own MMAs and copies in flight, frees its
    tensor memory and returns; pqg_cnn_status reports PQG_ERR_TIMEOUT once,
    and the next forward is bit-identical to one taken before the fault."""
    import ctypes
    import torch
    from pyqg_gb300 import _lib
    from pyqg_gb300.closure import ConvNet
    monkeypatch.setenv("PQG_CNN_ROWS", "0")      # halo-tile kernel on every layer it takes
    channels = (2, 128, 64, 32, 2)
    batch = 48                                    # several tiles per persistent CTA
    net = ConvNet(channels, max_batch=batch, seed=21)
    L = _lib.lib()
    h = net._h
    st = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    x = torch.from_numpy(np.random.default_rng(21).standard_normal((batch, 2, 64, 64)).astype(np.float32)).cuda()
    y0 = net.forward(x).cpu().numpy()
    assert L.pqg_cnn_status(h, st) == _lib.PQG_OK
    _lib.check(L.pqg_cnn_set_fault(h, 1, 2000000))
    net.forward(x)
    rc = L.pqg_cnn_status(h, st)
    assert rc == _lib.PQG_ERR_TIMEOUT
    assert b"timed out" in L.pqg_cnn_last_error()
    assert L.pqg_cnn_status(h, st) == _lib.PQG_OK          # reported once
    _lib.check(L.pqg_cnn_set_fault(h, -1, 0))
    y1 = net.forward(x).cpu().numpy()
    assert L.pqg_cnn_status(h, st) == _lib.PQG_OK
    np.testing.assert_array_equal(y1, y0)
    ref = _torch_net(channels, net.params, net.layer_slices(), x).cpu().numpy()
    assert rel_l2(y1, ref) < 1e-2
