"""GPU advection of arbitrary fields (Model._advect) and the spectral
coarse-graining / subgrid forcing against their numpy restatements."""
import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu


def _consts(m):
    return dict(a=np.asarray(m.a), kk=np.asarray(m.kk), ll=np.asarray(m.ll), ny=m.ny, nx=m.nx)


def test_advect_matches_oracle(quiet):
    import pyqg_gb300 as P
    from coarse_oracle import advect
    m = P.QGModel(nx=64, **quiet)
    rng = np.random.default_rng(0)
    q, u, v = (rng.standard_normal((2, 64, 64)) for _ in range(3))
    got = m._advect(q, u, v)
    assert isinstance(got, np.ndarray) and got.shape == (2, 64, 33)
    ref = advect(q, u, v, np.asarray(m.kk), np.asarray(m.ll))
    assert rel_l2(got, ref) < 1e-14
    # 2-D inputs give a 2-D result (pyqg/model.py:548-557)
    got2 = m._advect(q[0], u[0], v[0])
    assert got2.shape == (64, 33)
    assert rel_l2(got2, ref[0]) < 1e-14


def test_advect_device_tensors(quiet):
    import torch
    import pyqg_gb300 as P
    m = P.QGModel(nx=64, **quiet)
    rng = np.random.default_rng(1)
    m.q = 1e-6 * rng.standard_normal((2, 64, 64))
    m._invert()
    host = m._advect(m.q)
    dev = m._advect(m.device_field("q"))
    assert isinstance(dev, torch.Tensor) and dev.is_cuda
    np.testing.assert_array_equal(dev.cpu().numpy(), host)


@pytest.mark.parametrize("nxf,nxc", [(256, 64), (128, 32)])
def test_coarse_forcing_matches_oracle(quiet, nxf, nxc):
    import torch
    import pyqg_gb300 as P
    from pyqg_gb300.coarsen import CoarseGrainer, PHYSICS
    from coarse_oracle import coarse_forcing
    fine = P.QGModel(nx=nxf, dt=3600.0, **PHYSICS, **quiet)
    coarse = P.QGModel(nx=nxc, dt=3600.0, **PHYSICS, **quiet)
    rng = np.random.default_rng(2)
    fine.q = 1e-6 * rng.standard_normal((2, nxf, nxf))
    qh = np.asarray(fine.qh).copy()
    q_c, S = CoarseGrainer(fine, coarse)()
    torch.cuda.synchronize()
    rq, rS = coarse_forcing(qh, _consts(fine), _consts(coarse))
    assert rel_l2(q_c.cpu().numpy(), rq) < 1e-13
    assert rel_l2(S.cpu().numpy(), rS) < 1e-12


def test_single_wave_has_no_subgrid_forcing(quiet):
    """J(psi, q) vanishes for a single plane wave (psi and q share the
    wavevector), so the forcing is zero to rounding."""
    import pyqg_gb300 as P
    from pyqg_gb300.coarsen import CoarseGrainer, PHYSICS
    fine = P.QGModel(nx=128, dt=3600.0, **PHYSICS, **quiet)
    coarse = P.QGModel(nx=32, dt=3600.0, **PHYSICS, **quiet)
    x, y = np.meshgrid(np.asarray(fine.x)[0], np.asarray(fine.y)[:, 0])
    k0, l0 = 3 * 2 * np.pi / fine.L, 5 * 2 * np.pi / fine.W
    wave = np.cos(k0 * x + l0 * y)
    fine.q = np.stack([1e-6 * wave, -3e-7 * wave])
    q_c, S = CoarseGrainer(fine, coarse)()
    fine._invert()
    scale = np.abs(fine.u).max() * np.abs(fine.q).max() * np.hypot(k0, l0)
    assert np.abs(S.cpu().numpy()).max() < 1e-12 * scale
    # the wave is inside the coarse band: filtered q is the wave itself
    assert rel_l2(q_c.cpu().numpy(), np.asarray(fine.q)[:, ::4, ::4]) < 1e-13


def test_training_data_pipeline(quiet):
    import torch
    import pyqg_gb300 as P
    from pyqg_gb300.coarsen import CoarseGrainer, PHYSICS, generate_training_data, channel_stats
    X, Y = generate_training_data(nruns=3, nx_fine=128, nx_coarse=32, dt=3600.0, spinup_steps=20,
                                  snapshot_interval=10, nsnapshots=2, seed0=2000)
    assert X.shape == (6, 2, 32, 32) and Y.shape == (6, 2, 32, 32)
    assert torch.isfinite(X).all() and torch.isfinite(Y).all()
    # sample (snapshot 1, run 2) equals a single model advanced the same way
    m = P.QGModel(nx=128, dt=3600.0, **PHYSICS, **quiet)
    m.engine = "fp64"   # the FP64 ensemble matches the FP64-transform engine bit for bit
    m.q = 1e-7 * np.random.default_rng(2002).standard_normal((2, 128, 128))
    m._step_fused(30)
    m.q = np.array(m.q)   # the pipeline takes snapshots of q (qh = rfft2(q))
    coarse = P.QGModel(nx=32, dt=3600.0, **PHYSICS, **quiet)
    q_c, S = CoarseGrainer(m, coarse)()
    np.testing.assert_allclose(X[5].cpu().numpy(), q_c.float().cpu().numpy(), rtol=0, atol=0)
    np.testing.assert_allclose(Y[5].cpu().numpy(), S.float().cpu().numpy(), rtol=0, atol=0)
    mean, std = channel_stats(X)
    assert mean.shape == (2,) and np.all(std > 0)
