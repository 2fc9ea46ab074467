"""Physical parameterizations on the device against a host (numpy)
restatement of the same formulas, and device outputs inside the step."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _stepped(P, klass=None):
    m = (klass or P.QGModel)(nx=64, dt=7200.0, tavestart=1e30, taveint=1e30, log_level=0)
    m.q = 1e-6 * np.random.default_rng(3).standard_normal((m.nz, m.ny, m.nx))
    m._step_forward()
    m._invert()
    return m


def _host_smag(m, c=0.1):
    uh, vh = m.fft(m.u), m.fft(m.v)
    Sxx, Syy = m.ifft(uh * m.ik), m.ifft(vh * m.il)
    Sxy = 0.5 * m.ifft(uh * m.il + vh * m.ik)
    nu = (c * m.dx) ** 2 * np.sqrt(2 * (Sxx ** 2 + Syy ** 2 + 2 * Sxy ** 2))
    nSxx, nSxy, nSyy = m.fft(nu * Sxx), m.fft(nu * Sxy), m.fft(nu * Syy)
    du = 2 * (m.ifft(nSxx * m.ik) + m.ifft(nSxy * m.il))
    dv = 2 * (m.ifft(nSxy * m.ik) + m.ifft(nSyy * m.il))
    return nu, du, dv


def _close(a, b, tol=1e-12):
    a, b = np.asarray(a), np.asarray(b)
    assert a.shape == b.shape
    assert np.abs(a - b).max() <= tol * np.abs(b).max()


def test_smagorinsky_and_backscatter_match_host():
    import pyqg_gb300 as P
    m = _stepped(P)
    nu, du_h, dv_h = _host_smag(m)
    du, dv = P.Smagorinsky()(m)
    assert isinstance(du, np.ndarray)
    _close(du, du_h)
    _close(dv, dv_h)
    # backscatter biharmonic (host restatement)
    lap = m.ik ** 2 + m.il ** 2
    psi = m.ifft(m.ph)
    llp = m.ifft(lap ** 2 * m.ph)
    nu8 = _host_smag(m, 0.08)[0]
    diss = -m.ifft(lap * m.fft(llp * m.dx ** 2 * nu8))
    num = np.sum(m.Hi * np.mean(psi * diss, axis=(-1, -2)))
    den = np.sum(m.Hi * np.mean(psi * llp, axis=(-1, -2))) + 1e-32
    ref = diss - 0.99 * llp * (num / den)
    _close(P.BackscatterBiharmonic()(m), ref, 1e-11)


def test_zanna_bolton_matches_host():
    import pyqg_gb300 as P
    m = _stepped(P)
    uh, vh = m.fft(m.u), m.fft(m.v)
    vx, vy, ux, uy = m.ifft(vh * m.ik), m.ifft(vh * m.il), m.ifft(uh * m.ik), m.ifft(uh * m.il)
    rv, sh, st = vx - uy, vx + uy, ux - vy
    rs, rsh = m.fft(rv * st), m.fft(rv * sh)
    ss = m.fft(rv ** 2 + sh ** 2 + st ** 2) / 2.0
    k = -46761284
    du_h = k * m.ifft(m.ik * (ss - rsh) + m.il * rs)
    dv_h = k * m.ifft(m.il * (ss + rsh) + m.ik * rs)
    du, dv = P.ZannaBolton2020()(m)
    _close(du, du_h)
    _close(dv, dv_h)


def test_ring_forcing_statistics():
    import pyqg_gb300 as P
    m = _stepped(P)
    np.random.seed(0)
    r = P.RingForcing(k_in_forc=2e-5, k_out_forc=6e-5, mag_noise_forc=3.0)(m)
    assert r.shape == (m.nz, m.ny, m.nx)
    np.testing.assert_allclose(np.abs(r).mean(axis=(-1, -2)), 3.0, rtol=1e-12)
    np.testing.assert_allclose(r.mean(axis=(-1, -2)), 0.0, atol=1e-12)


def test_hooks_return_device_tensors_in_the_step():
    import torch
    import pyqg_gb300 as P
    from pyqg_gb300.parameterizations import QParameterization, UVParameterization

    class RecQ(QParameterization):
        def __call__(self, m):
            out = P.BackscatterBiharmonic()(m)
            self.kind = type(out)
            return out

    class RecUV(UVParameterization):
        def __call__(self, m):
            out = (0.5 * P.Smagorinsky() + 0.5 * P.ZannaBolton2020())(m)
            self.kind = type(out[0])
            return out

    rq, ruv = RecQ(), RecUV()
    m = P.QGModel(nx=64, dt=7200.0, q_parameterization=rq, uv_parameterization=ruv,
                  tavestart=1e30, taveint=1e30, log_level=0)
    m.q = 1e-6 * np.random.default_rng(4).standard_normal((2, 64, 64))
    for _ in range(3):
        m._step_forward()
    assert rq.kind is torch.Tensor and ruv.kind is torch.Tensor
    assert np.all(np.isfinite(m.q))
