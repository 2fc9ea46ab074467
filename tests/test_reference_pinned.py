"""Physical parameterizations and diagnostics pinned to the reference's own
outputs (fixtures written by ``tests/golden/make_golden.py`` from the stock
reference package):

* ``params_physical_nx32.npz``: Smagorinsky, BackscatterBiharmonic,
  ZannaBolton2020 and RingForcing (``pyqg/parameterizations.py:132-366``) on
  a seeded two-layer state at nx=32;
* ``diag_*.npz``: every registered diagnostic (time averages and counts,
  ``pyqg/model.py:802-814``) of short seeded runs of the two-layer and the
  three-layer model, and of runs with a uv and a q parameterization.

The CPU tests check the numpy restatement of the parameterization formulas
(the second line of the GPU tests in ``test_parameterizations_gpu.py``)
against the fixtures; the GPU tests check the device implementations.
"""
import numpy as np
import pytest

from conftest import golden

TWO_LAYER = dict(L=1e6, beta=1.5e-11, rd=15000.0, delta=0.25, H1=500, U1=0.025,
          U2=0.0, rek=5.787e-7, dt=7200.0, filterfac=23.6)
PARAM_TOL = 1e-12
DIAG_TOL = 1e-11


def close(got, want, tol, what=""):
    """max |got - want| <= tol * max |want|, with NaNs in the same places
    (RingForcing divides the unforced layers by zero, as the reference does)."""
    got, want = np.asarray(got), np.asarray(want)
    assert got.shape == want.shape, what
    nan = np.isnan(want)
    assert np.array_equal(np.isnan(got), nan), what
    g, w = got[~nan], want[~nan]
    scale = np.abs(w).max() if w.size else 0.0
    err = np.abs(g - w).max() if w.size else 0.0
    assert err <= tol * scale, (what, err / scale if scale else err)


class _HostModel:
    """numpy stand-in for the few model attributes the formulas read."""

    def __init__(self, g):
        self.nz, self.ny, self.nx = g["u"].shape
        self.k, self.l = np.meshgrid(g["kk"], g["ll"])
        self.wv = np.sqrt(self.k ** 2 + self.l ** 2)
        self.ik, self.il = 1j * self.k, 1j * self.l
        self.dx, self.Hi = float(g["dx"]), g["Hi"]
        self.u, self.v, self.ph = g["u"], g["v"], g["ph"]

    def fft(self, x):
        return np.fft.rfftn(x, axes=(-2, -1))

    def ifft(self, x):
        return np.fft.irfftn(x, axes=(-2, -1), s=(self.ny, self.nx))


def _host_smag(m, c=0.1):
    uh, vh = m.fft(m.u), m.fft(m.v)
    Sxx, Syy = m.ifft(uh * m.ik), m.ifft(vh * m.il)
    Sxy = 0.5 * m.ifft(uh * m.il + vh * m.ik)
    nu = (c * m.dx) ** 2 * np.sqrt(2 * (Sxx ** 2 + Syy ** 2 + 2 * Sxy ** 2))
    nSxx, nSxy, nSyy = m.fft(nu * Sxx), m.fft(nu * Sxy), m.fft(nu * Syy)
    du = 2 * (m.ifft(nSxx * m.ik) + m.ifft(nSxy * m.il))
    dv = 2 * (m.ifft(nSxy * m.ik) + m.ifft(nSyy * m.il))
    return nu, du, dv


def _host_backscatter(m, cs=0.08, cb=0.99, eps=1e-32):
    lap = m.ik ** 2 + m.il ** 2
    psi = m.ifft(m.ph)
    llp = m.ifft(lap ** 2 * m.ph)
    diss = -m.ifft(lap * m.fft(llp * m.dx ** 2 * _host_smag(m, cs)[0]))
    num = np.sum(m.Hi * np.mean(psi * diss, axis=(-1, -2)))
    den = np.sum(m.Hi * np.mean(psi * llp, axis=(-1, -2))) + eps
    return diss - cb * llp * (num / den)


def _host_zb(m, kappa=-46761284):
    uh, vh = m.fft(m.u), m.fft(m.v)
    vx, vy, ux, uy = m.ifft(vh * m.ik), m.ifft(vh * m.il), m.ifft(uh * m.ik), m.ifft(uh * m.il)
    rv, sh, st = vx - uy, vx + uy, ux - vy
    rs, rsh = m.fft(rv * st), m.fft(rv * sh)
    ss = m.fft(rv ** 2 + sh ** 2 + st ** 2) / 2.0
    return (kappa * m.ifft(m.ik * (ss - rsh) + m.il * rs),
            kappa * m.ifft(m.il * (ss + rsh) + m.ik * rs))


def test_host_restatement_of_parameterizations_matches_reference():
    g = golden("params_physical_nx32.npz")
    m = _HostModel(g)
    nu, du, dv = _host_smag(m)
    close(nu, g["smag_nu"], PARAM_TOL, "smag nu")
    close(du, g["smag_du"], PARAM_TOL, "smag du")
    close(dv, g["smag_dv"], PARAM_TOL, "smag dv")
    _, du, dv = _host_smag(m, 0.2)
    close(du, g["smag02_du"], PARAM_TOL, "smag 0.2 du")
    close(_host_backscatter(m), g["back_dq"], PARAM_TOL, "backscatter")
    close(_host_backscatter(m, 0.1, 0.5), g["back05_dq"], PARAM_TOL, "backscatter 0.1/0.5")
    du, dv = _host_zb(m)
    close(du, g["zb_du"], PARAM_TOL, "zb du")
    close(dv, g["zb_dv"], PARAM_TOL, "zb dv")


def _gpu_model_at(P, g):
    m = P.QGModel(nx=g["u"].shape[-1], **TWO_LAYER, tavestart=1e30, taveint=1e30, log_level=0)
    m.q = g["q"].copy()
    m._invert()
    close(m.ph, g["ph"], 1e-13, "ph")
    close(m.u, g["u"], 1e-13, "u")
    close(m.v, g["v"], 1e-13, "v")
    return m


@pytest.mark.gpu
def test_gpu_parameterizations_match_reference():
    import pyqg_gb300 as P
    g = golden("params_physical_nx32.npz")
    m = _gpu_model_at(P, g)
    du, dv = P.Smagorinsky()(m)
    close(du, g["smag_du"], PARAM_TOL, "smag du")
    close(dv, g["smag_dv"], PARAM_TOL, "smag dv")
    close(P.Smagorinsky()(m, just_viscosity=True), g["smag_nu"], PARAM_TOL, "smag nu")
    du, dv = P.Smagorinsky(constant=0.2)(m)
    close(du, g["smag02_du"], PARAM_TOL, "smag 0.2 du")
    close(dv, g["smag02_dv"], PARAM_TOL, "smag 0.2 dv")
    close(P.BackscatterBiharmonic()(m), g["back_dq"], PARAM_TOL, "backscatter")
    close(P.BackscatterBiharmonic(smag_constant=0.1, back_constant=0.5)(m), g["back05_dq"],
          PARAM_TOL, "backscatter 0.1/0.5")
    du, dv = P.ZannaBolton2020()(m)
    close(du, g["zb_du"], PARAM_TOL, "zb du")
    close(dv, g["zb_dv"], PARAM_TOL, "zb dv")
    ring = dict(k_in_forc=2e-5, k_out_forc=6e-5, mag_noise_forc=3.0)
    for seed, layers in zip(g["ring_seeds"], ("all", "surf", "bottom")):
        np.random.seed(int(seed))
        with np.errstate(invalid="ignore"):
            out = P.RingForcing(layers=layers, **ring)(m)
        close(out, g["ring_%s_dq" % layers], PARAM_TOL, "ring " + layers)


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["diag_qg_nx64.npz", "diag_layered_nz3_nx32.npz",
                                  "diag_qg_smag_nx32.npz", "diag_qg_back_nx32.npz"])
def test_gpu_diagnostics_match_reference(name):
    """Each diagnostic, per bin, within 1e-11 of its largest value."""
    import pyqg_gb300 as P
    g = golden(name)
    lay = dict(nz=3, H=[500., 1000., 2500.], U=[0.05, 0.02, 0.0], V=[0., 0., 0.],
               rek=5.787e-7, dt=7200.0)
    diag = dict(tavestart=0.0, taveint=7200.0, log_level=0)
    make = {
        "diag_qg_nx64.npz": lambda: P.QGModel(nx=64, **TWO_LAYER, **diag),
        "diag_layered_nz3_nx32.npz": lambda: P.LayeredModel(nx=32, **lay, **diag),
        "diag_qg_smag_nx32.npz": lambda: P.QGModel(nx=32, uv_parameterization=P.Smagorinsky(),
                                                   **TWO_LAYER, **diag),
        "diag_qg_back_nx32.npz": lambda: P.QGModel(nx=32, q_parameterization=P.BackscatterBiharmonic(),
                                                   **TWO_LAYER, **diag),
    }[name]
    m = make()
    assert m.gpu_diagnostics
    m.q = g["q0"].copy()
    for _ in range(int(g["nsteps"])):
        m._step_forward()
    close(m.q, g["q"], 1e-12, "q")
    names = [str(n) for n in g["names"]]
    assert len(names) >= 19
    for n in names:
        assert m.diagnostics[n]["count"] == int(g["count_" + n]), n
        assert "_acc" in m.diagnostics[n], n     # accumulated on the device
        want = g["diag_" + n]
        got = np.asarray(m.get_diagnostic(n))
        if np.abs(want).max() == 0:
            assert np.abs(got).max() == 0, n
        else:
            close(got, want, DIAG_TOL, n)
