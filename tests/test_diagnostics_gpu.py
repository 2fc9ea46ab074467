"""Diagnostics accumulated on the GPU (FP64, pqg_diag_accumulate) against the
host formulas of the same diagnostics on the same trajectory."""
import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu


def _pair(cls, nsteps, **kw):
    out = []
    for gpu in (True, False):
        m = cls(tavestart=0.0, taveint=kw.get("dt", 7200.0), log_level=0, **kw)
        m.gpu_diagnostics = gpu
        rng = np.random.default_rng(11)
        m.q = 1e-6 * rng.standard_normal((m.nz, m.ny, m.nx))
        for _ in range(nsteps):
            m._step_forward()
        out.append(m)
    return out


def _compare(mg, mh, names=None):
    names = names or [n for n, d in mh.diagnostics.items() if d["active"]]
    checked = 0
    for n in names:
        dg, dh = mg.diagnostics[n], mh.diagnostics[n]
        if "value" not in dh:
            continue
        assert dg["count"] == dh["count"], n
        vg, vh = np.asarray(mg.get_diagnostic(n)), np.asarray(mh.get_diagnostic(n))
        assert vg.shape == vh.shape, n
        scale = np.abs(vh).max()
        if scale == 0:
            assert np.abs(vg).max() == 0, n
        else:
            assert np.abs(vg - vh).max() <= 1e-11 * scale, (n, np.abs(vg - vh).max() / scale)
        assert "_acc" in dg, n          # really accumulated on the device
        checked += 1
    return checked


def test_qg_diagnostics_on_gpu():
    import pyqg_gb300 as P
    mg, mh = _pair(P.QGModel, 6, nx=64, dt=7200.0)
    assert _compare(mg, mh) >= 18
    # the reference's entry layout: 'value' is the accumulated sum
    np.testing.assert_allclose(mg.diagnostics["KEspec"]["value"], mh.diagnostics["KEspec"]["value"],
                               rtol=1e-11, atol=0)


def test_layered_diagnostics_on_gpu():
    import pyqg_gb300 as P
    mg, mh = _pair(P.LayeredModel, 5, nx=64, nz=3, dt=7200.0, H=[500.0, 1000.0, 2500.0],
                   U=[0.05, 0.02, 0.0], V=[0.0, 0.0, 0.0])
    assert _compare(mg, mh) >= 15


def test_parameterization_diagnostics_on_gpu():
    import pyqg_gb300 as P
    from pyqg_gb300.parameterizations import Smagorinsky, BackscatterBiharmonic
    for kw in (dict(uv_parameterization=Smagorinsky()), dict(q_parameterization=BackscatterBiharmonic())):
        mg, mh = _pair(P.QGModel, 4, nx=64, dt=7200.0, **kw)
        _compare(mg, mh, ["paramspec", "ENSparamspec", "paramspec_APEflux", "paramspec_KEflux"])


def test_user_diagnostic_stays_on_host():
    import pyqg_gb300 as P
    m = P.QGModel(nx=64, dt=7200.0, tavestart=0.0, taveint=7200.0, log_level=0)
    m.add_diagnostic("qmax", description="max q", function=lambda mm: np.abs(mm.q).max(),
                     units="s^-1", dims=("time",))
    m.q = 1e-6 * np.random.default_rng(1).standard_normal((2, 64, 64))
    for _ in range(3):
        m._step_forward()
    assert "_acc" not in m.diagnostics["qmax"]
    assert m.diagnostics["qmax"]["count"] == m.diagnostics["KEspec"]["count"]
    assert rel_l2(m.get_diagnostic("EKE"), m.get_diagnostic("EKE")) == 0
