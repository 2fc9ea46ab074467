"""``Model.to_dataset`` (pyqg/xarray_output.py:118-174) against the dataset
the reference itself builds: ``tests/golden/dataset_qg_nx32.npz`` holds the
arguments that the reference's unchanged ``model_to_dataset`` passed to
``xarray.Dataset`` for a seeded two-layer run of four steps with every
diagnostic filled (written by ``tests/golden/make_golden.py``).

CPU: the output format (variable, coordinate and attribute names, dims,
units, long names) against the fixture; the spec of a host stand-in model;
the ImportError without xarray.  GPU: every value of the GPU model's
dataset against the reference's.
"""
import json
import sys
import types

import numpy as np
import pytest

from conftest import golden


def _fixture():
    g = golden("dataset_qg_nx32.npz")
    return g, json.loads(str(g["meta_json"]))


def test_format_matches_reference():
    from pyqg_gb300 import xarray_output as xo
    g, meta = _fixture()
    state = set(xo.VARIABLE_DIMS) | set(xo.INVERTED.values())
    seen = 0
    for name, rec in meta["vars"].items():
        if name in xo.VARIABLE_DIMS:
            assert tuple(rec["dims"]) == xo.VARIABLE_DIMS[name], name
        if name in state:
            assert rec["attrs"] == xo.VARIABLE_ATTRS[name], name
            seen += 1
        else:   # a diagnostic: time first
            assert rec["dims"][0] == "time", name
    assert seen == len(state)
    assert set(meta["coords"]) == set(xo.COORD_ATTRS)
    for name, rec in meta["coords"].items():
        assert rec["dims"] == [name] and rec["attrs"] == xo.COORD_ATTRS[name], name
    names = {"pyqg:" + n for n in xo.GLOBAL_ATTRS} | {"title", "reference"}
    assert set(meta["attrs"]) <= names
    assert meta["attrs"]["title"] == xo.TITLE and meta["attrs"]["reference"] == xo.REFERENCE


class _HostModel:
    """Host stand-in with the attributes the dataset reads."""

    def __init__(self):
        rng = np.random.default_rng(3)
        self.nz, self.ny, self.nx, self.nk, self.nl = 2, 8, 8, 5, 8
        self.t, self.tc, self.dt, self.beta = 3600.0, 1, 3600.0, 1.5e-11
        self.x, self.y = np.meshgrid(np.arange(8.0), np.arange(8.0))
        self.kk, self.ll = np.arange(5.0), np.fft.fftfreq(8) * 8
        self.q = rng.standard_normal((2, 8, 8))
        self.u, self.v = 2 * self.q, 3 * self.q
        self.ufull, self.vfull = self.u + 1, self.v
        self.qh = np.fft.rfftn(self.q, axes=(-2, -1))
        self.ph, self.uh, self.vh, self.dqhdt = 2 * self.qh, 3 * self.qh, 4 * self.qh, 5 * self.qh
        self.Ubg, self.Qy = np.array([0.025, 0.0]), np.array([1e-11, 2e-11])
        self.diagnostics = {
            "EKE": dict(dims=("lev",), description="mean eddy kinetic energy", units="m^2 s^-2"),
            "EKEdiss": dict(dims=("time",), description="total energy dissipation", units="m^2 s^-3"),
            "KEspec": dict(dims=("lev", "l", "k"), description="kinetic energy spectrum", units="m^2 s^-2"),
        }

    def ifft(self, v):
        return np.fft.irfftn(v, axes=(-2, -1), s=(8, 8))

    def get_diagnostic(self, name):
        from pyqg_gb300.errors import DiagnosticNotFilledError
        if name == "KEspec":
            raise DiagnosticNotFilledError(name)
        return {"EKE": np.array([1.0, 2.0]), "EKEdiss": np.float64(3.0)}[name]


def test_spec_of_a_host_model():
    from pyqg_gb300.xarray_output import model_to_dataset_spec
    m = _HostModel()
    data_vars, coords, attrs = model_to_dataset_spec(m)
    assert data_vars["q"][0] == ("time", "lev", "y", "x") and data_vars["q"][1].shape == (1, 2, 8, 8)
    np.testing.assert_allclose(data_vars["p"][1][0], m.ifft(m.ph))
    np.testing.assert_allclose(data_vars["dqdt"][1][0], m.ifft(m.dqhdt))
    assert data_vars["Ubg"][0] == ("lev",)
    assert data_vars["EKE"][0] == ("time", "lev") and data_vars["EKE"][1].shape == (1, 2)
    assert data_vars["EKEdiss"][0] == ("time",) and data_vars["EKEdiss"][1].shape == (1,)
    assert "KEspec" not in data_vars                     # not filled: left out
    assert coords["lev"][1].tolist() == [1, 2] and coords["lev_mid"][1].tolist() == [1.5]
    assert attrs["pyqg:beta"] == 1.5e-11 and "pyqg:rho" not in attrs


def test_to_dataset_needs_xarray(monkeypatch):
    from pyqg_gb300.xarray_output import model_to_dataset
    monkeypatch.setitem(sys.modules, "xarray", None)
    with pytest.raises(ImportError, match="Xarray"):
        model_to_dataset(_HostModel())


def test_to_dataset_hands_the_spec_to_xarray(monkeypatch):
    from pyqg_gb300.xarray_output import model_to_dataset, model_to_dataset_spec

    class _Dataset:
        def __init__(self, data_vars, coords=None, attrs=None):
            self.data_vars, self.coords, self.attrs = data_vars, coords, attrs

    stub = types.ModuleType("xarray")
    stub.Dataset = _Dataset
    monkeypatch.setitem(sys.modules, "xarray", stub)
    ds = model_to_dataset(_HostModel())
    want = model_to_dataset_spec(_HostModel())
    assert set(ds.data_vars) == set(want[0]) and ds.attrs == want[2]


@pytest.mark.gpu
def test_gpu_dataset_matches_reference():
    """Every variable, coordinate and attribute of the GPU model's dataset
    against the reference's: state within 1e-12 and diagnostics within
    1e-11 of each field's largest value; names, dims and attrs exact."""
    import pyqg_gb300 as P
    from pyqg_gb300.xarray_output import model_to_dataset_spec
    g, meta = _fixture()
    two_layer = dict(nx=32, L=1e6, beta=1.5e-11, rd=15000.0, delta=0.25, H1=500, U1=0.025, U2=0.0,
              rek=5.787e-7, dt=7200.0, filterfac=23.6)
    m = P.QGModel(**two_layer, tavestart=0.0, taveint=7200.0, log_level=0)
    m.q = g["q0"].copy()
    for _ in range(int(g["nsteps"])):
        m._step_forward()
    data_vars, coords, attrs = model_to_dataset_spec(m)
    assert set(data_vars) == set(meta["vars"])
    state = {"q", "u", "v", "ufull", "vfull", "qh", "uh", "vh", "ph", "dqhdt", "Ubg", "Qy", "p", "dqdt"}
    for name, rec in meta["vars"].items():
        dims, got, dattrs = data_vars[name]
        assert list(dims) == rec["dims"] and dattrs == rec["attrs"], name
        want = g["var_" + name]
        assert got.shape == want.shape, name
        scale = np.abs(want).max()
        tol = 1e-12 if name in state else 1e-11
        assert np.abs(got - want).max() <= tol * max(scale, 1e-300), (name, np.abs(got - want).max() / scale)
    for name, rec in meta["coords"].items():
        dims, got, cattrs = coords[name]
        assert list(dims) == rec["dims"] and cattrs == rec["attrs"], name
        np.testing.assert_allclose(got, g["coord_" + name], rtol=1e-15, err_msg=name)
    for name, want in meta["attrs"].items():
        assert name in attrs, name
        np.testing.assert_allclose(np.asarray(attrs[name], dtype=float) if name.startswith("pyqg:") else 0,
                                   np.asarray(want, dtype=float) if name.startswith("pyqg:") else 0,
                                   rtol=1e-15, err_msg=name)
