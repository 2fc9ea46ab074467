"""pyqg's own, unchanged model classes over ``pyqg_gb300.kernel``.

The drop-in boundary is pyqg's kernel module: ``pyqg/model.py:8`` imports
``PseudoSpectralKernel`` and the ``tendency_*`` helpers from ``.kernel``, and
``Model`` derives from that class (``pyqg/model.py:22``).  These tests load
the reference's Python modules as they are (staged by
``oracle/build_ref.py``) with ``pyqg_gb300.kernel`` in place of the compiled
Cython module, then run the reference's ``QGModel``, ``LayeredModel``,
``BTModel`` and ``SQGModel`` on the GPU and compare with the golden states
that the stock reference produced.
"""
import sys

import numpy as np
import pytest

from conftest import golden, rel_l2

QUIET = dict(tavestart=1e30, taveint=1e30, log_level=0)
TWO_LAYER = dict(nx=64, L=1e6, beta=1.5e-11, rd=15000.0, delta=0.25, H1=500,
          U1=0.025, U2=0.0, rek=5.787e-7, dt=7200.0, filterfac=23.6)


def _staged():
    import ref_import
    if not ref_import.staged_available():
        pytest.skip("reference package not staged (oracle/build_ref.py with "
                    "PYQG_REFERENCE_ROOT)")
    return ref_import


@pytest.fixture(scope="module")
def ref_on_gpu_kernel():
    ref_import = _staged()
    import pyqg_gb300.kernel as K
    return ref_import.import_reference_on(K)


def test_reference_package_imports_over_gpu_kernel(ref_on_gpu_kernel):
    import pyqg_gb300.kernel as K
    pyqg = ref_on_gpu_kernel
    for cls in (pyqg.Model, pyqg.QGModel, pyqg.LayeredModel, pyqg.BTModel, pyqg.SQGModel):
        assert K.PseudoSpectralKernel in cls.__mro__
    assert pyqg.model.tendency_ab3 is K.tendency_ab3
    # the swap leaves no trace in sys.modules
    assert "pyqg" not in sys.modules or sys.modules["pyqg"] is not pyqg


def test_tendency_helpers_match_compiled_reference():
    """Module-level helpers of pyqg/kernel.pyx:640-663, bit for bit against
    the compiled reference kernel where it is built, and their typing."""
    import pyqg_gb300.kernel as K
    rng = np.random.default_rng(3)
    shp = (2, 8, 5)
    d = [rng.standard_normal(shp) + 1j * rng.standard_normal(shp) for _ in range(3)]
    dt = 3600.0
    want = [dt * d[0], 1.5 * dt * d[0] + (-0.5 * dt) * d[1],
            23 / 12. * dt * d[0] + (-16 / 12. * dt) * d[1] + 5 / 12. * dt * d[2]]
    got = [K.tendency_forward_euler(dt, d[0]), K.tendency_ab2(dt, d[0], d[1]),
           K.tendency_ab3(dt, d[0], d[1], d[2])]
    for g, w in zip(got, want):
        np.testing.assert_array_equal(g, w)
    import build_ref
    if build_ref.available():
        R = build_ref.load()
        np.testing.assert_array_equal(got[0], R.tendency_forward_euler(dt, d[0]))
        np.testing.assert_array_equal(got[1], R.tendency_ab2(dt, d[0], d[1]))
        np.testing.assert_array_equal(got[2], R.tendency_ab3(dt, d[0], d[1], d[2]))
    with pytest.raises(ValueError):
        K.tendency_forward_euler(dt, d[0].real.copy())
    with pytest.raises(ValueError):
        K.tendency_ab2(dt, d[0], d[1][0])
    with pytest.raises(TypeError):
        K.tendency_forward_euler(dt, [1j])


def _set_state(m, g):
    m.q = g["q0"].copy()


@pytest.mark.gpu
def test_unchanged_reference_qgmodel_nx64_100_steps(ref_on_gpu_kernel):
    pyqg = ref_on_gpu_kernel
    g = golden("qg_two_layer_nx64.npz")
    m = pyqg.QGModel(**TWO_LAYER, tmax=100 * TWO_LAYER["dt"], **QUIET)
    assert rel_l2(m.filtr, g["filtr"]) < 1e-12
    assert rel_l2(np.asarray(m.a).real, g["a"]) < 1e-13
    _set_state(m, g)
    m.run()
    assert m.tc == 100
    assert rel_l2(m.q, g["q_100"]) < 1e-12


@pytest.mark.gpu
def test_unchanged_reference_qgmodel_stage_by_stage(ref_on_gpu_kernel):
    """The reference's _step_forward drives the kernel's stage methods; the
    intermediate fields after one step equal the reference's."""
    pyqg = ref_on_gpu_kernel
    g = golden("qg_two_layer_nx64.npz")
    m = pyqg.QGModel(**TWO_LAYER, **QUIET)
    _set_state(m, g)
    m._invert()
    assert rel_l2(m.ph, g["s1_ph"]) < 1e-13
    assert rel_l2(m.u, g["s1_u"]) < 1e-13
    m._do_advection()
    assert rel_l2(m.uqh, g["s1_uqh"]) < 1e-13
    m._do_friction()
    assert rel_l2(m.dqhdt, g["s1_dqhdt"]) < 1e-13
    m._forward_timestep()
    assert rel_l2(m.qh, g["s1_qh"]) < 1e-13
    assert rel_l2(m.q, g["q_1"]) < 1e-13


@pytest.mark.gpu
def test_unchanged_reference_layered_bt_sqg(ref_on_gpu_kernel):
    pyqg = ref_on_gpu_kernel
    cases = [
        ("layered_nz3_nx32.npz",
         lambda: pyqg.LayeredModel(nz=3, nx=32, H=[500., 1000., 2500.], U=[0.05, 0.02, 0.0],
                                   V=[0., 0., 0.], rek=5.787e-7, dt=7200.0, **QUIET)),
        ("bt_nx32.npz",
         lambda: pyqg.BTModel(L=2. * np.pi, nx=32, beta=0., H=1., rek=0., rd=None,
                              dt=0.0025, **QUIET)),
        ("sqg_nx32.npz",
         lambda: pyqg.SQGModel(L=2. * np.pi, nx=32, beta=0., H=1., dt=0.0025, **QUIET)),
    ]
    for name, make in cases:
        g = golden(name)
        m = make()
        _set_state(m, g)
        for _ in range(20):
            m._step_forward()
        assert rel_l2(m.q, g["q_20"]) < 1e-13, name


@pytest.mark.gpu
def test_unchanged_reference_model_with_hooks(ref_on_gpu_kernel):
    """Both parameterization hooks, called by the reference's _step_forward
    (pyqg/model.py:419-425) through the kernel's hook stages."""
    pyqg = ref_on_gpu_kernel
    g = golden("qg_params_nx32.npz")
    dq, du, dv = g["param_dq"], g["param_du"], g["param_dv"]
    m = pyqg.QGModel(**dict(TWO_LAYER, nx=32), q_parameterization=lambda m: dq,
                     uv_parameterization=lambda m: (du, dv), **QUIET)
    _set_state(m, g)
    for _ in range(5):
        m._step_forward()
    assert rel_l2(m.q, g["q_5"]) < 1e-12
