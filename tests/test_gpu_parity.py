"""GPU parity of the CUDA step against the reference (golden vectors made by
the reference pyqg) and against the CPU oracle.

Tolerances: FP64 transforms agree with numpy.fft/pocketfft to ~1e-15
relative; the parity gate is relative L2 on q <= 1e-12 after 100 steps.
"""
import numpy as np
import pytest

from conftest import golden, rel_l2

pytestmark = pytest.mark.gpu

TWO_LAYER = dict(L=1e6, beta=1.5e-11, rd=15000.0, delta=0.25, H1=500, U1=0.025,
          U2=0.0, rek=5.787e-7, filterfac=23.6)
TOL_STAGE = 1e-13
TOL_100 = 1e-12


@pytest.fixture(scope="module")
def P():
    import pyqg_gb300
    return pyqg_gb300


def staged_step(m):
    """One step through the per-method entry points (reference order)."""
    m._invert()
    m._do_advection()
    m._do_friction()
    if m.uv_parameterization is not None:
        m._do_uv_subgrid_parameterization()
    if m.q_parameterization is not None:
        m._do_q_subgrid_parameterization()
    m._forward_timestep()


@pytest.mark.parametrize("n", [64, 96])
def test_transforms_match_reference(P, quiet, n):
    g = golden("fft_nx%d.npz" % n)
    m = P.QGModel(nx=n, **quiet)
    # a single input plane is broadcast over the nz = 2 layers, as in the
    # reference's fft()/ifft() helpers
    xh = m.fft(g["x"])
    assert xh.shape == g["xh_of_x"].shape
    assert rel_l2(xh, g["xh_of_x"]) < 1e-14
    # inverse with non-Hermitian k=0 / Nyquist columns (their imaginary
    # parts after the y transform are ignored, as in numpy / FFTW)
    x = m.ifft(g["xh"])
    assert x.shape == g["x_of_xh"].shape
    assert rel_l2(x, g["x_of_xh"]) < 1e-14


@pytest.mark.parametrize("n", [16, 32, 128, 256, 512, 60, 80])
def test_transforms_match_numpy(P, quiet, n):
    m = P.QGModel(nx=n, **quiet)
    rng = np.random.default_rng(n)
    x = rng.standard_normal((3, n, n))
    assert rel_l2(m.fft(x), np.fft.rfftn(x, axes=(-2, -1))) < 1e-14
    xh = rng.standard_normal((3, n, n // 2 + 1)) + 1j * rng.standard_normal((3, n, n // 2 + 1))
    assert rel_l2(m.ifft(xh), np.fft.irfftn(xh, axes=(-2, -1))) < 1e-14


def test_stage_by_stage_step1(P, quiet):
    g = golden("qg_two_layer_nx64.npz")
    m = P.QGModel(nx=64, dt=7200.0, **TWO_LAYER, **quiet)
    m.q = g["q0"]
    m._invert()
    assert rel_l2(m.ph, g["s1_ph"]) < TOL_STAGE
    assert rel_l2(m.u, g["s1_u"]) < TOL_STAGE
    assert rel_l2(m.v, g["s1_v"]) < TOL_STAGE
    m._do_advection()
    assert rel_l2(m.uqh, g["s1_uqh"]) < TOL_STAGE
    assert rel_l2(m.vqh, g["s1_vqh"]) < TOL_STAGE
    m._do_friction()
    assert rel_l2(m.dqhdt, g["s1_dqhdt"]) < TOL_STAGE
    m._forward_timestep()
    assert rel_l2(m.qh, g["s1_qh"]) < TOL_STAGE
    assert rel_l2(m.q, g["q_1"]) < TOL_STAGE


def test_100_steps_nx64(P, quiet):
    """Standard two-layer physics (nx=64, dt=7200): 1e-12 gate after 100 steps."""
    g = golden("qg_two_layer_nx64.npz")
    m = P.QGModel(nx=64, dt=7200.0, tmax=100 * 7200.0, **TWO_LAYER, **quiet)
    m.q = g["q0"]
    m._step_forward()
    assert rel_l2(m.q, g["q_1"]) < TOL_STAGE
    for _ in range(9):
        m._step_forward()
    assert rel_l2(m.q, g["q_10"]) < 1e-13
    m.run()
    assert m.tc == 100 and m.t == g["t_final"]
    assert rel_l2(m.q, g["q_100"]) < TOL_100


@pytest.mark.parametrize("engine", ["fp64", "fixed"])
def test_fused_is_bit_identical_to_staged(P, quiet, engine):
    rng = np.random.default_rng(5)
    q0 = 1e-7 * rng.standard_normal((2, 64, 64))
    a = P.QGModel(nx=64, dt=7200.0, **TWO_LAYER, **quiet)
    b = P.QGModel(nx=64, dt=7200.0, **TWO_LAYER, **quiet)
    a.engine = b.engine = engine
    a.q = q0
    b.q = q0
    for _ in range(40):
        staged_step(a)
    b._step_fused(40)
    for name in ("q", "qh", "ph", "u", "v", "uq", "vq", "uqh", "vqh",
                 "dqhdt", "dqhdt_p", "dqhdt_pp"):
        np.testing.assert_array_equal(getattr(a, name), getattr(b, name), err_msg=name)
    assert (a.t, a.tc, a.ablevel) == (b.t, b.tc, b.ablevel)


def test_nx256_vs_oracle(P, quiet):
    """Standard two-layer physics (nx=256, dt=3600): golden checksums after 1 and 10
    steps, then the CPU oracle after 100 steps (1e-12 gate)."""
    import pyqg_oracle as O
    g = golden("qg_two_layer_nx256_checksums.npz")
    q0 = 1e-7 * np.random.default_rng(0).standard_normal((2, 256, 256))
    m = P.QGModel(nx=256, dt=3600.0, tmax=100 * 3600.0, **TWO_LAYER, **quiet)
    m.q = q0
    idx = g["sample_idx"]
    for s in range(1, 11):
        m._step_forward()
        if s in (1, 10):
            q = m.q
            np.testing.assert_allclose(np.sqrt((q ** 2).sum(axis=(-2, -1))),
                                       g["q%d_layer_l2" % s], rtol=1e-13)
            np.testing.assert_allclose(q[:, idx[:, 0], idx[:, 1]],
                                       g["q%d_sample" % s], rtol=1e-11, atol=1e-22)
    m.run()
    c = O.qg_constants(256)
    o = O.OracleKernel(2, 256, 256, m.a.real, m.kk, m.ll, m.Ubg, m.Qy,
                       m.filtr, m.rek, m.dt)
    o.set_q(q0)
    for _ in range(100):
        o.step()
    np.testing.assert_allclose(c["a"], m.a.real, rtol=1e-15, atol=0)
    assert rel_l2(m.q, o.q) < TOL_100


@pytest.mark.parametrize("case", ["layered_nz3_nx32", "bt_nx32", "sqg_nx32"])
def test_model_families_vs_reference(P, quiet, case):
    g = golden(case + ".npz")
    if case.startswith("layered"):
        m = P.LayeredModel(nz=3, nx=32, H=[500., 1000., 2500.], U=[0.05, 0.02, 0.0],
                           V=[0., 0., 0.], rek=5.787e-7, dt=7200.0, **quiet)
    elif case.startswith("bt"):
        m = P.BTModel(L=2. * np.pi, nx=32, beta=0., H=1., rek=0., rd=None,
                      dt=0.0025, **quiet)
    else:
        m = P.SQGModel(L=2. * np.pi, nx=32, beta=0., H=1., dt=0.0025, **quiet)
    # host constants: numpy/libm/LAPACK differ slightly across hosts (exp of
    # large negative arguments in the filter, the 3x3 inverses)
    np.testing.assert_allclose(m.a.real, g["a"], rtol=1e-13, atol=0)
    np.testing.assert_allclose(m.filtr, g["filtr"], rtol=1e-11, atol=0)
    # step with the reference's exact constants: checks the GPU step alone
    m.a = g["a"]
    m.filtr = g["filtr"]
    m.q = g["q0"]
    m._step_forward()
    assert rel_l2(m.q, g["q_1"]) < TOL_STAGE
    for _ in range(19):
        m._step_forward()
    assert rel_l2(m.q, g["q_20"]) < 1e-13


def test_parameterization_hooks_vs_reference(P, quiet):
    g = golden("qg_params_nx32.npz")
    dq, du, dv = g["param_dq"], g["param_du"], g["param_dv"]
    m = P.QGModel(nx=32, dt=7200.0, **TWO_LAYER, q_parameterization=lambda m: dq,
                  uv_parameterization=lambda m: (du, dv), **quiet)
    m.q = g["q0"]
    m._step_forward()
    assert rel_l2(m.q, g["q_1"]) < TOL_STAGE
    for _ in range(4):
        m._step_forward()
    assert rel_l2(m.q, g["q_5"]) < 1e-13


def test_layered_fixture_inversion(P):
    import json
    g = golden("layered_fixture_nx64.npz")
    params = json.loads(str(g["params_json"]))
    m = P.LayeredModel(nx=64, **params)
    np.testing.assert_allclose(m.a.real, g["a"], rtol=1e-14, atol=0)
    m.q = g["q"]
    m._invert()
    assert rel_l2(m.ph, g["ph"]) < TOL_STAGE
    assert rel_l2(m.u, g["u"]) < TOL_STAGE


@pytest.mark.parametrize("engine", ["fp64", "fixed"])
def test_engines_100_steps(P, quiet, engine):
    """Both transform engines of the fused step pass the 1e-12 gate, at
    nx=64 (vs the reference) and nx=256 (vs the oracle)."""
    import pyqg_oracle as O
    g = golden("qg_two_layer_nx64.npz")
    m = P.QGModel(nx=64, dt=7200.0, tmax=100 * 7200.0, **TWO_LAYER, **quiet)
    m.engine = engine
    m.q = g["q0"]
    m.run()
    assert rel_l2(m.q, g["q_100"]) < TOL_100
    q0 = 1e-7 * np.random.default_rng(1).standard_normal((2, 256, 256))
    m = P.QGModel(nx=256, dt=3600.0, tmax=100 * 3600.0, **TWO_LAYER, **quiet)
    m.engine = engine
    m.q = q0
    m.run()
    o = O.OracleKernel(2, 256, 256, m.a.real, m.kk, m.ll, m.Ubg, m.Qy, m.filtr, m.rek, m.dt)
    o.set_q(q0)
    for _ in range(100):
        o.step()
    assert rel_l2(m.q, o.q) < TOL_100


def test_fixed_engine_extreme_magnitudes(P, quiet):
    """Block exponents follow the data: fields from 1e-150 to the largest
    amplitude the dynamics survives step like the FP64 engine, and a zero
    field stays exactly zero."""
    rng = np.random.default_rng(9)
    m = P.QGModel(nx=64, dt=7200.0, tmax=5 * 7200.0, **TWO_LAYER, **quiet)
    m.engine = "fixed"
    m.q = np.zeros((2, 64, 64))
    m.run()
    assert not np.any(m.q)
    for scale in (1e-150, 1e-7, 1e-6):
        q0 = scale * rng.standard_normal((2, 64, 64))
        res = {}
        for engine in ("fp64", "fixed"):
            m = P.QGModel(nx=64, dt=7200.0, tmax=20 * 7200.0, **TWO_LAYER, **quiet)
            m.engine = engine
            m.q = q0
            m.run()
            res[engine] = m.q.copy()
        assert np.all(np.isfinite(res["fixed"]))
        assert rel_l2(res["fixed"], res["fp64"]) < 1e-13


def test_fixed_engine_unavailable_on_odd_sizes(P, quiet):
    m = P.QGModel(nx=96, **quiet)
    assert m.engine == "fp64"
    with pytest.raises(NotImplementedError):
        m.engine = "fixed"


@pytest.mark.parametrize("nx,ny,engines", [(64, 32, ("fp64", "fixed")), (32, 96, ("fp64",))])
def test_non_square_kernel_vs_oracle(P, nx, ny, engines):
    """ny != nx at the kernel level (the model classes refuse it, see
    test_reference_api): wavenumbers of the (ny, nx) grid, stage-by-stage
    and fused steps of each engine against the oracle after 30 steps, and
    the fused step bit-identical to the staged one."""
    import pyqg_oracle as O
    from pyqg_gb300.kernel import PseudoSpectralKernel
    from pyqg_gb300.model import spectral_filter
    from pyqg_gb300.qg_model import qg_inversion_matrix
    L, W = 1e6, 1e6 * ny / nx
    kk = 2 * np.pi / L * np.arange(nx // 2 + 1)
    ll = 2 * np.pi / W * np.append(np.arange(0., ny / 2), np.arange(-ny / 2, 0.))
    k, l = np.meshgrid(kk, ll)
    F1 = TWO_LAYER["rd"] ** -2 / (1. + TWO_LAYER["delta"])
    F2 = TWO_LAYER["delta"] * F1
    a = qg_inversion_matrix(k ** 2 + l ** 2, F1, F2)
    filtr = spectral_filter(k, l, L / nx, W / ny, TWO_LAYER["filterfac"])
    Ubg = np.array([TWO_LAYER["U1"], TWO_LAYER["U2"]])
    Qy = np.array([TWO_LAYER["beta"] + F1 * (TWO_LAYER["U1"] - TWO_LAYER["U2"]), TWO_LAYER["beta"] - F2 * (TWO_LAYER["U1"] - TWO_LAYER["U2"])])
    q0 = 1e-7 * np.random.default_rng(12).standard_normal((2, ny, nx))

    def kernel(engine):
        kn = PseudoSpectralKernel(2, ny, nx)
        kn.kk, kn.ll, kn.a, kn.Ubg, kn.Qy = kk, ll, a, Ubg, Qy
        kn.filtr, kn.rek, kn.dt = filtr, TWO_LAYER["rek"], 7200.0
        kn.engine = engine
        kn.q = q0
        return kn

    o = O.OracleKernel(2, ny, nx, a, kk, ll, Ubg, Qy, filtr, TWO_LAYER["rek"], 7200.0)
    o.set_q(q0)
    for _ in range(30):
        o.step()
    for engine in engines:
        s, f = kernel(engine), kernel(engine)
        for _ in range(30):
            s._invert()
            s._do_advection()
            s._do_friction()
            s._forward_timestep()
        f._step_fused(30)
        assert rel_l2(s.q, o.q) < TOL_100, engine
        np.testing.assert_array_equal(f.q, s.q)


@pytest.mark.parametrize("engine", ["fixed", "fp64"])
def test_nonfinite_flag_and_status_assertion(engine, quiet):
    """A NaN placed in q on the host is caught by the step kernels' flag,
    read without synchronizing; with status output on, the CFL assertion
    fails as the reference's does for a NaN state (pyqg/model.py:564-574)."""
    import pyqg_gb300 as P
    q = 1e-7 * np.random.default_rng(17).standard_normal((2, 32, 32))
    m = P.QGModel(nx=32, dt=7200.0, tmax=4 * 7200.0, **quiet)
    m.engine = engine
    m.q = q
    m.run()
    torch_sync()
    assert not m.nonfinite
    bad = q.copy()
    bad[1, 3, 5] = np.nan
    m.q = bad
    m.tmax = m.t + 3 * 7200.0
    m.run()
    torch_sync()
    assert m.nonfinite
    m.clear_nonfinite()
    assert not m.nonfinite
    loud = P.QGModel(nx=32, dt=7200.0, twrite=1, log_level=1, tavestart=1e30, taveint=1e30)
    loud.engine = engine
    loud.q = bad
    with pytest.raises(AssertionError):
        loud._step_forward()


def torch_sync():
    import torch
    torch.cuda.synchronize()
