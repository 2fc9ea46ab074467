"""The reference test-suite's known-answer checks, run against this package
(pyqg/tests/test_model.py, test_fft2.py, test_advection.py,
test_reference_solns.py, test_layered.py, test_parameterizations.py,
test_diagnostics.py, test_diagnostic_tools.py).  Each test names the
reference test it restates; tolerances are the reference's."""
import json

import numpy as np
import pytest

from conftest import golden

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def P():
    import pyqg_gb300
    return pyqg_gb300


@pytest.fixture
def m(P):
    # beta, U and the filter switched off, as in the reference setUp
    return P.QGModel(beta=0., U1=0., U2=0., filterfac=0.)


def waves(m):
    kmax, lmax = int(m.nx / 8), int(m.ny / 8)
    for kw in range(1, kmax):
        for lw in range(1, lmax):
            yield kw, lw, 2 * np.pi * kw / m.L, 2 * np.pi * lw / m.W


# -- pyqg/tests/test_model.py ------------------------------------------------
def test_fft2_known_amplitudes(m, rtol=1e-15):
    amp = (m.nx / 2) ** 2 * m.ny ** 2
    for kw, lw, k, l in waves(m):
        np.testing.assert_allclose(m.kk[kw], k, rtol)
        np.testing.assert_allclose(m.ll[lw], l, rtol)
        np.testing.assert_allclose(m.ll[-lw], -l, rtol)
        m.set_q1q2(np.cos(k * m.x), np.sin(l * m.y))
        qhamp = np.real(m.qh * m.qh.conj())
        np.testing.assert_allclose(qhamp[0, 0, kw], amp, rtol)
        np.testing.assert_allclose(qhamp[1, lw, 0], amp, rtol)
        np.testing.assert_allclose(qhamp[1, -lw, 0], amp, rtol)
        rest = qhamp.copy()
        rest[0, 0, kw] = rest[1, lw, 0] = rest[1, -lw, 0] = 0.
        np.testing.assert_allclose(rest, 0., rtol=0., atol=rtol)


def test_inversion_barotropic(m, rtol=1e-13):
    for kw, lw, k, l in waves(m):
        q = np.cos(k * m.x) + np.sin(l * m.y)
        u = l ** -1 * np.cos(l * m.y)
        v = k ** -1 * np.sin(k * m.x)
        m.set_q1q2(q, q)
        m._invert()
        for z in range(m.nz):
            np.testing.assert_allclose(m.u[z], u, rtol)
            np.testing.assert_allclose(m.v[z], v, rtol)


def test_change_inversion_matrix(m):
    a_new = np.random.rand(m.nz, m.nz, m.nl, m.nk)
    m.a = a_new
    np.testing.assert_allclose(a_new, m.a)


def test_advection_known_answer(m, rtol=1e-14):
    """Velocities written through the returned arrays (m.u[0] = ...)."""
    amp = (m.nx / 2) ** 2 * m.ny ** 2
    for kw, lw, k, l in waves(m):
        m.set_q1q2(np.cos(k * m.x), np.sin(l * m.y))
        m.u[0] = np.sin(k * m.x)
        m.v[0] = np.zeros_like(m.y)
        m.u[1] = np.zeros_like(m.x)
        m.v[1] = np.cos(l * m.y)
        m.set_U1U2(0., 0.)
        m._do_advection()
        d = m.dqhdt
        tabs = np.real(d * d.conj())
        np.testing.assert_allclose(tabs[0, 0, 2 * kw], k ** 2 * amp, rtol)
        np.testing.assert_allclose(tabs[1, 2 * lw, 0], l ** 2 * amp, rtol)
        np.testing.assert_allclose(tabs[1, -2 * lw, 0], l ** 2 * amp, rtol)
        rest = tabs.copy()
        rest[0, 0, 2 * kw] = rest[1, 2 * lw, 0] = rest[1, -2 * lw, 0] = 0.
        np.testing.assert_allclose(rest, 0., rtol=0., atol=rtol)


def test_friction_known_answer(m, rtol=1e-15):
    for kw, lw, k, l in waves(m):
        m.set_q1q2(np.cos(k * m.x), np.sin(l * m.y))
        m._invert()
        m.dqhdt[:] = 0.
        m._do_friction()
        expected = m.rek * m.wv2 * m.ph[-1]
        np.testing.assert_allclose(m.dqhdt[-1], expected, rtol)
        np.testing.assert_allclose(m.dqhdt[:-1], 0., rtol)


def test_q_parameterization_adds_exactly_one(P, rtol=1e-15):
    m1 = P.QGModel(beta=0., U1=0., U2=0., filterfac=0.)
    m2 = P.QGModel(beta=0., U1=0., U2=0., filterfac=0.,
                   q_parameterization=lambda m: np.ones_like(m1.q))
    m2.q = m1.q
    m1._step_forward()
    m2._step_forward()
    np.testing.assert_allclose(m2.ifft(m2.dqhdt) - m1.ifft(m1.dqhdt), 1., rtol)


def test_uv_parameterization_zero_curl(P, rtol=1e-15):
    m1 = P.QGModel(beta=0., U1=0., U2=0., filterfac=0.)

    def uv(m):
        return (np.ones_like(m.u) * np.random.normal() + np.random.normal(),
                np.ones_like(m.v) * np.random.normal() + np.random.normal())

    m2 = P.QGModel(beta=0., U1=0., U2=0., filterfac=0., uv_parameterization=uv)
    m2.q = m1.q
    m1._step_forward()
    m2._step_forward()
    np.testing.assert_allclose(m2.ifft(m2.dqhdt) - m1.ifft(m1.dqhdt), 0., rtol)


def test_uv_parameterization_nonzero_curl(P, rtol=1e-15):
    m1 = P.QGModel(beta=0., U1=0., U2=0., filterfac=0.)

    def uv(m):
        return (np.random.normal(size=m.u.shape), np.random.normal(size=m.v.shape))

    m2 = P.QGModel(beta=0., U1=0., U2=0., filterfac=0., uv_parameterization=uv)
    m2.q = m1.q
    m1._step_forward()
    m2._step_forward()
    with pytest.raises(AssertionError):
        np.testing.assert_allclose(m2.ifft(m2.dqhdt) - m1.ifft(m1.dqhdt), 0., rtol)


def test_parameterization_buffers_only_when_present(P):
    kw = dict(beta=0., U1=0., U2=0., filterfac=0.)
    m1 = P.QGModel(**kw)
    m2 = P.QGModel(q_parameterization=lambda m: None, **kw)
    m3 = P.QGModel(uv_parameterization=lambda m: None, **kw)
    m4 = P.QGModel(q_parameterization=lambda m: None,
                   uv_parameterization=lambda m: None, **kw)
    for mm in (m2, m4):
        mm.dqh
    for mm in (m3, m4):
        mm.duh
        mm.dvh
    for mm in (m1, m3):
        with pytest.raises(AttributeError):
            mm.dqh
    for mm in (m1, m2):
        with pytest.raises(AttributeError):
            mm.duh
        with pytest.raises(AttributeError):
            mm.dvh


def test_parameterization_type_inference(P):
    back, smag = P.BackscatterBiharmonic(), P.Smagorinsky()
    assert P.QGModel(parameterization=smag).uv_parameterization == smag
    assert P.QGModel(parameterization=back).q_parameterization == back
    m = P.QGModel(uv_parameterization=smag, q_parameterization=back)
    assert m.q_parameterization == back and m.uv_parameterization == smag
    with pytest.raises(ValueError):
        P.QGModel(parameterization='boop')
    with pytest.raises(AssertionError):
        P.QGModel(uv_parameterization=smag, parameterization=smag)
    with pytest.raises(AssertionError):
        P.QGModel(q_parameterization=back, parameterization=back)


def test_timestepping_fe_ab2_ab3(m):
    """A constant tendency gives exactly 1, 2, 3 dt dqhdt (FE, AB2, AB3)."""
    m.set_q(np.zeros_like(m.q))
    dqhdt = np.random.rand(*m.dqhdt.shape) + 1j * np.random.rand(*m.dqhdt.shape)
    m.dqhdt[:] = dqhdt
    assert m.tc == 0
    for n in (1, 2, 3):
        m._forward_timestep()
        np.testing.assert_allclose(m.qh, n * m.dt * dqhdt)


def test_setter_type_errors(m):
    with pytest.raises(ValueError):
        m.q = np.zeros((2, 64, 64), dtype=np.float32)
    with pytest.raises(ValueError):
        m.q = np.zeros((64, 64))
    with pytest.raises(TypeError):
        m.kk = [0.0] * m.nk


# -- pyqg/tests/test_fft2.py -------------------------------------------------
@pytest.mark.parametrize("kind", ["BT", "QG"])
def test_parseval_and_round_trip(P, kind, rtol=1e-15):
    from pyqg_gb300.diagnostic_tools import spec_var
    if kind == "BT":
        m = P.BTModel(L=2. * np.pi, beta=0., U=0., rd=0., filterfac=0)
    else:
        m = P.QGModel(L=2. * np.pi, beta=0., U1=0., U2=0., filterfac=0.)
    p1 = np.random.randn(m.nz, m.ny, m.nx)
    p1 -= p1.mean(axis=(-2, -1))[:, np.newaxis, np.newaxis]
    err = np.abs((p1.var(axis=(-2, -1)) - spec_var(m, m.fft(p1))) / p1.var(axis=(-2, -1))).sum()
    assert err < rtol
    r = np.random.randn(m.nz, m.ny, m.nx)
    r -= r.mean(axis=(-2, -1))[:, np.newaxis, np.newaxis]
    assert np.allclose(r, m.ifft(m.fft(r)), rtol=1e-5)


# -- pyqg/tests/test_advection.py --------------------------------------------
def test_plane_wave_jacobian_vanishes(P, rtol=1e-13):
    m = P.QGModel(L=2. * np.pi, nx=256, U1=0)
    for kx, ky in zip([1., 5., 10., 0., 24., 2.], [2., 0., 10., 21., 12., 49.]):
        m.set_q1q2(np.cos(kx * m.x + ky * m.y), np.zeros_like(m.x))
        m._invert()
        jac = m.ifft(m._advect(m.q, m.u, m.v))
        assert np.abs(jac).sum() * m.dx * m.dy / (m.L ** 2) < rtol


# -- pyqg/tests/test_reference_solns.py --------------------------------------
def test_reference_solution_two_layer(P):
    year = 360 * 86400.
    m = P.QGModel(nx=32, L=1e6, beta=1.5e-11, rek=5.787e-7, rd=30000.0,
                  delta=0.25, U1=0.05, U2=0.0, filterfac=18.4, dt=12800.,
                  tmax=3 * year, tavestart=1 * year, taveint=12800.,
                  useAB2=True, diagnostics_list='all')
    m.set_q1q2(1e-6 * np.cos(2 * 5 * np.pi * m.x / m.L) +
               1e-7 * np.cos(2 * 5 * np.pi * m.y / m.W), np.zeros_like(m.x))
    m.run()
    assert m.t == 93312000.0
    rtol = 0.01
    # values of the reference's two-layer solution
    np.testing.assert_allclose((m.q[0] ** 2).sum(), 9.561430503712755e-08, rtol=rtol)
    np.testing.assert_allclose(m.get_diagnostic('APEgen'), 2.5225558013107688e-07 / m.nx ** 2, rtol=rtol)
    np.testing.assert_allclose(m.get_diagnostic('EKEdiss'), 1.4806764171539711e-07 / m.nx ** 2, rtol=rtol)
    np.testing.assert_allclose(m.get_diagnostic('EKE').sum(),
                               0.00818377631732826 + 0.00015616609033468579, rtol=rtol)
    from pyqg_gb300.diagnostic_tools import spec_sum
    for name, want in (('entspec', 1.5015983257921716e-06),
                       ('APEflux', 0.00017889483037254459),
                       ('KEflux', 0.00037067750708912918),
                       ('APEgenspec', 0.00025837684260178754),
                       ('KEspec', 2 * (8581.3114357188006 + 163.75201433878425))):
        got = spec_sum(np.abs(m.get_diagnostic(name))).sum()
        np.testing.assert_allclose(got, want / m.M ** 2, rtol=rtol, err_msg=name)


def _two_gaussians(m):
    p = np.exp(-(2. * (m.x - 1.75 * np.pi / 2)) ** 2. - (2. * (m.y - np.pi)) ** 2) + \
        np.exp(-(2. * (m.x - 2.25 * np.pi / 2)) ** 2. - (2. * (m.y - np.pi)) ** 2)
    ph = m.fft(p[np.newaxis, ...])
    ke = m.spec_var(m.filtr * m.wv * ph) / 2.
    return ph / np.sqrt(ke)


def test_reference_solution_bt(P):
    m = P.BTModel(L=2. * np.pi, nx=64, tmax=5, beta=0., H=1., rek=0., rd=None,
                  dt=0.0025, twrite=1000)
    qi = m.ifft(-m.wv2 * _two_gaussians(m))
    m.set_q(qi)
    m.run()
    assert m.t == 5.000000000000082
    rtol, atol = 1.e-5, 1.e-14
    np.testing.assert_allclose((m.q ** 2).sum(), 89101.741238768518, rtol, atol)
    np.testing.assert_allclose((m.ifft(m.ph) ** 2).sum(), 1493.217664248918, rtol, atol)
    np.testing.assert_allclose(m._calc_ke(), 0.9950360837282386, rtol, atol)


def test_reference_solution_sqg(P):
    m = P.SQGModel(L=2. * np.pi, nx=64, tmax=5., beta=0., H=1., dt=0.0025, twrite=1000)
    qi = m.ifft(m.wv * _two_gaussians(m))
    m.set_q(qi)
    m.run()
    assert m.t == 5.000000000000082
    rtol, atol = 1.e-4, 1.e-14
    np.testing.assert_allclose((m.q ** 2).sum(), 7847.5169609881032, rtol, atol)
    np.testing.assert_allclose((m.ifft(m.ph) ** 2).sum(), 1346.8874163575524, rtol, atol)
    np.testing.assert_allclose(m._calc_ke(), 0.9579493831013508, rtol, atol)


# -- pyqg/tests/test_layered.py ----------------------------------------------
def test_layered_stretching_background_inversion(P):
    m = P.LayeredModel(nz=3, U=[.1, .05, .0], V=[.1, .05, .0], rho=[.1, .3, .5],
                       H=[.1, .1, .3], f=1., beta=0.)
    F11 = m.f2 / m.gpi[0] / m.Hi[0]
    F12 = m.f2 / m.gpi[0] / m.Hi[1]
    F22 = m.f2 / m.gpi[1] / m.Hi[1]
    F23 = m.f2 / m.gpi[1] / m.Hi[2]
    S = np.array([[-F11, F11, 0.], [F12, -(F12 + F22), F22], [0., F23, -F23]])
    assert np.all(m.S.sum(axis=1) == 0.)
    np.testing.assert_allclose(m.S, S, atol=1e-16)
    np.testing.assert_allclose(-S @ m.Ubg, m.Qy, atol=1e-16)
    np.testing.assert_allclose(S @ m.Vbg, m.Qx, atol=1e-16)
    M = S - np.eye(3) * m.wv2[5, 5]
    np.testing.assert_allclose(m.a[:, :, 5, 5].real, np.linalg.inv(M), atol=1e-16)


# -- pyqg/tests/test_parameterizations.py --------------------------------------
@pytest.fixture(params=["QG", "Layered", "SQG", "BT"])
def stepped(P, request):
    klass = {"QG": P.QGModel, "Layered": P.LayeredModel, "SQG": P.SQGModel,
             "BT": P.BTModel}[request.param]
    mm = klass()
    mm._step_forward()
    return mm


def test_physical_parameterizations_run(P, stepped):
    du, dv = P.Smagorinsky()(stepped)
    dq = P.BackscatterBiharmonic()(stepped)
    du2, dv2 = P.ZannaBolton2020()(stepped)
    assert du.shape == stepped.u.shape and dq.shape == stepped.q.shape
    P.RingForcing()(stepped)


def test_parameterization_addition_and_scaling(P, stepped, rtol=1e-11):
    smag, zb = P.Smagorinsky(), P.ZannaBolton2020()
    du, dv = (0.5 * smag + 0.75 * zb)(stepped)
    np.testing.assert_allclose(du, 0.5 * smag(stepped)[0] + 0.75 * zb(stepped)[0], rtol=rtol)
    np.testing.assert_allclose(dv, 0.5 * smag(stepped)[1] + 0.75 * zb(stepped)[1], rtol=rtol)


# -- pyqg/tests/test_diagnostics.py ------------------------------------------
def test_describe_diagnostics(P):
    P.QGModel(1).describe_diagnostics()


def test_paramspec_additivity(P, rtol=1e-10):
    for klass in (P.QGModel, P.LayeredModel):
        m1 = klass()
        dq = np.random.normal(size=m1.q.shape)
        du = np.random.normal(size=m1.u.shape)
        dv = np.random.normal(size=m1.v.shape)
        m2 = klass(q_parameterization=lambda m: dq)
        m3 = klass(uv_parameterization=lambda m: (du, dv))
        m4 = klass(q_parameterization=lambda m: dq, uv_parameterization=lambda m: (du, dv))
        for mm in (m1, m2, m3, m4):
            mm.q = m1.q
        for mm in (m1, m2, m3, m4):
            mm._step_forward()
            mm._increment_diagnostics()
        np.testing.assert_allclose(m1.get_diagnostic('paramspec'), 0., rtol=rtol)
        for mm in (m2, m3, m4):
            with pytest.raises(AssertionError):
                np.testing.assert_allclose(mm.get_diagnostic('paramspec'), 0., rtol=rtol)
        np.testing.assert_allclose(m2.get_diagnostic('paramspec') + m3.get_diagnostic('paramspec'),
                                   m4.get_diagnostic('paramspec'), rtol=rtol)


def test_paramspec_decomposition(P, rtol=1e-10):
    dq = np.random.normal(size=(2, 64, 64))
    m = P.QGModel(q_parameterization=lambda m: dq)
    m._step_forward()
    m._increment_diagnostics()
    hr = (m.Hi / m.H)[:, np.newaxis, np.newaxis]
    dqh = m.fft(dq)
    ps1 = -np.real((hr * np.conj(m.ph) * dqh).sum(axis=0)) / m.M ** 2
    np.testing.assert_allclose(ps1, m.get_diagnostic('paramspec'), rtol=rtol)
    ape = -np.real(hr * m.ph.conj() * np.einsum("ij, jk..., k... -> i...", m.S, m.a, dqh)).sum(axis=0) / m.M ** 2
    ke = m.wv2 * np.real(hr * m.ph.conj() * np.einsum("ij..., j... -> i...", m.a, dqh)).sum(axis=0) / m.M ** 2
    np.testing.assert_allclose(ps1, ape + ke, rtol=rtol)
    np.testing.assert_allclose(ape, m.get_diagnostic('paramspec_APEflux'), rtol=rtol)
    np.testing.assert_allclose(ke, m.get_diagnostic('paramspec_KEflux'), rtol=rtol)


def test_dissspec_consistent_with_ab3(P, atol=1e-20):
    dt = 3600
    tmax = dt * 1000
    m = P.QGModel(tavestart=tmax, taveint=1, tmax=tmax, dt=dt)
    m.run()
    m._calc_diagnostics()
    dt1, dt2, dt3 = m._ab_coefficients()
    rhs = np.zeros_like(m.qh)
    for z in range(m.nz):
        rhs[z] = m.qh[z] + dt1 * m.dqhdt[z] + dt2 * m.dqhdt_p[z] + dt3 * m.dqhdt_pp[z]
    diss = np.array([(m.filtr - 1.) * rhs[z] for z in range(m.nz)])
    contrib = -np.real(np.tensordot(m.Hi, np.conj(m.ph) * diss, axes=(0, 0))) / m.H / m.dt / m.M ** 2
    model_contrib = m.get_diagnostic('Dissspec')
    np.testing.assert_allclose(contrib, model_contrib, atol=atol)
    filt = np.array([m.filtr * rhs[z] for z in range(m.nz)])
    f1 = -np.real(np.tensordot(m.Hi, np.conj(m.ph) * filt, axes=(0, 0))) / m.H / m.dt / m.M ** 2
    f0 = -np.real(np.tensordot(m.Hi, np.conj(m.ph) * rhs, axes=(0, 0))) / m.H / m.dt / m.M ** 2
    np.testing.assert_allclose(model_contrib, f1 - f0, atol=atol)


def test_calc_ispec_peak(P):
    from pyqg_gb300.diagnostic_tools import calc_ispec
    m = P.QGModel()
    radius = np.sqrt((m.x - m.x.mean()) ** 2 + (m.y - m.y.mean()) ** 2)
    freq = m.k[0][20]
    wave = np.sin(radius * freq)
    kr, spec = calc_ispec(m, m.fft(np.array([wave, wave]))[0])
    assert np.argmax(spec) == np.argmin(np.abs(kr - freq))


def test_layered_fixture_diagnostics_run(P):
    """Every LayeredModel diagnostic evaluates on the reference fixture state."""
    g = golden("layered_fixture_nx64.npz")
    m = P.LayeredModel(nx=64, **json.loads(str(g["params_json"])))
    m.q = g["q"]
    m._invert()
    m._calc_derived_fields()
    for name, d in m.diagnostics.items():
        if name == 'Dissspec':
            continue
        assert np.all(np.isfinite(d['function'](m))), name
