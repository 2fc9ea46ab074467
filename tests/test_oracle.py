"""CPU tests: the oracle against the reference's golden vectors (and against
the live reference when its tree is present), with planted-mistake checks
showing the comparisons can fail."""
import numpy as np
import pytest

from conftest import golden, rel_l2
import pyqg_oracle as O


def oracle_from(g, nz, n, q_param=None, uv_param=None):
    o = O.OracleKernel(nz, n, n, g["a"], g["kk"], g["ll"], g["Ubg"], g["Qy"],
                       g["filtr"], g["rek"], g["dt"])
    o.set_q(g["q0"])
    return o


@pytest.mark.parametrize("case,nz,n,steps", [
    ("qg_two_layer_nx64.npz", 2, 64, (1, 10, 100)),
    ("layered_nz3_nx32.npz", 3, 32, (1, 20)),
    ("bt_nx32.npz", 1, 32, (1, 20)),
    ("sqg_nx32.npz", 1, 32, (1, 20)),
])
def test_oracle_bit_identical_to_reference(case, nz, n, steps):
    """The oracle repeats the reference arithmetic with the same FFT
    (pocketfft), so its states equal the reference's bit for bit."""
    g = golden(case)
    o = oracle_from(g, nz, n)
    done = 0
    for s in steps:
        while done < s:
            o.step()
            done += 1
        np.testing.assert_array_equal(o.q, g["q_%d" % s])
    assert o.t == g["t_final"]


def test_oracle_stages_step1():
    g = golden("qg_two_layer_nx64.npz")
    o = oracle_from(g, 2, 64)
    o.invert()
    np.testing.assert_array_equal(o.ph, g["s1_ph"])
    np.testing.assert_array_equal(o.u, g["s1_u"])
    np.testing.assert_array_equal(o.v, g["s1_v"])
    o.do_advection()
    np.testing.assert_array_equal(o.uqh, g["s1_uqh"])
    np.testing.assert_array_equal(o.vqh, g["s1_vqh"])
    o.do_friction()
    np.testing.assert_array_equal(o.dqhdt, g["s1_dqhdt"])
    o.forward_timestep()
    np.testing.assert_array_equal(o.qh, g["s1_qh"])


def test_oracle_parameterization_hooks():
    g = golden("qg_params_nx32.npz")
    o = oracle_from(g, 2, 32)
    qp = lambda m: g["param_dq"]
    uvp = lambda m: (g["param_du"], g["param_dv"])
    for s in range(1, 6):
        o.step(q_param=qp, uv_param=uvp)
        if s in (1, 5):
            np.testing.assert_array_equal(o.q, g["q_%d" % s])


def test_oracle_nx256_checksums():
    g = golden("qg_two_layer_nx256_checksums.npz")
    c = O.qg_constants(256)
    o = O.OracleKernel(c["nz"], 256, 256, c["a"], c["kk"], c["ll"], c["Ubg"],
                       c["Qy"], c["filtr"], 5.787e-7, 3600.0)
    o.set_q(1e-7 * np.random.default_rng(0).standard_normal((2, 256, 256)))
    idx = g["sample_idx"]
    for s in range(1, 11):
        o.step()
        if s in (1, 10):
            np.testing.assert_allclose(np.sqrt((o.q ** 2).sum(axis=(-2, -1))),
                                       g["q%d_layer_l2" % s], rtol=1e-14)
            np.testing.assert_allclose(o.q[:, idx[:, 0], idx[:, 1]],
                                       g["q%d_sample" % s], rtol=1e-12, atol=1e-24)


@pytest.mark.parametrize("n", [64, 96])
def test_oracle_transform_conventions(n):
    # the reference's fft()/ifft() broadcast a single plane over nz = 2
    g = golden("fft_nx%d.npz" % n)
    for z in range(2):
        np.testing.assert_array_equal(O.rfft2(g["x"])[0], g["xh_of_x"][z])
        np.testing.assert_array_equal(O.irfft2(g["xh"])[0], g["x_of_xh"][z])


def test_planted_mistake_is_detected():
    """A wrong sign in the drag (planted in a copy of the oracle) must fail
    the same comparison the real tests use."""
    g = golden("qg_two_layer_nx64.npz")

    class Broken(O.OracleKernel):
        def do_friction(self):
            self.dqhdt[-1] = self.dqhdt[-1] - (self.rek * self._k2l2 * self.ph[-1])

    o = Broken(2, 64, 64, g["a"], g["kk"], g["ll"], g["Ubg"], g["Qy"],
               g["filtr"], g["rek"], g["dt"])
    o.set_q(g["q0"])
    for _ in range(10):
        o.step()
    assert rel_l2(o.q, g["q_10"]) > 1e-12


@pytest.mark.skipif(not __import__("ref_import").reference_available(),
                    reason="reference tree not present")
def test_oracle_vs_live_reference_nx96():
    """Against the reference itself (container with the reference tree):
    non-power-of-two grid, LayeredModel nz=2 closed-form inversion."""
    from ref_import import import_reference_pyqg
    pyqg = import_reference_pyqg()
    m = pyqg.QGModel(nx=96, dt=3600., tavestart=1e30, taveint=1e30, log_level=0)
    q0 = 1e-7 * np.random.default_rng(3).standard_normal((2, 96, 96))
    m.q = q0
    o = O.OracleKernel(2, 96, 96, m.a.real, m.kk, m.ll, m.Ubg, m.Qy, m.filtr,
                       m.rek, m.dt)
    o.set_q(q0)
    for _ in range(30):
        m._step_forward()
        o.step()
    np.testing.assert_array_equal(o.q, m.q)


def test_reference_multithreaded_fft_variant_is_bit_identical():
    """The CPU baseline's multithreaded-FFT variant of the compiled reference
    kernel (its FFT hooks on scipy.fft workers) gives the stock kernel's
    states bit for bit."""
    import os
    import sys
    build_ref = pytest.importorskip("build_ref")
    if not build_ref.available():
        pytest.skip("compiled reference kernel not built")
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench
    from pyqg_gb300.model import grid_constants, spectral_filter
    from pyqg_gb300.qg_model import qg_inversion_matrix
    mod = build_ref.load()
    nx, phys = 64, bench.TWO_LAYER
    g = grid_constants(nx, nx, phys["L"], phys["L"])
    F1 = phys["rd"] ** -2 / (1. + phys["delta"])
    F2 = phys["delta"] * F1
    q0 = 1e-7 * np.random.default_rng(4).standard_normal((2, nx, nx))
    out = []
    for workers in (0, 4):
        k = bench._ref_kernel(mod, workers)(2, nx, nx, 1, 0, 0)
        k.ll, k.kk = g["ll"], g["kk"]
        k.a = qg_inversion_matrix(g["wv2"], F1, F2)
        k.Ubg = np.array([phys["U1"], phys["U2"]])
        k.Qy = np.array([phys["beta"] + F1 * (phys["U1"] - phys["U2"]), phys["beta"] - F2 * (phys["U1"] - phys["U2"])])
        k.filtr = spectral_filter(g["k"], g["l"], g["dx"], g["dy"], phys["filterfac"])
        k.rek, k.dt = phys["rek"], 3600.0
        k.q = q0
        for _ in range(20):
            k._invert()
            k._do_advection()
            k._do_friction()
            k._forward_timestep()
        out.append(np.array(k.q))
    np.testing.assert_array_equal(out[0], out[1])
