"""Batched ensembles: FP64 members reproduce the single-model FP64 step bit
for bit; members are independent of their group; the FP32 form's error
against the FP64 oracle; FP64 energy and enstrophy sums."""
import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu

QUIET = dict(tavestart=1e30, taveint=1e30, log_level=0)


def _qg(seed_beta, rek, nx=64, dt=7200.0):
    return ("qg", dict(nx=nx, dt=dt, beta=seed_beta, rek=rek))


def test_fp64_members_equal_single_models():
    import pyqg_gb300 as P
    specs = [_qg(1.5e-11, 5.787e-7), _qg(2.1e-11, 3.0e-7), _qg(0.9e-11, 9.0e-7)]
    rng = np.random.default_rng(0)
    q0 = [1e-7 * rng.standard_normal((2, 64, 64)) for _ in specs]
    ens = P.Ensemble(specs, precision="fp64")
    ens.set_q(q0)
    ens.step(50)
    for i, (kind, kw) in enumerate(specs):
        m = P.QGModel(nx=64, dt=7200.0, beta=kw["beta"], rek=kw["rek"], tmax=50 * 7200.0, **QUIET)
        m.engine = "fp64"
        m.q = q0[i]
        m.run()
        np.testing.assert_array_equal(ens.q(i), m.q)


def test_members_are_independent_of_their_group():
    import pyqg_gb300 as P
    rng = np.random.default_rng(1)
    specs = [_qg(1.5e-11 * (1 + 0.1 * i), 5.787e-7) for i in range(5)]
    q0 = [1e-7 * rng.standard_normal((2, 64, 64)) for _ in specs]
    big = P.Ensemble(specs, precision="fp32")
    big.set_q(q0)
    big.step(30)
    alone = P.Ensemble([specs[3]], precision="fp32")
    alone.set_q([q0[3]])
    alone.step(30)
    np.testing.assert_array_equal(big.q(3), alone.q(0))


def test_uneven_sizes_and_layered_members():
    import pyqg_gb300 as P
    rng = np.random.default_rng(2)
    lay = dict(nz=3, H=[500., 1000., 2500.], U=[0.05, 0.02, 0.0], V=[0., 0., 0.])
    specs = [_qg(1.5e-11, 5.787e-7, nx=32), _qg(1.5e-11, 5.787e-7, nx=64),
             ("layered", dict(nx=64, dt=7200.0, **lay)), _qg(1.5e-11, 5.787e-7, nx=128)]
    q0 = []
    for kind, kw in specs:
        nz = 3 if kind == "layered" else 2
        q0.append(1e-7 * rng.standard_normal((nz, kw["nx"], kw["nx"])))
    ens = P.Ensemble(specs, precision="fp64")
    assert len(ens.groups) == 4
    ens.set_q(q0)
    ens.step(20)
    # the layered member against the single-model FP64 step
    m = P.LayeredModel(nx=64, dt=7200.0, tmax=20 * 7200.0, **lay, **QUIET)
    m.engine = "fp64"
    m.q = q0[2]
    m.run()
    np.testing.assert_array_equal(ens.q(2), m.q)
    ke, en = ens.energy()
    assert all(np.all(np.isfinite(k)) and np.all(k > 0) for k in ke)


def test_energy_sums_match_host_fp64():
    import pyqg_gb300 as P
    rng = np.random.default_rng(4)
    q0 = 1e-7 * rng.standard_normal((2, 64, 64))
    ens = P.Ensemble([_qg(1.5e-11, 5.787e-7)], precision="fp64")
    ens.set_q([q0])
    ens.step(10)
    ke, en = ens.energy()
    m = P.QGModel(nx=64, dt=7200.0, tmax=10 * 7200.0, **QUIET)
    m.engine = "fp64"
    m.q = q0
    m.run()
    m._invert()
    for z in range(2):
        np.testing.assert_allclose(ke[0][z], 0.5 * m.spec_var(m.wv * m.ph[z]), rtol=1e-12)
        np.testing.assert_allclose(en[0][z], 0.5 * m.spec_var(m.qh[z]), rtol=1e-12)


def test_fp32_form_error_vs_fp64_oracle():
    """FP32 state, transforms, products and AB3 (FP64-built matrices): the
    10-step pointwise relative L2 error on q against the FP64 oracle."""
    import pyqg_gb300 as P
    import pyqg_oracle as O
    rng = np.random.default_rng(5)
    q0 = 1e-7 * rng.standard_normal((2, 256, 256))
    ens = P.Ensemble([_qg(1.5e-11, 5.787e-7, nx=256, dt=3600.0)], precision="fp32")
    ens.set_q([q0])
    ens.step(10)
    c = O.qg_constants(256)
    o = O.OracleKernel(2, 256, 256, c["a"], c["kk"], c["ll"], c["Ubg"], c["Qy"], c["filtr"],
                       5.787e-7, 3600.0)
    o.set_q(q0)
    for _ in range(10):
        o.step()
    err = rel_l2(ens.q(0), o.q)
    print("FP32 form, nx=256, 10 steps: relative L2 error on q = %.3e" % err)
    assert err < 1e-5


def _two_groups(precision="fp64"):
    import pyqg_gb300 as P
    members = [("qg", dict(nx=64, dt=7200.0, beta=1.2e-11)), ("qg", dict(nx=128, dt=7200.0)),
               ("qg", dict(nx=64, dt=7200.0, rek=3e-7))]
    ens = P.Ensemble(members, precision=precision)
    rng = np.random.default_rng(21)
    ens.set_q([1e-6 * rng.standard_normal((2, kw["nx"], kw["nx"])) for _, kw in members])
    return ens


@pytest.mark.gpu
def test_graph_replay_equals_plain_launches(monkeypatch):
    a = _two_groups()
    monkeypatch.setenv("PQG_ENS_NO_GRAPHS", "1")
    a.step(50)
    b = _two_groups()
    monkeypatch.setenv("PQG_ENS_NO_GRAPHS", "0")
    b.step(20)
    b.step(30)          # graphs of 16 steps, then plain launches for the rest
    for i in range(3):
        np.testing.assert_array_equal(a.q(i), b.q(i))
    assert a.tc == b.tc


@pytest.mark.gpu
def test_autotune_keeps_the_state_and_results():
    a = _two_groups()
    b = _two_groups()
    a.step(5)
    b.step(5)
    choices = b.autotune()
    assert len(choices) == len(b.groups)
    for c in choices:
        assert c["rows_per_cta"] >= 1 and c["cols_per_cta"] >= 1 and c["col_ms"] > 0
    a.step(40)
    b.step(40)
    for i in range(3):
        np.testing.assert_array_equal(a.q(i), b.q(i))


def test_large_members_up_to_nx512():
    """Members of nx = 256 and 512 beside a small one: the FP64 form equals
    the single-model FP64 step bit for bit, and the FP32 form stays within
    FP32 rounding of it over a few steps."""
    import pyqg_gb300 as P
    rng = np.random.default_rng(5)
    specs = [_qg(1.5e-11, 5.787e-7, nx=512, dt=1800.0), _qg(1.2e-11, 4.0e-7, nx=256, dt=3600.0),
             _qg(1.5e-11, 5.787e-7, nx=64)]
    q0 = [1e-7 * rng.standard_normal((2, kw["nx"], kw["nx"])) for _, kw in specs]
    e64 = P.Ensemble(specs, precision="fp64")
    e32 = P.Ensemble(specs, precision="fp32")
    for e in (e64, e32):
        e.set_q(q0)
        e.step(6)
    for i in (0, 1):
        kw = specs[i][1]
        m = P.QGModel(nx=kw["nx"], dt=kw["dt"], beta=kw["beta"], rek=kw["rek"], tmax=6 * kw["dt"], **QUIET)
        m.engine = "fp64"
        m.q = q0[i]
        m.run()
        np.testing.assert_array_equal(e64.q(i), m.q)
        assert rel_l2(e32.q(i), m.q) < 1e-5


def test_member_kernel_equals_row_and_column_kernels(monkeypatch):
    """The per-member kernel (whole steps of one member per CTA, mixed planes
    in shared memory) runs the same operations as the block-wide row and
    column kernels: identical states, also through graph replay.  (FP32
    groups run the warp-owned kernels unless PQG_ENS_WARP=0.)"""
    import pyqg_gb300 as P
    monkeypatch.setenv("PQG_ENS_WARP", "0")
    rng = np.random.default_rng(7)
    lay = dict(nz=3, H=[500., 1000., 2500.], U=[0.05, 0.02, 0.0], V=[0., 0., 0.])
    specs = [_qg(1.5e-11, 5.787e-7), _qg(2.0e-11, 3.0e-7), ("layered", dict(nx=64, dt=7200.0, **lay)),
             _qg(1.1e-11, 6.0e-7, nx=32), _qg(1.5e-11, 5.787e-7, nx=16)]
    q0 = [1e-7 * rng.standard_normal((3 if k == "layered" else 2, kw["nx"], kw["nx"])) for k, kw in specs]
    out = []
    for fused in ("0", "1"):
        monkeypatch.setenv("PQG_ENS_FUSED", fused)
        e = P.Ensemble(specs, precision="fp32")
        e.set_q(q0)
        e.step(3)          # start-up steps
        e.step(37)         # graph replay of the steady state
        out.append([e.q(i) for i in range(len(specs))])
    for a, b in zip(*out):
        np.testing.assert_array_equal(a, b)


def test_member_kernel_fp64_equals_single_models(monkeypatch):
    import pyqg_gb300 as P
    monkeypatch.setenv("PQG_ENS_FUSED", "1")
    rng = np.random.default_rng(8)
    specs = [_qg(1.5e-11, 5.787e-7, nx=32), _qg(0.7e-11, 9.0e-7, nx=32)]
    q0 = [1e-7 * rng.standard_normal((2, 32, 32)) for _ in specs]
    ens = P.Ensemble(specs, precision="fp64")
    ens.set_q(q0)
    ens.step(30)
    for i, (kind, kw) in enumerate(specs):
        m = P.QGModel(nx=32, dt=7200.0, beta=kw["beta"], rek=kw["rek"], tmax=30 * 7200.0, **QUIET)
        m.engine = "fp64"
        m.q = q0[i]
        m.run()
        np.testing.assert_array_equal(ens.q(i), m.q)
    monkeypatch.delenv("PQG_ENS_FUSED")
    tuned = ens.autotune()
    assert set(tuned[0]) >= {"member_kernel", "member_threads", "member_ms_4_steps"}


def test_device_inversion_matrices_match_host_build():
    """FP64 inversion matrices built on the GPU (pqg_inversion_matrix): the
    two-layer closed forms bit for bit against the host build (the model
    classes' code, which restates pyqg/qg_model.py:146-161 and
    pyqg/layered_model.py:211-229), nz > 2 by Gauss-Jordan elimination
    within 1e-14 of each wavenumber's largest entry, the singular
    kappa = 0 entry 0."""
    from pyqg_gb300.ensemble import device_inversion_matrix
    from pyqg_gb300.layered_model import layered_inversion_matrix, stretching_matrix
    from pyqg_gb300.model import grid_constants
    from pyqg_gb300.qg_model import qg_inversion_matrix
    for nx in (64, 256):
        g = grid_constants(nx, nx, 1e6, 1e6)
        F1 = 15000.0 ** -2 / 1.25
        F2 = 0.25 * F1
        host = qg_inversion_matrix(g["wv2"], F1, F2)
        dev = device_inversion_matrix(np.array([[-F1, F1], [F2, -F2]]), g["kk"], g["ll"], True)
        np.testing.assert_array_equal(dev, host)
        f2, gg = 0.0001236812857687059 ** 2, 9.81
        for nz, H in ((2, [500., 2000.]), (3, [500., 1000., 2500.]), (4, [300., 600., 1200., 2400.]),
                      (8, [100., 150., 200., 300., 400., 500., 800., 1550.])):
            rho = np.arange(nz) * 0.3 + 1025
            gpi = gg * (rho[1:] - rho[:-1]) / rho[:-1]
            S = stretching_matrix(nz, f2, np.array(H), gpi)
            host = layered_inversion_matrix(S, g["wv2"])
            dev = device_inversion_matrix(S, g["kk"], g["ll"])
            assert np.all(dev[:, :, 0, 0] == 0)
            if nz == 2:
                np.testing.assert_array_equal(dev, host)
            else:
                scale = np.abs(host).max(axis=(0, 1))
                scale[0, 0] = 1.0
                assert (np.abs(dev - host).max(axis=(0, 1)) / scale).max() <= 1e-14, nz


def _mixed_specs():
    lay = dict(nz=3, H=[500., 1000., 2500.], U=[0.05, 0.02, 0.0], V=[0., 0., 0.])
    return [_qg(1.5e-11, 5.787e-7, nx=16), _qg(1.2e-11, 4.0e-7, nx=32), _qg(1.5e-11, 5.787e-7),
            ("layered", dict(nx=64, dt=7200.0, **lay)), _qg(1.1e-11, 6.0e-7, nx=128, dt=3600.0),
            ("layered", dict(nx=128, dt=3600.0, **lay)), _qg(1.5e-11, 5.787e-7, nx=256, dt=3600.0)]


def test_warp_kernels_match_block_kernels_and_fp64(monkeypatch):
    """The warp-owned FP32 row and column kernels (every FP32 group of
    16 <= nx <= 256 with at most three layers) take the same step as the
    block-wide FP32 kernels and as the FP64 form, up to FP32 rounding."""
    import pyqg_gb300 as P
    rng = np.random.default_rng(31)
    specs = _mixed_specs()
    q0 = [1e-7 * rng.standard_normal((3 if k == "layered" else 2, kw["nx"], kw["nx"])) for k, kw in specs]
    out = {}
    for name, prec, warp in (("warp", "fp32", "1"), ("block", "fp32", "0"), ("fp64", "fp64", "1")):
        monkeypatch.setenv("PQG_ENS_WARP", warp)
        e = P.Ensemble(specs, precision=prec)
        e.set_q(q0)
        e.step(3)
        e.step(37)
        out[name] = [e.q(i) for i in range(len(specs))]
    for i in range(len(specs)):
        ew, eb = rel_l2(out["warp"][i], out["fp64"][i]), rel_l2(out["block"][i], out["fp64"][i])
        print("member %d: warp %.2e block %.2e against FP64" % (i, ew, eb))
        assert ew < 1e-5 and eb < 1e-5, i
        assert rel_l2(out["warp"][i], out["block"][i]) < 1e-5, i


def test_warp_kernels_graphs_and_autotune_keep_results(monkeypatch):
    """FP32 groups on the warp-owned kernels: graph replay, plain launches
    and an autotuned launch shape give identical states."""
    a = _two_groups("fp32")
    b = _two_groups("fp32")
    a.step(5)
    b.step(5)
    choices = b.autotune()
    assert len(choices) == len(b.groups)
    for c in choices:
        assert c["rows_per_cta"] >= 1 and c["cols_per_cta"] >= 1 and c["col_ms"] > 0
        assert not c["member_kernel"]
    a.step(40)
    b.step(40)
    monkeypatch.setenv("PQG_ENS_NO_GRAPHS", "1")
    c = _two_groups("fp32")
    c.step(45)
    for i in range(3):
        np.testing.assert_array_equal(a.q(i), b.q(i))
        np.testing.assert_array_equal(a.q(i), c.q(i))
