"""Checkpoint / exact resume of the time-stepping state (no counterpart in
the reference, whose snapshot output drops the Adams-Bashforth history)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TWO_LAYER = dict(L=1e6, beta=1.5e-11, rd=15000.0, delta=0.25, H1=500, U1=0.025,
          U2=0.0, rek=5.787e-7, filterfac=23.6)
QUIET = dict(tavestart=1e30, taveint=1e30, log_level=0)


@pytest.mark.parametrize("engine", ["fp64", "fixed"])
def test_resume_is_bit_exact(tmp_path, engine):
    import pyqg_gb300 as P
    q0 = 1e-7 * np.random.default_rng(3).standard_normal((2, 64, 64))
    a = P.QGModel(nx=64, dt=7200.0, tmax=40 * 7200.0, **TWO_LAYER, **QUIET)
    a.engine = engine
    a.q = q0
    a.run()
    path = tmp_path / "state.npz"
    a.save_checkpoint(path)
    a.tmax = 90 * 7200.0
    a.run()
    b = P.QGModel(nx=64, dt=7200.0, tmax=90 * 7200.0, **TWO_LAYER, **QUIET)
    b.load_checkpoint(path)
    assert (b.t, b.tc, b.ablevel, b.engine) == (40 * 7200.0, 40, 2, engine)
    b.run()
    np.testing.assert_array_equal(a.q, b.q)
    np.testing.assert_array_equal(a.qh, b.qh)
    np.testing.assert_array_equal(a.dqhdt_p, b.dqhdt_p)
    assert a.t == b.t and a.tc == b.tc


def test_checkpoint_rejects_other_grid(tmp_path):
    import pyqg_gb300 as P
    a = P.QGModel(nx=32, **QUIET)
    a.save_checkpoint(tmp_path / "s.npz")
    b = P.QGModel(nx=64, **QUIET)
    with pytest.raises(ValueError, match="does not match"):
        b.load_checkpoint(tmp_path / "s.npz")
