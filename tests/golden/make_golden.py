"""Generate the golden fixtures in this folder from the reference pyqg.

Run in a container that has the reference tree (it imports the reference
package in place and its Cython kernel compiled by ``oracle/build_ref.py``):

    python tests/golden/make_golden.py

Every fixture holds the reference's own constants, inputs and outputs for a
seeded case, so the CPU oracle and the GPU path can be checked against the
reference on a machine where the reference is absent.
"""
import json
import os
import pickle
import sys
import warnings

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(REPO, "oracle"))
from ref_import import import_reference_pyqg, REF_ROOT  # noqa: E402

QUIET = dict(tavestart=1e30, taveint=1e30, log_level=0)


def consts(m):
    return dict(a=np.asarray(m.a).real.copy(), kk=np.asarray(m.kk).copy(),
                ll=np.asarray(m.ll).copy(), Ubg=np.asarray(m.Ubg).copy(),
                Qy=np.asarray(m.Qy).copy(), filtr=np.asarray(m.filtr).copy(),
                rek=np.float64(m.rek), dt=np.float64(m.dt))


def run_case(m, q0, steps, stage_step1=True, q_param=None):
    m.q = q0
    out = dict(q0=q0.copy())
    out.update(consts(m))
    done = 0
    for s in sorted(steps):
        while done < s:
            if done == 0 and stage_step1:
                m._invert()
                out["s1_ph"] = np.asarray(m.ph).copy()
                out["s1_u"] = np.asarray(m.u).copy()
                out["s1_v"] = np.asarray(m.v).copy()
                m._do_advection()
                out["s1_uqh"] = np.asarray(m.uqh).copy()
                out["s1_vqh"] = np.asarray(m.vqh).copy()
                m._do_friction()
                if m.uv_parameterization is not None:
                    m._do_uv_subgrid_parameterization()
                if m.q_parameterization is not None:
                    m._do_q_subgrid_parameterization()
                out["s1_dqhdt"] = np.asarray(m.dqhdt).copy()
                m._forward_timestep()
                out["s1_qh"] = np.asarray(m.qh).copy()
            else:
                m._step_forward()
            done += 1
        out["q_%d" % s] = np.asarray(m.q).copy()
    out["t_final"] = np.float64(m.t)
    return out


def main():
    pyqg = import_reference_pyqg()
    rng = np.random.default_rng
    files = {}

    # Config-1 two-layer physics at nx=64 (seed 0), 100 steps.
    c1 = dict(nx=64, L=1e6, beta=1.5e-11, rd=15000.0, delta=0.25, H1=500,
              U1=0.025, U2=0.0, rek=5.787e-7, dt=7200.0, filterfac=23.6)
    m = pyqg.QGModel(**c1, **QUIET)
    q0 = 1e-7 * rng(0).standard_normal((2, 64, 64))
    files["qg_c1_nx64.npz"] = run_case(m, q0, [1, 10, 100])

    # Config-2 physics at nx=256, dt=3600 (seed 0): checksums only (size).
    c2 = dict(c1, nx=256, dt=3600.0)
    m = pyqg.QGModel(**c2, **QUIET)
    q0 = 1e-7 * rng(0).standard_normal((2, 256, 256))
    m.q = q0
    idx = rng(7).integers(0, 256, size=(64, 2))
    rec = dict(seed=np.int64(0), sample_idx=idx)
    for s in range(1, 11):
        m._step_forward()
        if s in (1, 10):
            q = np.asarray(m.q)
            rec["q%d_layer_l2" % s] = np.sqrt((q ** 2).sum(axis=(-2, -1)))
            rec["q%d_layer_sum" % s] = q.sum(axis=(-2, -1))
            rec["q%d_sample" % s] = q[:, idx[:, 0], idx[:, 1]].copy()
    files["qg_c2_nx256_checksums.npz"] = rec

    # Three-layer LayeredModel (the ensemble's nz=3 physics) at nx=32.
    lay = dict(nz=3, nx=32, H=[500., 1000., 2500.], U=[0.05, 0.02, 0.0],
               V=[0., 0., 0.], rek=5.787e-7, dt=7200.0)
    m = pyqg.LayeredModel(**lay, **QUIET)
    q0 = 1e-7 * rng(1).standard_normal((3, 32, 32))
    files["layered_nz3_nx32.npz"] = run_case(m, q0, [1, 20])

    # Barotropic and SQG single-layer models.
    m = pyqg.BTModel(L=2. * np.pi, nx=32, beta=0., H=1., rek=0., rd=None,
                     dt=0.0025, **QUIET)
    q0 = 1e-3 * rng(2).standard_normal((1, 32, 32))
    files["bt_nx32.npz"] = run_case(m, q0, [1, 20])
    m = pyqg.SQGModel(L=2. * np.pi, nx=32, beta=0., H=1., dt=0.0025, **QUIET)
    q0 = 1e-3 * rng(3).standard_normal((1, 32, 32))
    files["sqg_nx32.npz"] = run_case(m, q0, [1, 20])

    # q and uv parameterization hooks with fixed, seeded forcings.
    dq = 1e-13 * rng(4).standard_normal((2, 32, 32))
    du = 1e-9 * rng(5).standard_normal((2, 32, 32))
    dv = 1e-9 * rng(6).standard_normal((2, 32, 32))
    cp = dict(c1, nx=32)
    m = pyqg.QGModel(**cp, q_parameterization=lambda m: dq,
                     uv_parameterization=lambda m: (du, dv), **QUIET)
    q0 = 1e-7 * rng(8).standard_normal((2, 32, 32))
    rec = run_case(m, q0, [1, 5])
    rec.update(param_dq=dq, param_du=du, param_dv=dv)
    files["qg_params_nx32.npz"] = rec

    # Transform conventions, incl. a non-power-of-two size (nx=96) and
    # non-Hermitian k=0 / Nyquist columns on the inverse.
    for n in (64, 96):
        mm = pyqg.QGModel(nx=n, **QUIET)
        x = rng(10 + n).standard_normal((1, n, n))
        xh = (rng(20 + n).standard_normal((1, n, n // 2 + 1))
              + 1j * rng(30 + n).standard_normal((1, n, n // 2 + 1)))
        files["fft_nx%d.npz" % n] = dict(x=x, xh_of_x=mm.fft(x), xh=xh,
                                         x_of_xh=mm.ifft(xh))

    # The reference's own LayeredModel fixture state at nx=64: one inversion.
    fx = os.path.join(REF_ROOT, "pyqg", "tests", "fixtures")
    with open(os.path.join(fx, "LayeredModel_params.pkl"), "rb") as f:
        params = pickle.load(f)
    m = pyqg.LayeredModel(nx=64, **params)
    m.q = np.load(os.path.join(fx, "LayeredModel_nx64_q.npy"))
    m._invert()
    rec = dict(q=np.asarray(m.q).copy(), ph=np.asarray(m.ph).copy(),
               u=np.asarray(m.u).copy())
    rec.update(consts(m))
    rec["params_json"] = np.array(json.dumps(
        {k: (np.asarray(v).tolist() if not isinstance(v, (int, float)) else v)
         for k, v in params.items()}))
    files["layered_fixture_nx64.npz"] = rec

    for name, rec in files.items():
        np.savez_compressed(os.path.join(HERE, name), **rec)
        print(name, os.path.getsize(os.path.join(HERE, name)))


if __name__ == "__main__":
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        main()
