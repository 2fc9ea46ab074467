"""Generate the golden fixtures in this folder from the reference pyqg.

Run in a container that has the reference tree (it imports the reference
package in place and its Cython kernel compiled by ``oracle/build_ref.py``):

    PYQG_REFERENCE_ROOT=<reference checkout> python tests/golden/make_golden.py [prefix ...]

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


def main(only=None):
    """Write every fixture, or those whose file names start with one of
    ``only`` (e.g. ``params diag``)."""
    pyqg = import_reference_pyqg()
    rng = np.random.default_rng
    files = {}

    # Standard two-layer physics at nx=64, dt=7200 (seed 0), 100 steps.
    two_layer = dict(nx=64, L=1e6, beta=1.5e-11, rd=15000.0, delta=0.25, H1=500,
              U1=0.025, U2=0.0, rek=5.787e-7, dt=7200.0, filterfac=23.6)
    m = pyqg.QGModel(**two_layer, **QUIET)
    q0 = 1e-7 * rng(0).standard_normal((2, 64, 64))
    files["qg_two_layer_nx64.npz"] = run_case(m, q0, [1, 10, 100])

    # Standard two-layer physics at nx=256, dt=3600 (seed 0): checksums only (size).
    two_layer_nx256 = dict(two_layer, nx=256, dt=3600.0)
    m = pyqg.QGModel(**two_layer_nx256, **QUIET)
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
    files["qg_two_layer_nx256_checksums.npz"] = rec

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
    cp = dict(two_layer, nx=32)
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

    files.update(physical_parameterizations(pyqg))
    files.update(diagnostics(pyqg))
    files.update(dataset(pyqg))
    save(files, only)


def save(files, only=None):
    for name, rec in files.items():
        if only and not any(name.startswith(o) for o in only):
            continue
        np.savez_compressed(os.path.join(HERE, name), **rec)
        print(name, os.path.getsize(os.path.join(HERE, name)))


def physical_parameterizations(pyqg):
    """The reference's Smagorinsky, BackscatterBiharmonic, ZannaBolton2020
    and RingForcing (pyqg/parameterizations.py:132-366) evaluated on a
    seeded state of standard two-layer physics at nx=32 after 10 steps, with u, v and ph refreshed from
    that state by one inversion."""
    two_layer = dict(nx=64, L=1e6, beta=1.5e-11, rd=15000.0, delta=0.25, H1=500,
              U1=0.025, U2=0.0, rek=5.787e-7, dt=7200.0, filterfac=23.6)
    m = pyqg.QGModel(**dict(two_layer, nx=32), **QUIET)
    m.q = 1e-6 * np.random.default_rng(3).standard_normal((2, 32, 32))
    for _ in range(10):
        m._step_forward()
    m._invert()
    rec = dict(q=np.asarray(m.q).copy(), ph=np.asarray(m.ph).copy(),
               u=np.asarray(m.u).copy(), v=np.asarray(m.v).copy(),
               dx=np.float64(m.dx), Hi=np.asarray(m.Hi).copy())
    rec.update(consts(m))
    rec["smag_du"], rec["smag_dv"] = pyqg.Smagorinsky()(m)
    rec["smag_nu"] = pyqg.Smagorinsky()(m, just_viscosity=True)
    rec["smag02_du"], rec["smag02_dv"] = pyqg.Smagorinsky(constant=0.2)(m)
    rec["back_dq"] = pyqg.BackscatterBiharmonic()(m)
    rec["back05_dq"] = pyqg.BackscatterBiharmonic(smag_constant=0.1, back_constant=0.5)(m)
    rec["zb_du"], rec["zb_dv"] = pyqg.ZannaBolton2020()(m)
    ring = dict(k_in_forc=2e-5, k_out_forc=6e-5, mag_noise_forc=3.0)
    for i, layers in enumerate(("all", "surf", "bottom")):
        np.random.seed(100 + i)
        rec["ring_%s_dq" % layers] = pyqg.RingForcing(layers=layers, **ring)(m)
    rec["ring_seeds"] = np.array([100, 101, 102])
    return {"params_physical_nx32.npz": rec}


def _numpy1_modal_projection(self, p, forward=True):
    """pyqg/model.py:307-317 with numpy 1's reading of its ``solve`` call.

    The reference solves ``pmodes x = p[:, l, k]`` for every wavenumber by
    passing ``p.T`` of shape (nk, nl, nz) as a stack of vectors; numpy 2
    reads a right-hand side of more than one dimension as matrices, and the
    call fails.  The same solves are written here with an explicit vector
    axis; nothing else of the reference is changed."""
    if forward:
        return np.linalg.solve(self.pmodes[np.newaxis, np.newaxis], p.T[..., np.newaxis])[..., 0].T
    return np.einsum("ik,k...->i...", self.pmodes, p)


def diagnostics(pyqg):
    """Every registered diagnostic of short runs that accumulate each step
    (tavestart = 0, taveint = dt; pyqg/model.py:802-814), as time averages
    (get_diagnostic) with their sample counts.  The layered model's modal
    diagnostics need the numpy-1 reading of ``modal_projection``."""
    pyqg.Model.modal_projection = _numpy1_modal_projection
    two_layer = dict(nx=64, L=1e6, beta=1.5e-11, rd=15000.0, delta=0.25, H1=500,
              U1=0.025, U2=0.0, rek=5.787e-7, dt=7200.0, filterfac=23.6)
    lay = dict(nz=3, nx=32, H=[500., 1000., 2500.], U=[0.05, 0.02, 0.0],
               V=[0., 0., 0.], rek=5.787e-7, dt=7200.0)
    cases = {
        "diag_qg_nx64.npz": (pyqg.QGModel, two_layer, {}, 11, 6),
        "diag_layered_nz3_nx32.npz": (pyqg.LayeredModel, lay, {}, 12, 6),
        "diag_qg_smag_nx32.npz": (pyqg.QGModel, dict(two_layer, nx=32),
                                  dict(uv_parameterization=pyqg.Smagorinsky()), 13, 5),
        "diag_qg_back_nx32.npz": (pyqg.QGModel, dict(two_layer, nx=32),
                                  dict(q_parameterization=pyqg.BackscatterBiharmonic()), 14, 5),
    }
    out = {}
    for name, (cls, kw, hooks, seed, nsteps) in cases.items():
        m = cls(**kw, **hooks, tavestart=0.0, taveint=kw["dt"], log_level=0)
        m.q = 1e-6 * np.random.default_rng(seed).standard_normal((m.nz, m.ny, m.nx))
        q0 = np.asarray(m.q).copy()
        for _ in range(nsteps):
            m._step_forward()
        rec = dict(q0=q0, nsteps=np.int64(nsteps), q=np.asarray(m.q).copy())
        names = []
        for n, d in m.diagnostics.items():
            if not d["active"]:
                continue
            rec["diag_" + n] = np.asarray(m.get_diagnostic(n))
            rec["count_" + n] = np.int64(d["count"])
            names.append(n)
        rec["names"] = np.array(names)
        out[name] = rec
    return out


def _jsonable(v):
    if v is None:
        return None
    a = np.asarray(v)
    if np.iscomplexobj(a):
        return {"re": a.real.tolist(), "im": a.imag.tolist()}
    return a.tolist()


def dataset(pyqg):
    """``Model.to_dataset`` (pyqg/xarray_output.py:118-174) of a short seeded
    run with every diagnostic filled: the reference module runs unchanged
    against a stand-in ``xarray`` whose ``Dataset`` records its arguments
    (xarray is not installed here).  Stored: each data variable's and
    coordinate's dims, attrs and values, and the global attrs."""
    import types

    class _Dataset:
        def __init__(self, data_vars, coords=None, attrs=None):
            self.data_vars, self.coords, self.attrs = data_vars, coords, dict(attrs or {})

    stub = types.ModuleType("xarray")
    stub.Dataset = _Dataset
    saved = sys.modules.get("xarray")
    sys.modules["xarray"] = stub
    sys.modules.pop("pyqg.xarray_output", None)
    try:
        import pyqg.xarray_output as xo
        two_layer = dict(nx=32, L=1e6, beta=1.5e-11, rd=15000.0, delta=0.25, H1=500,
                  U1=0.025, U2=0.0, rek=5.787e-7, dt=7200.0, filterfac=23.6)
        m = pyqg.QGModel(**two_layer, tavestart=0.0, taveint=7200.0, log_level=0)
        m.q = 1e-6 * np.random.default_rng(15).standard_normal((2, 32, 32))
        q0 = np.asarray(m.q).copy()
        for _ in range(4):
            m._step_forward()
        ds = xo.model_to_dataset(m)
    finally:
        sys.modules.pop("pyqg.xarray_output", None)
        if saved is None:
            sys.modules.pop("xarray", None)
        else:
            sys.modules["xarray"] = saved
    rec = dict(q0=q0, nsteps=np.int64(4))
    meta = {"vars": {}, "coords": {}}
    for n, (dims, data, attrs) in ds.data_vars.items():
        meta["vars"][n] = {"dims": [dims] if isinstance(dims, str) else list(dims), "attrs": attrs}
        rec["var_" + n] = np.asarray(data)
    for n, (dims, data, attrs) in ds.coords.items():
        meta["coords"][n] = {"dims": [dims] if isinstance(dims, str) else list(dims), "attrs": attrs}
        rec["coord_" + n] = np.asarray(data)
    meta["attrs"] = {k: _jsonable(v) for k, v in ds.attrs.items()}
    rec["meta_json"] = np.array(json.dumps(meta))
    return {"dataset_qg_nx32.npz": rec}


if __name__ == "__main__":
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        main(sys.argv[1:] or None)
