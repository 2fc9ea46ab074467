"""The FP32 form against the FP64 step (two-layer QG, nx=256,
dt=3600 s).

No counterpart in the reference.  From FP64 states spun up from seeded
1e-7 N(0, 1) PV, an FP64 and an FP32 ensemble (the FP32 form: transforms,
products and AB3 in FP32, matrices built in FP64) advance side by side.
Reported: the pointwise relative L2 error on q after 10 steps, and after the
statistics window the time-mean isotropic KE spectrum and the layer-wise
eddy PV flux mean(v q) of the FP32 runs relative to the FP64 runs.

``python -m pyqg_gb300.precision_experiment --help`` lists the sizes; the
result is one JSON document.
"""
import argparse
import json
import time

import numpy as np

from .closure_experiment import YEAR, ke_spectrum
from .coarsen import PHYSICS, QUIET


def eddy_pv_flux(model, q):
    """Layer-wise mean of v q (host FP64) for PV q (nz, ny, nx)."""
    qh = np.fft.rfftn(q, axes=(-2, -1))
    ph = np.einsum("ijlk,jlk->ilk", np.asarray(model.a), qh)
    v = np.fft.irfftn(1j * np.asarray(model.k) * ph, s=q.shape[-2:], axes=(-2, -1))
    return (v * q).mean(axis=(-1, -2))


def run(members=8, spinup_years=5.0, years=2.0, sample_every=240, seed0=2000, log=print):
    import torch
    import pyqg_gb300 as P
    dt, nx = 3600.0, 256
    t0 = time.time()
    spec = [("qg", dict(nx=nx, dt=dt, **PHYSICS)) for _ in range(members)]
    e64 = P.Ensemble(spec, precision="fp64")
    e64.set_q([1e-7 * np.random.default_rng(seed0 + i).standard_normal((2, nx, nx)) for i in range(members)])
    e64.step(int(round(spinup_years * YEAR / dt)))
    q0 = e64.groups[0].get_q()
    e32 = P.Ensemble(spec, precision="fp32")
    e32.set_q([q0[j] for j in range(members)])
    ref = P.Ensemble(spec, precision="fp64")
    ref.set_q([q0[j] for j in range(members)])
    # 10 steps from the same state
    ref.step(10)
    e32.step(10)
    a, b = ref.groups[0].get_q(), e32.groups[0].get_q()
    err10 = float(np.linalg.norm((b - a).ravel()) / np.linalg.norm(a.ravel()))
    log("10-step relative L2 on q: %.3e" % err10)
    # statistics window (both advance from the 10-step states)
    m = P.QGModel(nx=nx, dt=dt, **PHYSICS, **QUIET)
    n = int(round(years * YEAR / dt))
    ke = {"fp64": 0.0, "fp32": 0.0}
    flux = {"fp64": 0.0, "fp32": 0.0}
    cnt = 0
    done = 0
    while done < n:
        c = min(sample_every, n - done)
        ref.step(c)
        e32.step(c)
        done += c
        for name, ens in (("fp64", ref), ("fp32", e32)):
            qs = ens.groups[0].get_q()
            for j in range(members):
                ke[name] = ke[name] + ke_spectrum(m, qs[j])[1] / members
                flux[name] = flux[name] + eddy_pv_flux(m, qs[j]) / members
        cnt += 1
    torch.cuda.synchronize()
    s64, s32 = ke["fp64"] / cnt, ke["fp32"] / cnt
    energetic = s64 >= 0.1 * s64.max()
    rel = np.abs(s32 - s64) / np.maximum(s64, 1e-300)
    f64, f32 = flux["fp64"] / cnt, flux["fp32"] / cnt
    rep = {
        "config": dict(members=members, nx=nx, dt=dt, spinup_years=spinup_years, years=years,
                       samples=cnt, seed0=seed0,
                       model_steps=int(round(spinup_years * YEAR / dt)) + 10 + n),
        "ten_step_rel_l2_q": err10,
        "ke_spectrum": dict(max_rel_diff_energy_containing=float(rel[energetic].max()),
                            mean_rel_diff_energy_containing=float(rel[energetic].mean()),
                            total_ke_ratio=float(s32.sum() / s64.sum()),
                            bins_energy_containing=int(energetic.sum())),
        "eddy_pv_flux": dict(fp64=[float(x) for x in f64], fp32=[float(x) for x in f32],
                             rel_diff=[float(abs(x - y) / abs(y)) for x, y in zip(f32, f64)]),
        "seconds": time.time() - t0,
    }
    return rep


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--members", type=int, default=8)
    ap.add_argument("--spinup-years", type=float, default=5.0)
    ap.add_argument("--years", type=float, default=2.0)
    ap.add_argument("--out", default=None)
    a = ap.parse_args(argv)
    rep = run(members=a.members, spinup_years=a.spinup_years, years=a.years)
    txt = json.dumps(rep)
    print(txt)
    if a.out:
        with open(a.out, "w") as f:
            f.write(txt + "\n")


if __name__ == "__main__":
    main()
