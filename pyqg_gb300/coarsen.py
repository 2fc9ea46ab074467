"""Spectral coarse-graining and training data for the learned closure.

No counterpart in the reference (its ``Model.subgrid_forcing`` raises,
``pyqg/model.py:397-402``).  :class:`CoarseGrainer` maps a fine state to the
coarse grid with a sharp spectral cutoff and computes the subgrid PV forcing

    S = filtered(J(psi, q)) - J(filtered psi, filtered q),

J(psi, q) = u q_x + v q_y, on the GPU in FP64 (``pqg_coarse_forcing``).
:func:`generate_training_data` runs an FP64 ensemble of fine models, takes
snapshots and coarse-grains them into (q, S) pairs.
"""
import ctypes

import numpy as np

from . import _lib

# two-layer eddy physics of the closure experiments
PHYSICS = dict(L=1e6, beta=1.5e-11, rd=15000.0, delta=0.25, H1=500.0, U1=0.025, U2=0.0,
               rek=5.787e-7, filterfac=23.6)
QUIET = dict(tavestart=1e30, taveint=1e30, log_level=0)


class CoarseGrainer:
    """Coarse-grains states of `fine` (a model) onto the grid of `coarse`.

    Both models must share the domain and physics; the coarse grid must be
    even-sized and no finer than the fine one.
    """

    def __init__(self, fine, coarse):
        if fine.nz != coarse.nz:
            raise ValueError("models must have the same number of layers")
        self.fine, self.coarse = fine, coarse

    def __call__(self, qh=None, out=None):
        """(q_c, S) of the fine spectral PV `qh` (a CUDA complex128 tensor
        (nz, nl, nk); default: the fine model's current state)."""
        import torch
        f, c = self.fine, self.coarse
        if qh is None:
            qh = f.device_field("qh")
        qh = qh.to(f._device, torch.complex128).contiguous()
        if out is None:
            q_c = torch.empty((c.nz, c.ny, c.nx), dtype=torch.float64, device=f._device)
            S = torch.empty_like(q_c)
        else:
            q_c, S = out
        with torch.cuda.stream(f._stream):
            _lib.check(_lib.lib().pqg_coarse_forcing(f._plan, c._plan, qh.data_ptr(), q_c.data_ptr(),
                                                     S.data_ptr(), f._sp()))
        return q_c, S


def generate_training_data(nruns=64, nx_fine=256, nx_coarse=64, dt=3600.0, spinup_steps=86400,
                           snapshot_interval=1000, nsnapshots=780, seed0=2000, physics=None,
                           progress=None, return_ensemble=False):
    """(X, Y) CUDA float32 tensors (N, 2, nx_coarse, nx_coarse) of coarse PV
    and subgrid forcing from `nruns` FP64 fine runs (initial PV 1e-7 N(0, 1)
    seeded by seed0 + i), snapshots every `snapshot_interval` steps after
    `spinup_steps`.  Defaults: 64 runs, 10 years of spin-up (360-day years)
    and snapshots every 1000 h.  With `return_ensemble` the fine ensemble
    (at the last snapshot) is returned too."""
    import torch
    from .ensemble import Ensemble
    from .qg_model import QGModel
    phys = dict(PHYSICS if physics is None else physics)
    members = [("qg", dict(nx=nx_fine, dt=dt, **phys)) for _ in range(nruns)]
    ens = Ensemble(members, precision="fp64")
    ens.set_q([1e-7 * np.random.default_rng(seed0 + i).standard_normal((2, nx_fine, nx_fine))
               for i in range(nruns)])
    if spinup_steps:
        ens.step(spinup_steps)
    fine = QGModel(nx=nx_fine, dt=dt, **phys, **QUIET)
    coarse = QGModel(nx=nx_coarse, dt=dt, **phys, **QUIET)
    cg = CoarseGrainer(fine, coarse)
    n = nruns * nsnapshots
    X = torch.empty((n, 2, nx_coarse, nx_coarse), dtype=torch.float32, device=fine._device)
    Y = torch.empty_like(X)
    grp = ens.groups[0]
    order = [i for i, _ in grp.members]
    for s in range(nsnapshots):
        if s:
            ens.step(snapshot_interval)
        qs = grp.get_q()
        for j, i in enumerate(order):
            fine.q = qs[j]
            q_c, S = cg()
            X[s * nruns + i] = q_c
            Y[s * nruns + i] = S
        if progress:
            progress(s, nsnapshots)
    if return_ensemble:
        return X, Y, ens
    return X, Y


def channel_stats(X):
    """Per-channel mean and standard deviation of (N, C, ny, nx)."""
    x = X.double()
    mean = x.mean(dim=(0, 2, 3))
    std = x.std(dim=(0, 2, 3))
    return mean.cpu().numpy(), std.cpu().numpy()
