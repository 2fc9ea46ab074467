"""Batched ensembles of independent QG models (FP32 or FP64) on one GPU.

No counterpart in the reference, which runs one model per process.  An
:class:`Ensemble` groups its members by grid shape (nz, nx) and advances all
groups together: each group is one batched CUDA step (rows of all members,
then columns of all members), groups run on concurrent stream branches.

Members are described by the same keyword arguments as the model classes
(``QGModel`` or ``LayeredModel``); the constants come from those classes'
FP64 host code and are rounded once to the ensemble precision.  Within a group
all members must share the inversion matrix and filter (same grid, layer
depths, stratification and deformation radius); beta, bottom drag and the
background flow may differ per member.
"""
import ctypes

import numpy as np

from . import _lib
from .layered_model import layered_inversion_matrix, stretching_matrix
from .model import grid_constants, spectral_filter
from .qg_model import qg_inversion_matrix

YEAR = 360 * 86400.0


_device_matrices = {}


def device_inversion_matrix(S, kk, ll, two_layer_qg=False):
    """The FP64 inversion matrix a (nz, nz, nl, nk) = (S - kappa^2 I)^-1,
    built on the GPU (``pqg_inversion_matrix``), as a host array.  With
    ``two_layer_qg`` the two-layer QG closed form with F1 = S[0, 1],
    F2 = S[1, 0] (``pyqg/qg_model.py:146-161``), else the layered form
    (``pyqg/layered_model.py:211-229``).  Results are cached per input."""
    import torch
    S = np.ascontiguousarray(S, dtype=np.float64)
    kk = np.ascontiguousarray(kk, dtype=np.float64)
    ll = np.ascontiguousarray(ll, dtype=np.float64)
    key = (bool(two_layer_qg), S.tobytes(), kk.tobytes(), ll.tobytes())
    hit = _device_matrices.get(key)
    if hit is not None:
        return hit
    L = _lib.lib()
    nz, nl, nk = S.shape[0], ll.size, kk.size
    dev = torch.device("cuda", torch.cuda.current_device())
    stream = torch.cuda.current_stream(dev)
    with torch.cuda.stream(stream):
        kk_d = torch.from_numpy(kk).to(dev)
        ll_d = torch.from_numpy(ll).to(dev)
        a = torch.empty((nz, nz, nl, nk), dtype=torch.float64, device=dev)
        _lib.check(L.pqg_inversion_matrix(0 if two_layer_qg else 1, nz, nl, nk, S.ctypes.data,
                                          kk_d.data_ptr(), ll_d.data_ptr(), a.data_ptr(),
                                          ctypes.c_void_p(stream.cuda_stream)))
        out = a.cpu().numpy()
    if len(_device_matrices) > 64:
        _device_matrices.clear()
    _device_matrices[key] = out
    return out


def _member_constants(kind, kw, device_matrices=False):
    """FP64 constants of one member: (nz, nx, a, kk, ll, filtr, Ubg, Qy, rek).
    With ``device_matrices`` the inversion matrix is built in FP64 on the
    GPU (the precision form), else by the model classes' host code."""
    nx = kw.get("nx", 64)
    L = kw.get("L", 1e6)
    g = grid_constants(nx, nx, L, L)
    filtr = spectral_filter(g["k"], g["l"], g["dx"], g["dy"], kw.get("filterfac", 23.6))
    rek = kw.get("rek", 5.787e-7)
    beta = kw.get("beta", 1.5e-11)
    if kind == "qg":
        rd, delta = kw.get("rd", 15000.0), kw.get("delta", 0.25)
        U1, U2 = kw.get("U1", 0.025), kw.get("U2", 0.0)
        F1 = rd ** -2 / (1. + delta)
        F2 = delta * F1
        if device_matrices:
            a = device_inversion_matrix(np.array([[-F1, F1], [F2, -F2]]), g["kk"], g["ll"], True)
        else:
            a = qg_inversion_matrix(g["wv2"], F1, F2)
        Qy = np.array([beta + F1 * (U1 - U2), beta - F2 * (U1 - U2)])
        Ubg = np.array([U1, U2])
        nz = 2
    elif kind == "layered":
        nz = kw.get("nz", 3)
        H = np.array(kw.get("H", [500] + [1750] * (nz - 1)), dtype=float)
        U = np.array(kw.get("U", (np.arange(nz) * 0.025)[::-1]), dtype=float)
        rho = np.array(kw.get("rho", np.arange(nz) * 0.3 + 1025), dtype=float)
        f = kw.get("f", 0.0001236812857687059)
        gg = kw.get("g", 9.81)
        gpi = gg * (rho[1:] - rho[:-1]) / rho[:-1]
        S = stretching_matrix(nz, f ** 2, H, gpi, kw.get("rd"), kw.get("delta"))
        a = (device_inversion_matrix(S, g["kk"], g["ll"]) if device_matrices
             else layered_inversion_matrix(S, g["wv2"]))
        Qy = beta - S @ U
        Ubg = U
    else:
        raise ValueError("kind must be 'qg' or 'layered'")
    return nz, nx, np.ascontiguousarray(a), g["kk"], g["ll"], filtr, Ubg, Qy, float(rek)


def shard_members(n, rank, world):
    """Member indices of `rank` when n independent members are spread over
    `world` GPUs (contiguous blocks, sizes differing by at most one); the
    members need no exchange, so a multi-GPU ensemble is one Ensemble per
    rank over its shard."""
    if not 0 <= rank < world:
        raise ValueError("rank out of range")
    base, extra = divmod(n, world)
    lo = rank * base + min(rank, extra)
    return list(range(lo, lo + base + (1 if rank < extra else 0)))


class EnsembleGroup:
    """B members of one shape, advanced by the batched CUDA step."""

    def __init__(self, members, dt, precision):
        import torch
        if not torch.cuda.is_available():
            raise RuntimeError("pyqg_gb300 needs a CUDA device; none is visible")
        self._L = _lib.lib()
        self.members = members          # list of (index, constants tuple)
        c0 = members[0][1]
        self.nz, self.nx = c0[0], c0[1]
        self.B = len(members)
        self.dt = float(dt)
        self.precision = precision
        for _, c in members[1:]:
            if not (np.array_equal(c[2], c0[2]) and np.array_equal(c[5], c0[5])):
                raise ValueError("members of one group must share the inversion matrix and filter")
        h = ctypes.c_void_p()
        rc = self._L.pqg_ens_create(ctypes.byref(h), self.B, self.nz, self.nx, self.nx,
                                    4 if precision == "fp32" else 8)
        self._check(rc)
        self._h = h
        self._stream = torch.cuda.current_stream()
        a, kk, ll, filtr = c0[2], c0[3], c0[4], np.ascontiguousarray(c0[5])
        self._check(self._L.pqg_ens_set_constants(h, a.ctypes.data, kk.ctypes.data, ll.ctypes.data,
                                                  filtr.ctypes.data, self.dt))
        Ubg = np.ascontiguousarray(np.stack([c[6] for _, c in members]), dtype=np.float64)
        Qy = np.ascontiguousarray(np.stack([c[7] for _, c in members]), dtype=np.float64)
        rek = np.ascontiguousarray([c[8] for _, c in members], dtype=np.float64)
        self._check(self._L.pqg_ens_set_members(h, Ubg.ctypes.data, Qy.ctypes.data, rek.ctypes.data))

    def _check(self, rc):
        if rc != _lib.PQG_OK:
            msg = self._L.pqg_ens_last_error().decode(errors="replace")
            if rc == _lib.PQG_ERR_INVALID:
                raise ValueError(msg)
            if rc == _lib.PQG_ERR_UNSUPPORTED:
                raise NotImplementedError(msg)
            raise _lib.PQGError(rc, msg)

    def _sp(self):
        return ctypes.c_void_p(self._stream.cuda_stream)

    def set_q(self, q):
        q = np.ascontiguousarray(q, dtype=np.float64)
        if q.shape != (self.B, self.nz, self.nx, self.nx):
            raise ValueError("q must have shape %s" % ((self.B, self.nz, self.nx, self.nx),))
        self._check(self._L.pqg_ens_set_q(self._h, q.ctypes.data, self._sp()))

    def get_q(self):
        out = np.empty((self.B, self.nz, self.nx, self.nx))
        self._check(self._L.pqg_ens_get_q(self._h, out.ctypes.data, self._sp()))
        return out

    def energy(self):
        ke = np.empty((self.B, self.nz))
        en = np.empty((self.B, self.nz))
        self._check(self._L.pqg_ens_energy(self._h, ke.ctypes.data, en.ctypes.data, self._sp()))
        return ke, en

    def autotune(self):
        """Pick the fastest row / column launch configuration on this
        group's state (the state is restored); returns the choice."""
        out = np.zeros(10)
        self._check(self._L.pqg_ens_autotune(self._h, out.ctypes.data, self._sp()))
        return dict(rows_per_cta=int(out[0]), row_threads=int(out[1]), row_ms=float(out[2]),
                    cols_per_cta=int(out[3]), col_threads=int(out[4]), col_ms=float(out[5]),
                    member_kernel=bool(out[6]), member_threads=int(out[7]),
                    member_ms_4_steps=float(out[8]), two_kernel_ms_4_steps=float(out[9]))

    def set_closure(self, net):
        """Attach a :class:`~pyqg_gb300.closure.ConvNet` (or None): every step
        adds its PV forcing, as a q_parameterization would."""
        self._net = net
        self._check(self._L.pqg_ens_set_closure(self._h, None if net is None else net._h))

    def state(self):
        q, qh = ctypes.c_void_p(), ctypes.c_void_p()
        tc, t = ctypes.c_longlong(), ctypes.c_double()
        self._check(self._L.pqg_ens_state(self._h, ctypes.byref(q), ctypes.byref(qh),
                                          ctypes.byref(tc), ctypes.byref(t)))
        return q.value, qh.value, tc.value, t.value

    def __del__(self):
        h = self.__dict__.get("_h")
        if h is not None and h.value:
            try:
                import torch
                torch.cuda.synchronize()
                self._L.pqg_ens_destroy(h)
            except Exception:
                pass
            self._h = None


class Ensemble:
    """An ensemble of independent members of possibly different sizes.

    ``members`` is a list of ``(kind, kwargs)`` with kind ``"qg"`` or
    ``"layered"`` and the keyword arguments of ``QGModel`` / ``LayeredModel``
    (including ``nx`` and ``dt``).  ``precision`` is ``"fp32"`` (default) or
    ``"fp64"``.
    """

    def __init__(self, members, precision="fp32"):
        if precision not in ("fp32", "fp64"):
            raise ValueError("precision must be 'fp32' or 'fp64'")
        self.precision = precision
        # the FP32 form builds its inversion matrices in FP64 on the GPU and
        # rounds them once; FP64 members keep the host build, so that they
        # reproduce the single-model step bit for bit
        consts = [_member_constants(kind, kw, device_matrices=precision == "fp32") for kind, kw in members]
        dts = [float(kw.get("dt", 7200.0)) for _, kw in members]
        keys = {}
        for i, c in enumerate(consts):
            keys.setdefault((c[0], c[1], dts[i]), []).append((i, c))
        self.groups = []
        self._index = {}
        for (nz, nx, dt), mem in sorted(keys.items()):
            # split further if the shared constants differ inside a shape
            subgroups = []
            for i, c in mem:
                for sg in subgroups:
                    c0 = sg[0][1]
                    if np.array_equal(c[2], c0[2]) and np.array_equal(c[5], c0[5]):
                        sg.append((i, c))
                        break
                else:
                    subgroups.append([(i, c)])
            for sg in subgroups:
                grp = EnsembleGroup(sg, dt, precision)
                for j, (i, _) in enumerate(sg):
                    self._index[i] = (len(self.groups), j)
                self.groups.append(grp)
        self.n = len(members)
        self.tc = 0

    def set_q(self, qs):
        """Initial PV per member (list of (nz, nx, nx) arrays)."""
        for gi, grp in enumerate(self.groups):
            grp.set_q(np.stack([qs[i] for i, _ in grp.members]))

    def q(self, i):
        gi, j = self._index[i]
        return self.groups[gi].get_q()[j]

    def step(self, nsteps):
        """Advance every member by `nsteps` steps (each on its own dt)."""
        arr = (ctypes.c_void_p * len(self.groups))(*[g._h.value for g in self.groups])
        L = self.groups[0]._L
        rc = L.pqg_ens_step_many(arr, len(self.groups), int(nsteps), self.groups[0]._sp())
        self.groups[0]._check(rc)
        self.tc += nsteps

    def set_closure(self, net):
        """Attach a learned closure to every group whose members match the
        network's channels and image size; returns the number of groups."""
        n = 0
        for grp in self.groups:
            if net is None or (grp.nz == net.channels[0] == net.channels[-1] and grp.nx == net.nx):
                grp.set_closure(net)
                n += 1
        return n

    def autotune(self):
        """Autotune every group's launch configuration; returns the choices."""
        return [g.autotune() for g in self.groups]

    def energy(self):
        """FP64 (ke, enstrophy) per member and layer, in member order."""
        ke = [None] * self.n
        en = [None] * self.n
        for grp in self.groups:
            k, e = grp.energy()
            for j, (i, _) in enumerate(grp.members):
                ke[i], en[i] = k[j], e[j]
        return ke, en
