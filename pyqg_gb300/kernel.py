"""GPU-backed drop-in for pyqg's ``PseudoSpectralKernel``.

Mirrors the constructor, properties and methods of the reference Cython class
(``pyqg/kernel.pyx:32-637``).  Every field lives in device memory (torch
CUDA tensors used only as allocations); the arithmetic runs in the CUDA
library ``libpyqg_gb300.so`` through its C ABI.  There is no CPU path: a
kernel cannot be constructed without a CUDA device and the built library.

Aliasing views.  The reference hands out numpy views of its buffers and code
writes through them (``m.u[0] = ...``, ``m.dqhdt[:] = ...``).  Here a getter
downloads the field into a persistent pinned host array (the same array
object every time) and returns it; before the next device operation every
array handed out since the last operation is uploaded back, so writes
through the returned array reach the device.  Arrays held across a device
operation are refreshed by the next getter call, not automatically.

History buffers.  ``dqhdt``, ``dqhdt_p`` and ``dqhdt_pp`` are three logical
roles over three device buffers.  The reference shifts the history by
copying (``pyqg/kernel.pyx:509-510``); here roles are re-pointed instead and
a role that shares its buffer with another is given a free buffer before it
is written (copy-on-write).
"""
import ctypes
import os

import numpy as np
import torch

from . import _lib

_PHYS = ("q", "u", "v", "uq", "vq", "dq", "du", "dv")
_SPEC = ("qh", "ph", "uh", "vh", "uqh", "vqh", "dqh", "duh", "dvh")
_TEND = ("dqhdt", "dqhdt_p", "dqhdt_pp")
_AUX = ("ph", "uh", "vh", "u", "v", "uq", "vq", "uqh", "vqh")

# Transform engine of the fused step for new kernels: "fixed" (64-bit block
# fixed point, used where the grid allows it) or "fp64".  PQG_ENGINE
# overrides it.
DEFAULT_ENGINE = os.environ.get("PQG_ENGINE", "fixed")


def _check_array(x, dtype, ndim, name):
    """Typed-buffer checks of the reference setters (np.ndarray[T, ndim=N])."""
    if not isinstance(x, np.ndarray):
        raise TypeError("%s must be a numpy.ndarray, got %s" % (name, type(x).__name__))
    if x.dtype != dtype:
        raise ValueError("Buffer dtype mismatch for %s: expected %s but got %s"
                         % (name, np.dtype(dtype), x.dtype))
    if x.ndim != ndim:
        raise ValueError("Buffer has wrong number of dimensions for %s "
                         "(expected %d, got %d)" % (name, ndim, x.ndim))
    return x


class PseudoSpectralKernel:
    """Drop-in replacement of ``pyqg.kernel.PseudoSpectralKernel``."""

    def __new__(cls, *args, **kwargs):
        self = super().__new__(cls)
        # properties may be set before __init__ (pyqg/layered_model.py:121)
        self.__dict__["_pre"] = {}
        self.__dict__["_plan"] = None
        return self

    def __init__(self, nz, ny, nx, fftw_num_threads=1, has_q_param=0,
                 has_uv_param=0):
        if not torch.cuda.is_available():
            raise RuntimeError("pyqg_gb300 needs a CUDA device; none is visible")
        L = _lib.lib()
        self.nz, self.ny, self.nx = int(nz), int(ny), int(nx)
        self.nl = self.ny
        self.nk = int(self.nx / 2 + 1)
        self.num_threads = fftw_num_threads
        self._L = L
        self._device = torch.device("cuda", torch.cuda.current_device())
        self._stream = torch.cuda.current_stream(self._device)
        plan = ctypes.c_void_p()
        _lib.check(L.pqg_plan_create(ctypes.byref(plan), self.nz, self.ny, self.nx))
        self._plan = plan
        self._engine = "fp64"
        if DEFAULT_ENGINE == "fixed" and L.pqg_set_engine(plan, 1) == _lib.PQG_OK:
            self._engine = "fixed"
        dev = self._device
        shp_r = (self.nz, self.ny, self.nx)
        shp_c = (self.nz, self.nl, self.nk)
        self._d = {}
        names_r = ["q", "u", "v", "uq", "vq"]
        names_c = ["qh", "ph", "uh", "vh", "uqh", "vqh"]
        self._has_uv = bool(has_uv_param)
        self._has_q = bool(has_q_param)
        if self._has_uv:
            names_r += ["du", "dv"]
            names_c += ["duh", "dvh"]
        if self._has_q:
            names_r += ["dq"]
            names_c += ["dqh"]
        for n in names_r:
            self._d[n] = torch.zeros(shp_r, dtype=torch.float64, device=dev)
        for n in names_c:
            self._d[n] = torch.zeros(shp_c, dtype=torch.complex128, device=dev)
        self._tend = [torch.zeros(shp_c, dtype=torch.complex128, device=dev)
                      for _ in range(3)]
        self._role = {"dqhdt": 0, "dqhdt_p": 1, "dqhdt_pp": 2}
        self._shadow = {}       # name -> (pinned tensor, numpy view)
        self._current = set()   # names whose host array holds the latest value
        # time (pyqg/kernel.pyx:190-194)
        self._dt = 0.0
        self._t = 0.0
        self._tc = 0
        self._ablevel = 0
        self._rek = 0.0
        # constants (pyqg/kernel.pyx:127-132)
        self._a = np.zeros((self.nz, self.nz, self.nl, self.nk), np.complex128)
        self._kk = np.zeros(self.nk)
        self._ll = np.zeros(self.nl)
        self._ik = np.zeros(self.nk, np.complex128)
        self._il = np.zeros(self.nl, np.complex128)
        self.__dict__["_k2l2_arr"] = np.zeros((self.nl, self.nk))
        self._Ubg = None
        self._Qy = None
        self._ikQy = None
        self._filtr = None
        zero_u = np.zeros(self.nz)
        _lib.check(L.pqg_set_ubg(plan, zero_u.ctypes.data))
        _lib.check(L.pqg_set_qy(plan, zero_u.ctypes.data))
        # apply properties set before __init__
        pre = self.__dict__.pop("_pre")
        for name, val in pre.items():
            setattr(self, name, val)

    def __del__(self):
        plan = self.__dict__.get("_plan")
        if plan is not None and plan.value:
            try:
                torch.cuda.synchronize(self._device)
                self._L.pqg_plan_destroy(plan)
            except Exception:
                pass
            self.__dict__["_plan"] = None

    @property
    def engine(self):
        """Transform engine of the fused step: 'fixed' (64-bit block fixed
        point, the default on power-of-two grids) or 'fp64'."""
        return self._engine

    @engine.setter
    def engine(self, name):
        if name not in ("fixed", "fp64"):
            raise ValueError("engine must be 'fixed' or 'fp64'")
        _lib.check(self._L.pqg_set_engine(self._plan, 1 if name == "fixed" else 0))
        self._engine = name

    # ------------------------------------------------------------------
    # buffer plumbing
    # ------------------------------------------------------------------
    def _ready(self):
        return self.__dict__.get("_plan") is not None

    def _sp(self):
        return ctypes.c_void_p(self._stream.cuda_stream)

    def _buf(self, name):
        if name in _TEND:
            return self._tend[self._role[name]]
        try:
            return self._d[name]
        except KeyError:
            raise AttributeError("%s is not allocated (no matching "
                                 "parameterization)" % name) from None

    def _ptr(self, name):
        return self._buf(name).data_ptr()

    def _host(self, name):
        sh = self._shadow.get(name)
        if sh is None:
            t = torch.empty(self._buf(name).shape, dtype=self._buf(name).dtype,
                            pin_memory=True)
            sh = (t, t.numpy())
            self._shadow[name] = sh
        return sh

    def _get(self, name):
        """Download (once per device update) and return the host array."""
        buf = self._buf(name)
        t, arr = self._host(name)
        if name not in self._current:
            with torch.cuda.stream(self._stream):
                t.copy_(buf, non_blocking=True)
            self._stream.synchronize()
            self._current.add(name)
        return arr

    def _sync_in(self):
        """Upload every host array handed out since the last device update."""
        if not self._current:
            return
        for name in list(self._current):
            if name in _TEND:
                self._own(name, copy=False)
            t, _ = self._shadow[name]
            with torch.cuda.stream(self._stream):
                self._buf(name).copy_(t)
        self._current.clear()

    def _shared(self, role):
        i = self._role[role]
        return sum(1 for v in self._role.values() if v == i) > 1

    def _own(self, role, copy):
        """Give `role` a buffer of its own (copy-on-write when `copy`)."""
        if not self._shared(role):
            return
        used = set(self._role.values())
        j = next(i for i in range(3) if i not in used)
        if copy:
            with torch.cuda.stream(self._stream):
                self._tend[j].copy_(self._tend[self._role[role]])
        self._role[role] = j

    def _invalidate(self, *names):
        for n in names:
            self._current.discard(n)

    def _upload(self, name, arr):
        t, host = self._host(name)
        host[...] = arr
        with torch.cuda.stream(self._stream):
            self._buf(name).copy_(t)
        self._current.discard(name)

    # ------------------------------------------------------------------
    # transforms (pyqg/kernel.pyx:245-267,291-309)
    # ------------------------------------------------------------------
    def _device_rfft2(self, x):
        """Device real field (n, ny, nx) float64 -> new (n, nl, nk) complex."""
        x = x.contiguous()
        out = torch.empty((x.shape[0], self.nl, self.nk), dtype=torch.complex128,
                          device=self._device)
        _lib.check(self._L.pqg_rfft2(self._plan, x.data_ptr(), out.data_ptr(),
                                     x.shape[0], self._sp()))
        return out

    def _device_advect(self, f, u, v):
        """ik fft(u f) + il fft(v f) of device real fields (n, ny, nx)."""
        f, u, v = (t.to(self._device, torch.float64).contiguous() for t in (f, u, v))
        out = torch.empty((f.shape[0], self.nl, self.nk), dtype=torch.complex128,
                          device=self._device)
        _lib.check(self._L.pqg_advect(self._plan, f.data_ptr(), u.data_ptr(), v.data_ptr(),
                                      f.shape[0], out.data_ptr(), self._sp()))
        return out

    def _device_irfft2(self, xh):
        xh = xh.contiguous()
        out = torch.empty((xh.shape[0], self.ny, self.nx), dtype=torch.float64,
                          device=self._device)
        _lib.check(self._L.pqg_irfft2(self._plan, xh.data_ptr(), out.data_ptr(),
                                      xh.shape[0], self._sp()))
        return out

    def fft(self, v):
        """Forward transform of a real (n, ny, nx) field; returns a new array.
        numpy input -> numpy output, CUDA tensor input -> CUDA tensor output."""
        if isinstance(v, torch.Tensor):
            return self._device_rfft2(v.to(self._device, torch.float64).reshape(-1, self.ny, self.nx))
        v = np.asarray(v)
        if v.dtype != np.float64:
            raise ValueError("Buffer dtype mismatch, expected 'double' but got %s" % v.dtype)
        if v.ndim != 3:
            raise ValueError("Buffer has wrong number of dimensions (expected 3, got %d)" % v.ndim)
        v = self._planes(v)
        with torch.cuda.stream(self._stream):
            d = torch.from_numpy(np.ascontiguousarray(v)).to(self._device)
            out = self._device_rfft2(d).cpu()
        return out.numpy()

    def _planes(self, v):
        """A single plane is broadcast over the nz layers, as the reference
        does when copying it into its (nz, ...) transform buffer."""
        if v.shape[0] == 1 and self.nz > 1:
            v = np.broadcast_to(v, (self.nz,) + v.shape[1:])
        return v

    def ifft(self, v):
        """Inverse transform of a complex (n, nl, nk) field; returns a new array."""
        if isinstance(v, torch.Tensor):
            return self._device_irfft2(v.to(self._device, torch.complex128).reshape(-1, self.nl, self.nk))
        v = np.asarray(v)
        if v.dtype != np.complex128:
            raise ValueError("Buffer dtype mismatch, expected 'double complex' but got %s" % v.dtype)
        if v.ndim != 3:
            raise ValueError("Buffer has wrong number of dimensions (expected 3, got %d)" % v.ndim)
        v = self._planes(v)
        with torch.cuda.stream(self._stream):
            d = torch.from_numpy(np.ascontiguousarray(v)).to(self._device)
            out = self._device_irfft2(d).cpu()
        return out.numpy()

    # ------------------------------------------------------------------
    # stages (pyqg/kernel.pyx:312-526)
    # ------------------------------------------------------------------
    def _invert(self):
        self._sync_in()
        _lib.check(self._L.pqg_invert(
            self._plan, self._ptr("qh"), self._ptr("ph"), self._ptr("uh"),
            self._ptr("vh"), self._ptr("u"), self._ptr("v"), self._sp()))

    def _do_advection(self):
        self._sync_in()
        self._own("dqhdt", copy=False)
        _lib.check(self._L.pqg_do_advection(
            self._plan, self._ptr("q"), self._ptr("u"), self._ptr("v"),
            self._ptr("ph"), self._ptr("uq"), self._ptr("vq"), self._ptr("uqh"),
            self._ptr("vqh"), self._ptr("dqhdt"), self._sp()))

    def _do_friction(self):
        self._sync_in()
        if self._rek:
            self._own("dqhdt", copy=True)
            _lib.check(self._L.pqg_do_friction(self._plan, self._ptr("ph"),
                                               self._ptr("dqhdt"), self._sp()))

    def _to_device_field(self, name, x):
        """Copy a parameterization output into device buffer `name`."""
        dst = self._buf(name)
        with torch.cuda.stream(self._stream):
            if isinstance(x, torch.Tensor):
                dst.copy_(x.reshape(dst.shape))
            else:
                x = np.asarray(x, dtype=np.float64)
                if x.shape != tuple(dst.shape):
                    x = np.broadcast_to(x, dst.shape)
                dst.copy_(torch.from_numpy(np.ascontiguousarray(x)))

    def _call_hook(self, hook):
        """Run a parameterization with device outputs allowed."""
        self._hook_on_device = True
        try:
            return hook(self)
        finally:
            self._hook_on_device = False

    def _do_q_subgrid_parameterization(self):
        dq = self._call_hook(self.q_parameterization)
        self._sync_in()
        self._to_device_field("dq", dq)
        self._own("dqhdt", copy=True)
        _lib.check(self._L.pqg_do_q_forcing(self._plan, self._ptr("dq"),
                                            self._ptr("dqh"), self._ptr("dqhdt"),
                                            self._sp()))

    def _do_uv_subgrid_parameterization(self):
        res = self._call_hook(self.uv_parameterization)
        du, dv = res[0], res[1]
        self._sync_in()
        self._to_device_field("du", du)
        self._to_device_field("dv", dv)
        self._own("dqhdt", copy=True)
        _lib.check(self._L.pqg_do_uv_forcing(
            self._plan, self._ptr("du"), self._ptr("dv"), self._ptr("duh"),
            self._ptr("dvh"), self._ptr("dqhdt"), self._sp()))

    def _forward_timestep(self):
        """Filtered FE/AB2/AB3 update and q = irfft2(qh)
        (pyqg/kernel.pyx:467-526)."""
        self._sync_in()
        _lib.check(self._L.pqg_forward_timestep(
            self._plan, self._ablevel, self._dt, self._ptr("qh"),
            self._ptr("dqhdt"), self._ptr("dqhdt_p"), self._ptr("dqhdt_pp"),
            self._ptr("q"), 0, self._sp()))
        # history shift by roles: pp <- p, p <- dqhdt (dqhdt keeps its value)
        self._role["dqhdt_pp"] = self._role["dqhdt_p"]
        self._role["dqhdt_p"] = self._role["dqhdt"]
        self._ablevel = min(self._ablevel + 1, 2)
        self._tc += 1
        self._t += self._dt

    def _step_fused(self, nsteps):
        """Advance `nsteps` whole steps (no parameterization hooks) with the
        fused two-kernel step replayed from CUDA graphs; leaves every field
        as the stage-by-stage path would."""
        if nsteps <= 0:
            return
        self._sync_in()
        if self._role["dqhdt_p"] == self._role["dqhdt_pp"]:
            self._own("dqhdt_pp", copy=True)
        st = _lib.State(self._ptr("q"), self._ptr("qh"), self._ptr("dqhdt"),
                        self._ptr("dqhdt_p"), self._ptr("dqhdt_pp"),
                        self._ablevel, self._tc, self._t, self._dt)
        aux = _lib.Aux(*[self._ptr(n) for n in _AUX])
        _lib.check(self._L.pqg_step(self._plan, ctypes.byref(st), int(nsteps),
                                    ctypes.byref(aux), self._sp()))
        idx = {b.data_ptr(): i for i, b in enumerate(self._tend)}
        self._role = {"dqhdt": idx[st.dqhdt], "dqhdt_p": idx[st.dqhdt_p],
                      "dqhdt_pp": idx[st.dqhdt_pp]}
        self._ablevel = st.ablevel
        self._tc = st.tc
        self._t = st.t

    # ------------------------------------------------------------------
    # properties (pyqg/kernel.pyx:528-637)
    # ------------------------------------------------------------------
    def __setattr__(self, name, value):
        # before __init__ only record the properties the reference lets
        # subclasses set early (plain attributes pass through)
        if name in _PRE_INIT and not self._ready():
            self.__dict__["_pre"][name] = value
            return
        object.__setattr__(self, name, value)

    @property
    def dt(self):
        return self._dt

    @dt.setter
    def dt(self, dt):
        self._dt = float(dt)
        self._ablevel = 0  # reset timestepping to forward Euler (:531-534)

    @property
    def t(self):
        return self._t

    @property
    def tc(self):
        return self._tc

    @property
    def ablevel(self):
        return self._ablevel

    @property
    def rek(self):
        return self._rek

    @rek.setter
    def rek(self, rek):
        self._rek = float(rek)
        _lib.check(self._L.pqg_set_rek(self._plan, self._rek))

    @property
    def kk(self):
        return self._kk

    @kk.setter
    def kk(self, k):
        _check_array(k, np.float64, 1, "kk")
        self._kk = np.ascontiguousarray(k)
        self._ik = 1j * self._kk
        self._push_wavenumbers()

    @property
    def ll(self):
        return self._ll

    @ll.setter
    def ll(self, l):
        _check_array(l, np.float64, 1, "ll")
        self._ll = np.ascontiguousarray(l)
        self._il = 1j * self._ll
        self._push_wavenumbers()

    def _push_wavenumbers(self):
        kk = np.ascontiguousarray(self._kk[: self.nk], dtype=np.float64)
        ll = np.ascontiguousarray(self._ll[: self.nl], dtype=np.float64)
        self.__dict__["_k2l2_arr"] = kk[np.newaxis, :] ** 2 + ll[:, np.newaxis] ** 2
        _lib.check(self._L.pqg_set_wavenumbers(self._plan, kk.ctypes.data,
                                               ll.ctypes.data))
        if self._Qy is not None:
            self._ikQy = 1j * (self._kk[np.newaxis, :] * self._Qy[:, np.newaxis])

    @property
    def _k2l2(self):
        return self.__dict__["_k2l2_arr"]

    @_k2l2.setter
    def _k2l2(self, v):
        v = np.ascontiguousarray(_check_array(v, np.float64, 2, "_k2l2"))
        self.__dict__["_k2l2_arr"] = v
        _lib.check(self._L.pqg_set_k2l2(self._plan, v.ctypes.data))

    @property
    def _ik(self):
        return self.__dict__["_ik_arr"]

    @_ik.setter
    def _ik(self, v):
        self.__dict__["_ik_arr"] = v

    @property
    def _il(self):
        return self.__dict__["_il_arr"]

    @_il.setter
    def _il(self, v):
        self.__dict__["_il_arr"] = v

    @property
    def _ikQy(self):
        return self.__dict__.get("_ikQy_arr")

    @_ikQy.setter
    def _ikQy(self, v):
        self.__dict__["_ikQy_arr"] = v

    @property
    def a(self):
        return self._a

    @a.setter
    def a(self, b):
        _check_array(b, np.float64, 4, "a")
        self._a[:] = b.astype(np.complex128)
        ar = np.ascontiguousarray(self._a.real)
        _lib.check(self._L.pqg_set_inversion(self._plan, ar.ctypes.data))

    @property
    def Ubg(self):
        return self._Ubg

    @Ubg.setter
    def Ubg(self, U):
        _check_array(U, np.float64, 1, "Ubg")
        self._Ubg = U
        u = np.zeros(self.nz)
        u[: min(self.nz, U.size)] = U[: self.nz]
        _lib.check(self._L.pqg_set_ubg(self._plan, u.ctypes.data))

    @property
    def Qy(self):
        return self._Qy

    @Qy.setter
    def Qy(self, Qy):
        _check_array(Qy, np.float64, 1, "Qy")
        self._Qy = Qy
        self._ikQy = 1j * (np.asarray(self._kk)[np.newaxis, :] *
                           np.asarray(Qy)[:, np.newaxis])
        q = np.zeros(self.nz)
        q[: min(self.nz, Qy.size)] = Qy[: self.nz]
        _lib.check(self._L.pqg_set_qy(self._plan, q.ctypes.data))

    @property
    def filtr(self):
        return self._filtr

    @filtr.setter
    def filtr(self, f):
        f = np.asarray(f, dtype=np.float64)
        if f.ndim != 2:
            raise ValueError("filtr must be 2-D (nl, nk)")
        self._filtr = np.ascontiguousarray(np.broadcast_to(f, (self.nl, self.nk)))
        _lib.check(self._L.pqg_set_filter(self._plan, self._filtr.ctypes.data))

    # -- state ------------------------------------------------------------
    @property
    def q(self):
        return self._get("q")

    @q.setter
    def q(self, b):
        _check_array(b, np.float64, 3, "q")
        if b.shape != (self.nz, self.ny, self.nx):
            raise ValueError("q has shape %s, expected %s"
                             % (b.shape, (self.nz, self.ny, self.nx)))
        self._sync_in()
        self._upload("q", b)
        _lib.check(self._L.pqg_rfft2(self._plan, self._ptr("q"), self._ptr("qh"),
                                     self.nz, self._sp()))

    @property
    def qh(self):
        return self._get("qh")

    @qh.setter
    def qh(self, b):
        _check_array(b, np.complex128, 3, "qh")
        if b.shape != (self.nz, self.nl, self.nk):
            raise ValueError("qh has shape %s, expected %s"
                             % (b.shape, (self.nz, self.nl, self.nk)))
        self._sync_in()
        self._upload("qh", b)
        _lib.check(self._L.pqg_irfft2(self._plan, self._ptr("qh"), self._ptr("q"),
                                      self.nz, self._sp()))

    @property
    def ufull(self):
        return self._get("u") + np.asarray(self._Ubg)[:, np.newaxis, np.newaxis]

    @property
    def vfull(self):
        return self._get("v")

    # -- checkpoint / exact resume ------------------------------------------
    def save_checkpoint(self, path):
        """Write the complete time-stepping state to `path` (.npz): q, qh,
        the three tendencies, ablevel, t, tc, dt.  Loading it into a model
        built with the same parameters resumes the run bit for bit (the
        reference's snapshot output drops the Adams-Bashforth history)."""
        state = dict(q=self._get("q").copy(), qh=self._get("qh").copy(),
                     dqhdt=self._get("dqhdt").copy(),
                     dqhdt_p=self._get("dqhdt_p").copy(),
                     dqhdt_pp=self._get("dqhdt_pp").copy(),
                     ablevel=np.int64(self._ablevel), t=np.float64(self._t),
                     tc=np.int64(self._tc), dt=np.float64(self._dt),
                     shape=np.array([self.nz, self.ny, self.nx]),
                     engine=np.array(self._engine))
        np.savez(path, **state)

    def load_checkpoint(self, path):
        """Restore a state written by :meth:`save_checkpoint`."""
        with np.load(path, allow_pickle=False) as f:
            st = {k: f[k] for k in f.files}
        if tuple(st["shape"]) != (self.nz, self.ny, self.nx):
            raise ValueError("checkpoint grid %s does not match this model %s"
                             % (tuple(st["shape"]), (self.nz, self.ny, self.nx)))
        self._sync_in()
        self._role = {"dqhdt": 0, "dqhdt_p": 1, "dqhdt_pp": 2}
        for name in ("q", "qh", "dqhdt", "dqhdt_p", "dqhdt_pp"):
            self._upload(name, st[name])
        self._stream.synchronize()
        self._dt = float(st["dt"])
        self._ablevel = int(st["ablevel"])
        self._t = float(st["t"])
        self._tc = int(st["tc"])
        if str(st["engine"]) != self._engine:
            self.engine = str(st["engine"])

    # -- non-finite state ------------------------------------------------
    @property
    def nonfinite(self):
        """True once a step has produced an Inf or NaN spectral PV value.
        The step kernels set the flag in host-mapped memory, so reading it
        does not synchronize: it covers the steps that have completed."""
        flag = ctypes.c_int(0)
        _lib.check(self._L.pqg_nonfinite(self._plan, ctypes.byref(flag)))
        return bool(flag.value)

    def clear_nonfinite(self):
        """Reset the non-finite flag (waits for the queued steps first)."""
        self._stream.synchronize()
        _lib.check(self._L.pqg_clear_nonfinite(self._plan))

    # -- device views (no host copy): for GPU-side parameterizations -------
    def device_field(self, name):
        """The device tensor holding field `name` (read it, do not keep it
        across steps: history buffers change roles)."""
        self._sync_in()
        return self._buf(name)


def _field_property(name):
    def getter(self):
        return self._get(name)
    getter.__name__ = name
    return property(getter)


for _n in ("ph", "u", "v", "uh", "vh", "uq", "vq", "uqh", "vqh", "dqh", "duh",
           "dvh", "dqhdt", "dqhdt_p", "dqhdt_pp"):
    setattr(PseudoSpectralKernel, _n, _field_property(_n))

_PRE_INIT = ("Ubg", "Qy", "a", "kk", "ll", "filtr", "rek", "dt", "q", "qh")


# ---------------------------------------------------------------------------
# Module-level time-stepping helpers (pyqg/kernel.pyx:640-663).  pyqg's
# Model imports them from its kernel module (pyqg/model.py:8), so they are
# part of the module's interface; they act on host complex arrays, typed as
# the reference's (double dt, complex128 arrays of three dimensions).
# ---------------------------------------------------------------------------
def _tendency_args(dt, *arrays):
    dt = float(dt)
    for i, x in enumerate(arrays):
        _check_array(x, np.complex128, 3, "dqdt" + "_p" * i)
    return dt


def tendency_forward_euler(dt, dqdt):
    """Forward Euler tendency dt * dqdt."""
    dt = _tendency_args(dt, dqdt)
    return dt * dqdt


def tendency_ab2(dt, dqdt, dqdt_p):
    """Second-order Adams-Bashforth tendency."""
    dt = _tendency_args(dt, dqdt, dqdt_p)
    return (1.5 * dt) * dqdt + (-0.5 * dt) * dqdt_p


def tendency_ab3(dt, dqdt, dqdt_p, dqdt_pp):
    """Third-order Adams-Bashforth tendency."""
    dt = _tendency_args(dt, dqdt, dqdt_p, dqdt_pp)
    return ((23 / 12. * dt) * dqdt + (-16 / 12. * dt) * dqdt_p
            + (5 / 12. * dt) * dqdt_pp)
