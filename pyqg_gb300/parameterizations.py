"""Subgrid parameterizations (same API as ``pyqg/parameterizations.py``).

A parameterization is a callable taking the model and returning either a
(nz, ny, nx) array to add to dq/dt (``q_parameterization``) or a pair
(du, dv) whose curl is added (``uv_parameterization``).

The physical closures below run on the GPU: their inputs are the model's
device fields, their transforms the model's CUDA transforms and their
pointwise stages the library's kernels (``pqg_smag_*``, ``pqg_zb_*``,
``pqg_lap_power``, ``pqg_mul_scaled``, ``pqg_backscatter``,
``pqg_ring_normalize``); PyTorch only allocates their device buffers.
Called by the model's step (the hook) they return CUDA tensors, which the
step consumes without a host copy; called directly they return numpy
arrays, as the reference's do.
"""
import ctypes
from abc import ABC, abstractmethod

import numpy as np

from . import _lib

__all__ = ["Parameterization", "CompositeParameterization",
           "WeightedParameterization", "UVParameterization",
           "QParameterization", "Smagorinsky", "BackscatterBiharmonic",
           "ZannaBolton2020", "RingForcing"]


def _dev(m, name):
    """Model constant `name` as a cached CUDA tensor."""
    import torch
    val = np.asarray(getattr(m, name))
    cache = m.__dict__.setdefault("_param_consts", {})
    t = cache.get(name)
    if t is None or tuple(t.shape) != val.shape:
        t = torch.from_numpy(np.ascontiguousarray(val)).to(m._device)
        cache[name] = t
    return t


def _p(t):
    return ctypes.c_void_p(t.data_ptr())


def _empty(m, shape, complex_=False):
    import torch
    return torch.empty(shape, dtype=torch.complex128 if complex_ else torch.float64, device=m._device)


def _run(m, name, *args):
    """Call library entry point `name` on the model's stream."""
    _lib.check(getattr(_lib.lib(), name)(*args, m._sp()))


def _as_output(m, x):
    """CUDA tensors inside the model's step, numpy arrays otherwise."""
    if getattr(m, "_hook_on_device", False):
        return x
    if isinstance(x, tuple):
        return tuple(t.cpu().numpy() for t in x)
    return x.cpu().numpy()


def _is_tensor(x):
    return type(x).__module__.startswith("torch")


class Parameterization(ABC):
    """Base class of subgrid parameterizations; supports ``p1 + p2`` and
    ``c * p``."""

    @abstractmethod
    def __call__(self, m):
        """Return the forcing for model `m`."""

    @property
    @abstractmethod
    def parameterization_type(self):
        """``'uv_parameterization'`` or ``'q_parameterization'``."""

    def __add__(self, other):
        return CompositeParameterization(self, other)

    def __mul__(self, constant):
        return WeightedParameterization(self, constant)

    __rmul__ = __mul__


class CompositeParameterization(Parameterization):
    """Sum of parameterizations acting on the same variable."""

    def __init__(self, *params):
        kinds = set(p.parameterization_type for p in params)
        assert len(kinds) == 1, \
            "all parameterizations must target the same variable (uv or q)"
        self.params = params

    @property
    def parameterization_type(self):
        return self.params[0].parameterization_type

    def __call__(self, m):
        outs = [p(m) for p in self.params]
        if isinstance(outs[0], tuple):
            return tuple(sum(o[i] for o in outs) for i in range(len(outs[0])))
        if _is_tensor(outs[0]):
            return sum(outs[1:], outs[0])
        return np.sum(outs, axis=0)

    def __repr__(self):
        return f"CompositeParameterization{self.params}"


class WeightedParameterization(Parameterization):
    """A parameterization scaled by a constant."""

    def __init__(self, param, weight):
        self.param = param
        self.weight = weight

    @property
    def parameterization_type(self):
        return self.param.parameterization_type

    def __call__(self, m):
        out = self.param(m)
        if isinstance(out, tuple):
            return tuple(o * self.weight for o in out)
        if _is_tensor(out):
            return out * self.weight
        return np.array(out) * self.weight

    def __repr__(self):
        return f"{self.weight} * {self.param}"


class UVParameterization(Parameterization):
    """Base of velocity parameterizations."""
    parameterization_type = 'uv_parameterization'


class QParameterization(Parameterization):
    """Base of potential-vorticity parameterizations."""
    parameterization_type = 'q_parameterization'


class Smagorinsky(UVParameterization):
    r"""Smagorinsky (1963) eddy viscosity
    nu = (C_S dx)^2 sqrt(2 (Sxx^2 + Syy^2 + 2 Sxy^2)), forcing
    du = 2 (d_x(nu Sxx) + d_y(nu Sxy)), dv = 2 (d_x(nu Sxy) + d_y(nu Syy))
    (pyqg/parameterizations.py:132-192)."""

    def __init__(self, constant=0.1):
        self.constant = constant

    def _viscosity(self, m, stresses):
        """Device nu (nz, ny, nx) and, if `stresses`, the three stress
        fields nu Sxx, nu Sxy, nu Syy as one (3 nz, ny, nx) array."""
        import torch
        with torch.cuda.stream(m._stream):
            uh = m.fft(m.device_field("u"))
            vh = m.fft(m.device_field("v"))
            n, nl, nk = uh.shape
            kk, ll = _dev(m, "kk"), _dev(m, "ll")
            strain_h = _empty(m, (3 * n, nl, nk), True)
            _run(m, "pqg_smag_strain", n, nl, nk, _p(kk), _p(ll), _p(uh), _p(vh), _p(strain_h))
            strain = m._device_irfft2(strain_h)
            nu = _empty(m, (n, m.ny, m.nx))
            p3 = _empty(m, (3 * n, m.ny, m.nx)) if stresses else None
            _run(m, "pqg_smag_stress", n, m.ny, m.nx, _p(strain), float((self.constant * m.dx) ** 2), _p(nu),
                 _p(p3) if stresses else None)
        return nu, p3

    def __call__(self, m, just_viscosity=False):
        import torch
        nu, p3 = self._viscosity(m, not just_viscosity)
        if just_viscosity:
            return _as_output(m, nu)
        with torch.cuda.stream(m._stream):
            n = nu.shape[0]
            n3 = m._device_rfft2(p3)
            kk, ll = _dev(m, "kk"), _dev(m, "ll")
            d2 = _empty(m, (2 * n, m.nl, m.nk), True)
            _run(m, "pqg_smag_divergence", n, m.nl, m.nk, _p(kk), _p(ll), _p(n3), _p(d2))
            duv = m._device_irfft2(d2)
        return _as_output(m, (duv[:n], duv[n:]))

    def __repr__(self):
        return f"Smagorinsky(Cs={self.constant})"


class BackscatterBiharmonic(QParameterization):
    """Smagorinsky-type biharmonic dissipation with a fraction C_B of the
    dissipated energy returned at large scales (Jansen & Held 2014,
    Jansen et al. 2015)."""

    def __init__(self, smag_constant=0.08, back_constant=0.99, eps=1e-32):
        self.smagorinsky = Smagorinsky(smag_constant)
        self.back_constant = back_constant
        self.eps = eps

    def __call__(self, m):
        import torch
        with torch.cuda.stream(m._stream):
            ph = m.device_field("ph")
            n, nl, nk = ph.shape
            kk, ll = _dev(m, "kk"), _dev(m, "ll")
            psi = m._device_irfft2(ph)
            lap2_ph = _empty(m, (n, nl, nk), True)
            _run(m, "pqg_lap_power", n, nl, nk, _p(kk), _p(ll), 2, 1.0, _p(ph), _p(lap2_ph))
            lap_lap_psi = m._device_irfft2(lap2_ph)
            nu = self.smagorinsky._viscosity(m, False)[0]
            x = _empty(m, (n, m.ny, m.nx))
            _run(m, "pqg_mul_scaled", n * m.ny * m.nx, _p(lap_lap_psi), float(m.dx ** 2), _p(nu), _p(x))
            xh = m._device_rfft2(x)
            yh = _empty(m, (n, nl, nk), True)
            _run(m, "pqg_lap_power", n, nl, nk, _p(kk), _p(ll), 1, 1.0, _p(xh), _p(yh))
            dissipation = m._device_irfft2(yh)      # -ifft(lap X) with lap = -(k^2 + l^2)
            sums = _empty(m, (2 * n,))
            out = _empty(m, (n, m.ny, m.nx))
            _run(m, "pqg_backscatter", n, m.ny, m.nx, _p(psi), _p(dissipation), _p(lap_lap_psi),
                 _p(_dev(m, "Hi")), float(self.back_constant), float(self.eps), _p(sums), _p(out))
        return _as_output(m, out)

    def __repr__(self):
        return (f"BackscatterBiharmonic(Cs={self.smagorinsky.constant}, "
                f"Cb={self.back_constant})")


class ZannaBolton2020(UVParameterization):
    """Equation-discovered velocity closure of Zanna & Bolton (2020), eq. 6."""

    def __init__(self, constant=-46761284):
        self.constant = constant

    def __call__(self, m):
        import torch
        with torch.cuda.stream(m._stream):
            uh = m.fft(m.device_field("u"))
            vh = m.fft(m.device_field("v"))
            n, nl, nk = uh.shape
            kk, ll = _dev(m, "kk"), _dev(m, "ll")
            grad_h = _empty(m, (4 * n, nl, nk), True)
            _run(m, "pqg_zb_gradients", n, nl, nk, _p(kk), _p(ll), _p(uh), _p(vh), _p(grad_h))
            grad = m._device_irfft2(grad_h)        # vx, vy, ux, uy
            prod = _empty(m, (3 * n, m.ny, m.nx))
            _run(m, "pqg_zb_products", n, m.ny, m.nx, _p(grad), _p(prod))
            prod_h = m._device_rfft2(prod)
            d2 = _empty(m, (2 * n, nl, nk), True)
            _run(m, "pqg_zb_combine", n, nl, nk, _p(kk), _p(ll), _p(prod_h), float(self.constant), _p(d2))
            duv = m._device_irfft2(d2)
        return _as_output(m, (duv[:n], duv[n:]))

    def __repr__(self):
        return f"ZannaBolton2020(κ={self.constant:.2e})"


class RingForcing(QParameterization):
    """Vertically uniform stochastic forcing on a ring of wavenumbers
    k_in < |k| <= k_out (Uchida et al. 2023), normalised to unit mean
    absolute amplitude and scaled by `mag_noise_forc`."""

    def __init__(self, k_in_forc=0, k_out_forc=0, mag_noise_forc=0, layers='all'):
        self.k_in_forc = k_in_forc
        self.k_out_forc = k_out_forc
        self.mag_noise_forc = mag_noise_forc
        self.layers = layers

    def __call__(self, m):
        import torch
        nhx, nhy = m.wv.shape
        wvx = np.sqrt(m.k ** 2. + m.l ** 2.)
        mask = np.ones_like(wvx)
        mask[wvx <= self.k_in_forc] = 0.
        mask[wvx > self.k_out_forc] = 0.
        # the random draws stay on numpy's generator, as in the reference
        ring_hat = mask * (np.random.randn(nhx, nhy) + 1j * np.random.randn(nhx, nhy))
        keep = np.ones(m.nz, dtype=np.int32)
        if self.layers != 'all':
            keep[:] = 0
            if self.layers == 'surf':
                keep[0] = 1
            elif self.layers == 'bottom':
                keep[-1] = 1
        with torch.cuda.stream(m._stream):
            one = m.ifft(torch.from_numpy(ring_hat[np.newaxis]).to(m._device))
            keep_d = torch.from_numpy(keep).to(m._device)
            moments = _empty(m, (2,))
            out = _empty(m, (m.nz, m.ny, m.nx))
            _run(m, "pqg_ring_normalize", m.nz, m.ny, m.nx, _p(one), _p(keep_d), float(self.mag_noise_forc),
                 _p(moments), _p(out))
        return _as_output(m, out)

    def __repr__(self):
        return f"RingForcing(k_in_forc={self.k_in_forc}, k_out_forc={self.k_out_forc})"
