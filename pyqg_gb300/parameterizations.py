"""Subgrid parameterizations (same API as ``pyqg/parameterizations.py``).

A parameterization is a callable taking the model and returning either a
(nz, ny, nx) array to add to dq/dt (``q_parameterization``) or a pair
(du, dv) whose curl is added (``uv_parameterization``).

The physical closures below run on the GPU: their inputs are the model's
device fields, their transforms the model's CUDA transforms and their
pointwise arithmetic CUDA tensors.  Called by the model's step (the hook)
they return CUDA tensors, which the step consumes without a host copy;
called directly they return numpy arrays, as the reference's do.
"""
from abc import ABC, abstractmethod

import numpy as np

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
    du = 2 (d_x(nu Sxx) + d_y(nu Sxy)), dv = 2 (d_x(nu Sxy) + d_y(nu Syy))."""

    def __init__(self, constant=0.1):
        self.constant = constant

    def _viscosity(self, m):
        import torch
        ik, il = _dev(m, "ik"), _dev(m, "il")
        uh = m.fft(m.device_field("u"))
        vh = m.fft(m.device_field("v"))
        Sxx = m.ifft(uh * ik)
        Syy = m.ifft(vh * il)
        Sxy = 0.5 * m.ifft(uh * il + vh * ik)
        nu = (self.constant * m.dx) ** 2 * torch.sqrt(2 * (Sxx ** 2 + Syy ** 2 + 2 * Sxy ** 2))
        return nu, Sxx, Syy, Sxy

    def __call__(self, m, just_viscosity=False):
        nu, Sxx, Syy, Sxy = self._viscosity(m)
        if just_viscosity:
            return _as_output(m, nu)
        ik, il = _dev(m, "ik"), _dev(m, "il")
        nSxx = m.fft(nu * Sxx)
        nSxy = m.fft(nu * Sxy)
        nSyy = m.fft(nu * Syy)
        du = 2 * (m.ifft(nSxx * ik) + m.ifft(nSxy * il))
        dv = 2 * (m.ifft(nSxy * ik) + m.ifft(nSyy * il))
        return _as_output(m, (du, dv))

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
        ik, il = _dev(m, "ik"), _dev(m, "il")
        Hi = _dev(m, "Hi")
        ph = m.device_field("ph")
        lap = ik ** 2 + il ** 2
        psi = m.ifft(ph)
        lap_lap_psi = m.ifft(lap ** 2 * ph)
        nu = self.smagorinsky._viscosity(m)[0]
        dissipation = -m.ifft(lap * m.fft(lap_lap_psi * m.dx ** 2 * nu))
        num = (Hi * (psi * dissipation).mean(dim=(-1, -2))).sum()
        den = (Hi * (psi * lap_lap_psi).mean(dim=(-1, -2))).sum() + self.eps
        backscatter = -self.back_constant * lap_lap_psi * (num / den)
        return _as_output(m, dissipation + backscatter)

    def __repr__(self):
        return (f"BackscatterBiharmonic(Cs={self.smagorinsky.constant}, "
                f"Cb={self.back_constant})")


class ZannaBolton2020(UVParameterization):
    """Equation-discovered velocity closure of Zanna & Bolton (2020), eq. 6."""

    def __init__(self, constant=-46761284):
        self.constant = constant

    def __call__(self, m):
        ik, il = _dev(m, "ik"), _dev(m, "il")
        uh = m.fft(m.device_field("u"))
        vh = m.fft(m.device_field("v"))
        vx = m.ifft(vh * ik)
        vy = m.ifft(vh * il)
        ux = m.ifft(uh * ik)
        uy = m.ifft(uh * il)
        rel_vort = vx - uy
        shearing = vx + uy
        stretching = ux - vy
        rv_stretch = m.fft(rel_vort * stretching)
        rv_shear = m.fft(rel_vort * shearing)
        sum_sqs = m.fft(rel_vort ** 2 + shearing ** 2 + stretching ** 2) / 2.0
        kappa = self.constant
        du = kappa * m.ifft(ik * (sum_sqs - rv_shear) + il * rv_stretch)
        dv = kappa * m.ifft(il * (sum_sqs + rv_shear) + ik * rv_stretch)
        return _as_output(m, (du, dv))

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
        one = m.ifft(torch.from_numpy(ring_hat[np.newaxis]).to(m._device))
        ring = one.expand(m.nz, m.ny, m.nx).clone()
        if self.layers != 'all':
            keep = torch.zeros((m.nz, 1, 1), dtype=ring.dtype, device=ring.device)
            if self.layers == 'surf':
                keep[0] = 1.0
            elif self.layers == 'bottom':
                keep[-1] = 1.0
            ring = ring * keep
        ring = ring - ring.mean(dim=(-1, -2), keepdim=True)
        ring = ring / ring.abs().mean(dim=(-1, -2), keepdim=True)
        return _as_output(m, self.mag_noise_forc * ring)

    def __repr__(self):
        return f"RingForcing(k_in_forc={self.k_in_forc}, k_out_forc={self.k_out_forc})"
