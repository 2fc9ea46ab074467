"""Subgrid parameterizations (same API as ``pyqg/parameterizations.py``).

A parameterization is a callable taking the model and returning either a
(nz, ny, nx) array to add to dq/dt (``q_parameterization``) or a pair
(du, dv) whose curl is added (``uv_parameterization``).  The physical closures
below use the model's ``fft`` / ``ifft`` (CUDA transforms).
"""
from abc import ABC, abstractmethod

import numpy as np

__all__ = ["Parameterization", "CompositeParameterization",
           "WeightedParameterization", "UVParameterization",
           "QParameterization", "Smagorinsky", "BackscatterBiharmonic",
           "ZannaBolton2020", "RingForcing"]


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
        return np.sum([p(m) for p in self.params], axis=0)

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
        return np.array(self.param(m)) * self.weight

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

    def __call__(self, m, just_viscosity=False):
        uh = m.fft(m.u)
        vh = m.fft(m.v)
        Sxx = m.ifft(uh * m.ik)
        Syy = m.ifft(vh * m.il)
        Sxy = 0.5 * m.ifft(uh * m.il + vh * m.ik)
        nu = (self.constant * m.dx) ** 2 * np.sqrt(2 * (Sxx ** 2 + Syy ** 2 + 2 * Sxy ** 2))
        if just_viscosity:
            return nu
        nSxx = m.fft(nu * Sxx)
        nSxy = m.fft(nu * Sxy)
        nSyy = m.fft(nu * Syy)
        du = 2 * (m.ifft(nSxx * m.ik) + m.ifft(nSxy * m.il))
        dv = 2 * (m.ifft(nSxy * m.ik) + m.ifft(nSyy * m.il))
        return du, dv

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
        lap = m.ik ** 2 + m.il ** 2
        psi = m.ifft(m.ph)
        lap_lap_psi = m.ifft(lap ** 2 * m.ph)
        nu = self.smagorinsky(m, just_viscosity=True)
        dissipation = -m.ifft(lap * m.fft(lap_lap_psi * m.dx ** 2 * nu))
        num = np.sum(m.Hi * np.mean(psi * dissipation, axis=(-1, -2)))
        den = np.sum(m.Hi * np.mean(psi * lap_lap_psi, axis=(-1, -2))) + self.eps
        backscatter = -self.back_constant * lap_lap_psi * (num / den)
        return dissipation + backscatter

    def __repr__(self):
        return (f"BackscatterBiharmonic(Cs={self.smagorinsky.constant}, "
                f"Cb={self.back_constant})")


class ZannaBolton2020(UVParameterization):
    """Equation-discovered velocity closure of Zanna & Bolton (2020), eq. 6."""

    def __init__(self, constant=-46761284):
        self.constant = constant

    def __call__(self, m):
        uh = m.fft(m.u)
        vh = m.fft(m.v)
        vx = m.ifft(vh * m.ik)
        vy = m.ifft(vh * m.il)
        ux = m.ifft(uh * m.ik)
        uy = m.ifft(uh * m.il)
        rel_vort = vx - uy
        shearing = vx + uy
        stretching = ux - vy
        rv_stretch = m.fft(rel_vort * stretching)
        rv_shear = m.fft(rel_vort * shearing)
        sum_sqs = m.fft(rel_vort ** 2 + shearing ** 2 + stretching ** 2) / 2.0
        kappa = self.constant
        du = kappa * m.ifft(m.ik * (sum_sqs - rv_shear) + m.il * rv_stretch)
        dv = kappa * m.ifft(m.il * (sum_sqs + rv_shear) + m.ik * rv_stretch)
        return du, dv

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
        nhx, nhy = m.wv.shape
        wvx = np.sqrt(m.k ** 2. + m.l ** 2.)
        mask = np.ones_like(wvx)
        mask[wvx <= self.k_in_forc] = 0.
        mask[wvx > self.k_out_forc] = 0.
        ring_hat = mask * (np.random.randn(nhx, nhy) + 1j * np.random.randn(nhx, nhy))
        if self.layers == 'all':
            ring = m.ifft(ring_hat[np.newaxis, :, :])
        else:
            ring = np.zeros_like(m.u)
            if self.layers == 'surf':
                ring[0] = m.ifft(ring_hat[np.newaxis, :, :])[0]
            elif self.layers == 'bottom':
                ring[-1] = m.ifft(ring_hat[np.newaxis, :, :])[-1]
        ring = ring - ring.mean(axis=(-1, -2))[:, np.newaxis, np.newaxis]
        ring = ring / np.abs(ring).mean(axis=(-1, -2))[:, np.newaxis, np.newaxis]
        return self.mag_noise_forc * ring

    def __repr__(self):
        return f"RingForcing(k_in_forc={self.k_in_forc}, k_out_forc={self.k_out_forc})"
