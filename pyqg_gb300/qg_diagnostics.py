"""Diagnostics shared by the layered models (``pyqg/qg_diagnostics.py``)."""
import numpy as np

from . import model


class QGDiagnostics(model.Model):
    """Adds barotropic enstrophy and parameterization-flux diagnostics, and
    the layer-weighted KE and CFL of the multi-layer models."""

    def _layer_sum(self, x):
        """sum_z Hi[z] x[z] / H"""
        return (self.Hi[:, np.newaxis, np.newaxis] * x).sum(axis=0) / self.H

    def _initialize_model_diagnostics(self):
        M2 = self.M ** 2
        add = self.add_diagnostic
        add('entspec', gpu=True, description='barotropic enstrophy spectrum',
            function=lambda m: np.abs(m._layer_sum(m.qh)) ** 2 / m.M ** 2,
            units='m s^-2', dims=('l', 'k'))
        add('paramspec_APEflux', gpu=True,
            description='total additional APE flux due to subgrid parameterization',
            function=lambda m: -m._calc_paramspec_contribution(np.einsum(
                "ij, jk..., k... -> i...", m.S, m.a,
                m._calc_parameterization_contribution())),
            units='m^2 s^-3', dims=('l', 'k'), skip_comparison=True)
        add('paramspec_KEflux', gpu=True,
            description='total additional KE flux due to subgrid parameterization',
            function=lambda m: m.wv2 * m._calc_paramspec_contribution(np.einsum(
                "ij..., j... -> i...", m.a, m._calc_parameterization_contribution())),
            units='m^2 s^-3', dims=('l', 'k'), skip_comparison=True)
        add('ENSflux', gpu=True, description='barotropic enstrophy flux',
            function=lambda m: -m._layer_sum((m.qh.conj() * m.Jq).real) / m.M ** 2,
            units='s^-3', dims=('l', 'k'))
        add('ENSgenspec', gpu=True,
            description='the spectrum of the rate of generation of barotropic enstrophy',
            function=lambda m: m._layer_sum(((m.ilQx - m.ikQy) * m.Sph.conj() * m.ph).real) / m.M ** 2,
            units='s^-3', dims=('l', 'k'))
        add('ENSfrictionspec', gpu=True,
            description='the spectrum of the rate of dissipation of barotropic enstrophy due to bottom friction',
            function=lambda m: m.rek * m.Hi[-1] / m.H * m.wv2 *
            (m.qh[-1].conj() * m.ph[-1]).real / m.M ** 2,
            units='s^-3', dims=('l', 'k'))
        add('APEgenspec', gpu=True,
            description='the spectrum of the rate of generation of available potential energy',
            function=lambda m: m._layer_sum(
                (m.Ubg[:, np.newaxis, np.newaxis] * m.k + m.Vbg[:, np.newaxis, np.newaxis] * m.l) *
                (1j * m.ph.conj() * m.Sph).real) / m.M ** 2,
            units='m^2 s^-3', dims=('l', 'k'))
        del M2

    def _calc_paramspec_contribution(self, term):
        return np.real(self._height_ratios() * self.ph.conj() * term).sum(axis=0) / self.M ** 2

    def _calc_cfl(self):
        return np.abs(np.hstack([self.u + self.Ubg[:, np.newaxis, np.newaxis],
                                 self.v])).max() * self.dt / self.dx

    def _calc_ke(self):
        """Layer-weighted kinetic energy (m^2 s^-2)."""
        ke = 0.
        ph = self.ph
        for j in range(self.nz):
            ke += .5 * self.Hi[j] * self.spec_var(self.wv * ph[j])
        return ke.sum() / self.H

    def _calc_eddy_time(self):
        """Eddy turnover time estimate (days)."""
        ens = 0.
        ph = self.ph
        for j in range(self.nz):
            ens = .5 * self.Hi[j] * self.spec_var(self.wv2 * ph[j])
        return 2. * np.pi * np.sqrt(self.H / ens.sum()) / 86400
