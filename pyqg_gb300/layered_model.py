"""N-layer quasigeostrophic model (same API as ``pyqg.LayeredModel``,
``pyqg/layered_model.py:17-303``)."""
import numpy as np

from . import qg_diagnostics


def stretching_matrix(nz, f2, Hi, gpi, rd=None, delta=None):
    """Stretching matrix S (m^-2) of ``pyqg/layered_model.py:136-168``:
    the two-layer (rd, delta) form when both are given for nz = 2, otherwise
    the tridiagonal f^2 / (H_i g'_i) form."""
    S = np.zeros((nz, nz))
    if nz == 2 and rd and delta:
        F1 = rd ** -2 / (1. + delta)
        F2 = delta * F1
        S[0, 0], S[0, 1] = -F1, F1
        S[1, 0], S[1, 1] = F2, -F2
        return S
    for i in range(nz):
        if i == 0:
            S[i, i] = -f2 / Hi[i] / gpi[i]
            S[i, i + 1] = f2 / Hi[i] / gpi[i]
        elif i == nz - 1:
            S[i, i] = -f2 / Hi[i] / gpi[i - 1]
            S[i, i - 1] = f2 / Hi[i] / gpi[i - 1]
        else:
            S[i, i - 1] = f2 / Hi[i] / gpi[i - 1]
            S[i, i] = -(f2 / Hi[i] / gpi[i] + f2 / Hi[i] / gpi[i - 1])
            S[i, i + 1] = f2 / Hi[i] / gpi[i]
    return S


def layered_inversion_matrix(S, wv2):
    """a = (S - kappa^2 I)^-1 per wavenumber, 0 at kappa = 0
    (``pyqg/layered_model.py:211-229``)."""
    nz = S.shape[0]
    nl, nk = wv2.shape
    a = np.ma.zeros((nz, nz, nl, nk), np.dtype('float64'))
    if nz == 2:
        det_inv = np.ma.masked_equal(
            (S[0, 0] - wv2) * (S[1, 1] - wv2) - S[0, 1] * S[1, 0], 0.) ** -1
        a[0, 0] = (S[1, 1] - wv2) * det_inv
        a[0, 1] = -S[0, 1] * det_inv
        a[1, 0] = -S[1, 0] * det_inv
        a[1, 1] = (S[0, 0] - wv2) * det_inv
    else:
        eye = np.eye(nz)[:, :, np.newaxis, np.newaxis]
        Mx = S[:, :, np.newaxis, np.newaxis] - eye * wv2
        Mx[:, :, 0, 0] = np.nan   # kappa = 0 is singular
        a = np.linalg.inv(Mx.T).T
    return np.ma.masked_invalid(a).filled(0.)


class LayeredModel(qg_diagnostics.QGDiagnostics):
    """Layered QG model with background flow (U, V), layer thicknesses H and
    densities rho (reduced gravities g'_i = g (rho_{i+1} - rho_i) / rho_i)."""

    def __init__(self, beta=1.5e-11, nz=3, rd=15000.0,
                 f=0.0001236812857687059, H=None, U=None, V=None, rho=None,
                 delta=None, **kwargs):
        self.beta = beta
        self.rd = rd
        self.delta = delta
        if U is None:
            U = (np.arange(nz) * 0.025)[::-1]
        if V is None:
            V = np.zeros(nz)
        if H is None:
            H = [500] + [1750 for _ in range(nz - 1)]
        if rho is None:
            rho = np.arange(nz) * 0.3 + 1025
        self.Ubg = np.array(U)
        self.Vbg = np.array(V)
        self.Hi = np.array(H)
        self.rhoi = np.array(rho)
        super().__init__(nz=nz, f=f, **kwargs)
        self.vertical_modes()
        # unseeded initial condition of the reference
        # (pyqg/layered_model.py:130-132)
        self.q = 1e-7 * np.vstack([np.random.randn(self.nx, self.ny)[np.newaxis, ]
                                   for _ in range(nz)])

    def set_q(self, q):
        self.q = np.ascontiguousarray(q, dtype=np.float64)

    def _initialize_stretching_matrix(self):
        if self.nz == 2 and self.rd and self.delta:
            self.del1 = self.delta / (self.delta + 1.)
            self.del2 = (self.delta + 1.) ** -1
            self.Us = self.Ubg[0] - self.Ubg[1]
            self.F1 = self.rd ** -2 / (1. + self.delta)
            self.F2 = self.delta * self.F1
        self.S = stretching_matrix(self.nz, getattr(self, "f2", None), self.Hi,
                                   getattr(self, "gpi", None), self.rd, self.delta)

    def _initialize_background(self):
        self.H = self.Hi.sum()
        if self.nz != 2:
            self.gpi = self.g * (self.rhoi[1:] - self.rhoi[:-1]) / self.rhoi[:-1]
            self.f2gpi = (self.f2 / self.gpi)[:, np.newaxis, np.newaxis]
            assert self.gpi.size == self.nz - 1, "Invalid size of gpi"
            assert np.all(self.gpi > 0.), "Buoyancy jump has negative sign!"
            assert self.Hi.size == self.nz, self.logger.error(
                'size of Hi does not' + 'match number of vertical levels nz')
            assert self.rhoi.size == self.nz, self.logger.error(
                'size of rhoi does not' + 'match number of vertical levels nz')
            assert self.Ubg.size == self.nz, self.logger.error(
                'size of Ubg does not' + 'match number of vertical levels nz')
            assert self.Vbg.size == self.nz, self.logger.error(
                'size of Vbg does not' + 'match number of vertical levels nz')
        else:
            self.f2gpi = np.array(self.rd ** -2 *
                                  (self.Hi[0] * self.Hi[1]) / self.H)[np.newaxis, np.newaxis]
            if not (self.rd and self.delta):
                self.gpi = self.g * (self.rhoi[1:] - self.rhoi[:-1]) / self.rhoi[:-1]
        self._initialize_stretching_matrix()
        self.Qy = self.beta - np.dot(self.S, self.Ubg)
        self.Qx = np.dot(self.S, self.Vbg)
        self.ikQy = self.Qy[:, np.newaxis, np.newaxis] * 1j * self.k
        self.ilQx = self.Qx[:, np.newaxis, np.newaxis] * 1j * self.l

    def _initialize_inversion_matrix(self):
        self.a = layered_inversion_matrix(self.S, self.wv2)

    def _initialize_forcing(self):
        pass

    def _calc_derived_fields(self):
        u, v = self.u, self.v
        self.p = self.ifft(self.ph)
        self.xi = self.ifft(-self.wv2 * self.ph)
        self.Jpxi = self._advect(self.xi, u, v)
        self.Jq = self._advect(self.q, u, v)
        self.Sph = np.einsum("ij,jkl->ikl", self.S, self.ph)
        self.Sp = self.ifft(self.Sph)
        self.JSp = self._advect(self.Sp, u, v)
        self.phn = self.modal_projection(self.ph)

    def _initialize_model_diagnostics(self):
        super()._initialize_model_diagnostics()
        add = self.add_diagnostic
        add('KEspec_modal', gpu=True, description='modal kinetic energy spectra',
            function=lambda m: m.wv2 * (np.abs(m.phn) ** 2) / m.M ** 2,
            units='m^2 s^-2', dims=('lev', 'l', 'k'))
        add('PEspec_modal', gpu=True, description='modal potential energy spectra',
            function=lambda m: m.kdi2[1:, np.newaxis, np.newaxis] *
            (np.abs(m.phn[1:, :, :]) ** 2) / m.M ** 2,
            units='m^2 s^-2', dims=('lev_mid', 'l', 'k'))
        add('APEspec', gpu=True, description='available potential energy spectrum',
            function=lambda m: (m.f2gpi * np.abs(m.ph[:-1] - m.ph[1:]) ** 2).sum(axis=0)
            / m.H / m.M ** 2,
            units='m^2 s^-2', dims=('l', 'k'))
        add('KEflux_div', gpu=True, description='spectral divergence of flux of kinetic energy',
            function=lambda m: m._layer_sum((m.ph.conj() * m.Jpxi).real) / m.M ** 2,
            units='m^2 s^-3', dims=('l', 'k'), sums_with=['paramspec_KEflux'])
        add('APEflux_div', gpu=True,
            description='spectral divergence of flux of available potential energy',
            function=lambda m: m._layer_sum((m.ph.conj() * m.JSp).real) / m.M ** 2,
            units='m^2 s^-3', dims=('l', 'k'), sums_with=['paramspec_APEflux'])
