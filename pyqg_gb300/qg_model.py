"""Two-layer quasigeostrophic model (same API as ``pyqg.QGModel``,
``pyqg/qg_model.py:17-263``)."""
import numpy as np

from . import qg_diagnostics


def qg_inversion_matrix(wv2, F1, F2):
    """Two-layer inversion ph = a qh per wavenumber
    (``pyqg/qg_model.py:146-161``): a = inverse of [[-(k2+F1), F1],
    [F2, -(k2+F2)]], set to 0 at kappa = 0 where it is singular."""
    nl, nk = wv2.shape
    a = np.ma.zeros((2, 2, nl, nk), np.dtype('float64'))
    det_inv = np.ma.masked_equal(wv2 * (wv2 + F1 + F2), 0.) ** -1
    a[0, 0] = -(wv2 + F2) * det_inv
    a[0, 1] = -F1 * det_inv
    a[1, 0] = -F2 * det_inv
    a[1, 1] = -(wv2 + F1) * det_inv
    return np.ma.masked_invalid(a).filled(0.)


class QGModel(qg_diagnostics.QGDiagnostics):
    r"""Two-layer quasigeostrophic model driven by the shear U1 - U2.

    q1 = lap psi1 + F1 (psi2 - psi1),  q2 = lap psi2 + F2 (psi1 - psi2),
    F1 = rd^-2 / (1 + delta), F2 = delta F1, delta = H1 / H2.
    """

    def __init__(self, beta=1.5e-11, rd=15000.0, delta=0.25, H1=500,
                 U1=0.025, U2=0.0, **kwargs):
        self.beta = beta
        self.rd = rd
        self.delta = delta
        self.Hi = np.array([H1, H1 / delta])
        self.U1 = U1
        self.U2 = U2
        super().__init__(nz=2, **kwargs)
        # unseeded initial condition of the reference (pyqg/qg_model.py:103-106)
        self.set_q1q2(
            1e-7 * np.random.rand(self.ny, self.nx) + 1e-6 * (
                np.ones((self.ny, 1)) * np.random.rand(1, self.nx)),
            np.zeros_like(self.x))

    def _initialize_background(self):
        self.H = self.Hi.sum()
        self.set_U1U2(self.U1, self.U2)
        self.U = self.U1 - self.U2
        self.Vbg = np.zeros_like(self.Ubg)
        self.F1 = self.rd ** -2 / (1. + self.delta)
        self.F2 = self.delta * self.F1
        self.Qy1 = self.beta + self.F1 * (self.U1 - self.U2)
        self.Qy2 = self.beta - self.F2 * (self.U1 - self.U2)
        self.Qy = np.array([self.Qy1, self.Qy2])
        self.ikQy1 = self.Qy1 * 1j * self.k
        self.ikQy2 = self.Qy2 * 1j * self.k
        self.ikQy = np.vstack([self.ikQy1[np.newaxis, ...],
                               self.ikQy2[np.newaxis, ...]])
        self.ilQx = 0.
        self.del1 = self.delta / (self.delta + 1.)
        self.del2 = (self.delta + 1.) ** -1

    @property
    def S(self):
        """Stretching matrix."""
        return np.array([[-self.F1, self.F1],
                         [self.F2, -self.F2]]).astype(np.float64)

    def _initialize_inversion_matrix(self):
        self.a = qg_inversion_matrix(self.wv2, self.F1, self.F2)

    def _initialize_forcing(self):
        pass

    def set_q1q2(self, q1, q2, check=False):
        """Set upper and lower layer PV anomalies."""
        self.set_q(np.vstack([q1[np.newaxis, :, :], q2[np.newaxis, :, :]]))
        if check:
            np.testing.assert_allclose(self.q[0], q1)
            np.testing.assert_allclose(self.q[1], q2)

    def set_q(self, q):
        self.q = np.ascontiguousarray(q, dtype=np.float64)

    def set_U1U2(self, U1, U2):
        """Set the background zonal flow of both layers."""
        self.U1 = U1
        self.U2 = U2
        self.Ubg = np.array([U1, U2])

    def _calc_derived_fields(self):
        self.p = self.ifft(self.ph)
        self.xi = self.ifft(-self.wv2 * self.ph)
        u, v = self.u, self.v
        self.Jptpc = -self._advect(
            (self.p[0] - self.p[1]),
            (self.del1 * u[0] + self.del2 * u[1]),
            (self.del1 * v[0] + self.del2 * v[1]))
        self.Jpxi = self._advect(self.xi, u, v)
        self.Jq = self._advect(self.q, u, v)
        self.Sph = np.einsum("ij,jkl->ikl", self.S, self.ph)

    def _initialize_model_diagnostics(self):
        super()._initialize_model_diagnostics()
        add = self.add_diagnostic
        add('APEflux', gpu=True, description='spectral flux of available potential energy',
            function=lambda m: m.rd ** -2 * m.del1 * m.del2 *
            np.real((m.ph[0] - m.ph[1]) * np.conj(m.Jptpc)) / m.M ** 2,
            units='m^2 s^-3', dims=('l', 'k'), sums_with=['paramspec_APEflux'])
        add('KEflux', gpu=True, description='spectral flux of kinetic energy',
            function=lambda m: (np.real(m.del1 * m.ph[0] * np.conj(m.Jpxi[0])) +
                                np.real(m.del2 * m.ph[1] * np.conj(m.Jpxi[1]))) / m.M ** 2,
            units='m^2 s^-3', dims=('l', 'k'), sums_with=['paramspec_KEflux'])
        add('APEgen', gpu=True, description='total available potential energy generation',
            function=lambda m: m._ape_generation(),
            units='m^2 s^-3', dims=('time',))

    def _ape_generation(self):
        """Domain-total APE generation by the mean shear; the interior k
        columns are counted twice for the missing half plane (the reference
        uses the slice 1:-2 for them)."""
        ph = self.ph
        bt = self.del1 * ph[0] + self.del2 * ph[1]
        bc = np.conj(ph[0] - ph[1])
        full = (1j * self.k * bt * bc).sum()
        half = (1j * self.k[:, 1:-2] * bt[:, 1:-2] * bc[:, 1:-2]).sum()
        return self.U * self.rd ** -2 * self.del1 * self.del2 * np.real(full + half) / self.M ** 2
