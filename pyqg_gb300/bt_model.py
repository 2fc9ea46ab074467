"""Single-layer (barotropic / equivalent-barotropic) QG model, same API as
``pyqg.BTModel`` (``pyqg/bt_model.py:6-110``)."""
import numpy as np

from . import model


class BTModel(model.Model):
    r"""dq/dt + J(psi, q) + beta psi_x = ssd,  q = lap psi - kd^2 psi."""

    def __init__(self, beta=0., rd=None, H=1., U=0., **kwargs):
        self.beta = beta
        self.rd = rd
        self.H = H
        self.Hi = np.array(H)[np.newaxis, ...]
        self.U = U
        self.nz = 1
        self.kd2 = rd ** -2 if rd else 0.
        super().__init__(**kwargs)
        # unseeded initial condition of the reference (pyqg/bt_model.py:62)
        self.q = 1e-3 * np.random.rand(1, self.ny, self.nx)

    def _initialize_background(self):
        self.Qy = np.asarray(self.beta)[np.newaxis, ...]
        self.set_U(self.U)
        self.ikQy = self.Qy * 1j * self.k
        self.ilQx = 0.

    def _initialize_inversion_matrix(self):
        # ph = -(kappa^2 + kd^2)^-1 qh (pyqg/bt_model.py:78-85)
        if self.rd:
            self.a = -(1. / (self.wv2 + self.kd2))[np.newaxis, np.newaxis, :, :]
        else:
            self.a = -self.wv2i[np.newaxis, np.newaxis, :, :]

    def _initialize_forcing(self):
        pass

    def set_U(self, U):
        """Set the background zonal flow."""
        self.Ubg = np.asarray(U)[np.newaxis, ...]

    def _diagnostics_due(self, t, tc):
        # no tavestart condition for the single-layer models
        return (t >= self.dt) and (tc % self.taveints == 0)

    def _calc_cfl(self):
        return np.abs(np.hstack([self.u + self.Ubg, self.v])).max() * self.dt / self.dx

    def _calc_ke(self):
        return (.5 * self.spec_var(self.wv * self.ph)).sum()

    def _calc_eddy_time(self):
        ens = .5 * self.H * self.spec_var(self.wv2 * self.ph)
        return 2. * np.pi * np.sqrt(self.H / ens) / 86400
