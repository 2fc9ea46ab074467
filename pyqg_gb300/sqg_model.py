"""Surface quasigeostrophic model, same API as ``pyqg.SQGModel``
(``pyqg/sqg_model.py:6-96``)."""
import numpy as np

from . import model


class SQGModel(model.Model):
    """Surface QG: ph = f_0 / (N kappa) qh."""

    def __init__(self, beta=0., Nb=1., f_0=1., H=1., U=0., **kwargs):
        self.beta = beta
        self.Nb = Nb
        self.f_0 = f_0
        self.H = H
        self.Hi = np.array(H)[np.newaxis, ...]
        self.U = U
        self.nz = 1
        super().__init__(**kwargs)
        # unseeded initial condition of the reference (pyqg/sqg_model.py:42)
        self.q = 1e-3 * np.random.rand(1, self.ny, self.nx)

    def _initialize_background(self):
        self.Qy = np.asarray(self.beta)[np.newaxis, ...]
        self.set_U(self.U)
        self.ikQy = self.Qy * 1j * self.k
        self.ilQx = 0.

    def _initialize_inversion_matrix(self):
        self.a = np.asarray(self.f_0 / self.Nb * np.sqrt(self.wv2i))[np.newaxis, np.newaxis, :, :]

    def _initialize_forcing(self):
        pass

    def set_U(self, U):
        """Set the background zonal flow."""
        self.Ubg = np.asarray(U)[np.newaxis, ...]

    def _diagnostics_due(self, t, tc):
        return (t >= self.dt) and (tc % self.taveints == 0)

    def _calc_cfl(self):
        return np.abs(np.hstack([self.u + self.Ubg, self.v])).max() * self.dt / self.dx

    def _calc_ke(self):
        return (.5 * self.spec_var(self.wv * self.ph)).sum()
