"""CPU oracle: a numpy restatement of pyqg's pseudo-spectral time step.

TEST INFRASTRUCTURE ONLY.  Only ``tests/``, ``__graft_entry__.smoke()`` and
``bench.py``'s CPU-baseline leg may import this module, and only to compare
against (or as the timed CPU baseline); the product path never calls it.

Each function restates one stage of the reference ``PseudoSpectralKernel``
(``pyqg/kernel.pyx``) with the same arithmetic order, using ``numpy.fft``
(pocketfft) -- the same FFT the reference uses when pyFFTW is absent
(``pyqg/kernel.pyx:17-19,245-267``).  Against the compiled reference kernel it
is pinned bit-for-bit by ``tests/test_oracle.py`` (golden vectors in
``tests/golden/`` made by ``tests/golden/make_golden.py``).

Array layouts are the reference's: physical fields ``(nz, ny, nx)`` float64,
spectral fields ``(nz, nl, nk)`` complex128 with ``nl = ny``, ``nk = nx//2+1``.
"""
import numpy as np
import numpy.fft as npfft


def rfft2(x):
    """Forward real 2-D transform over the last two axes, unnormalised
    (``pyqg/kernel.pyx:246-263``: ``npfft.rfftn(..., axes=(-2,-1))``)."""
    return npfft.rfftn(x, axes=(-2, -1))


def irfft2(xh):
    """Inverse real 2-D transform, scaled by ``1/(nx*ny)``
    (``pyqg/kernel.pyx:248-253``: ``npfft.irfftn(..., axes=(-2,-1))``)."""
    return npfft.irfftn(xh, axes=(-2, -1))


class OracleKernel:
    """Stateful restatement of ``PseudoSpectralKernel`` (``pyqg/kernel.pyx:32``).

    Constants are given explicitly (the reference receives them through its
    property setters, ``pyqg/kernel.pyx:528-575``):

    ``a``      (nz, nz, nl, nk) real inversion matrix
    ``kk``     (nk,) zonal wavenumbers, ``ll`` (nl,) meridional wavenumbers
    ``Ubg``    (nz,) background zonal velocity, ``Qy`` (nz,) PV gradient
    ``filtr``  (nl, nk) spectral filter, ``rek`` bottom drag, ``dt`` step
    """

    def __init__(self, nz, ny, nx, a, kk, ll, Ubg, Qy, filtr, rek, dt):
        self.nz, self.ny, self.nx = nz, ny, nx
        self.nl, self.nk = ny, nx // 2 + 1
        self.a = np.asarray(a, dtype=np.float64).astype(np.complex128)
        self.kk = np.asarray(kk, dtype=np.float64)
        self.ll = np.asarray(ll, dtype=np.float64)
        # pyqg/kernel.pyx:536-556
        self._ik = 1j * self.kk
        self._il = 1j * self.ll
        self._k2l2 = self.kk[np.newaxis, :] ** 2 + self.ll[:, np.newaxis] ** 2
        self.Ubg = np.asarray(Ubg, dtype=np.float64)
        # pyqg/kernel.pyx:569-575
        self.Qy = np.asarray(Qy, dtype=np.float64)
        self._ikQy = 1j * (self.kk[np.newaxis, :] * self.Qy[:, np.newaxis])
        self.filtr = np.asarray(filtr, dtype=np.float64)
        self.rek = float(rek)
        self.dt = float(dt)
        self.t = 0.0
        self.tc = 0
        self.ablevel = 0
        shp_r = (nz, ny, nx)
        shp_c = (nz, self.nl, self.nk)
        self.q = np.zeros(shp_r)
        self.qh = np.zeros(shp_c, np.complex128)
        self.ph = np.zeros(shp_c, np.complex128)
        self.u = np.zeros(shp_r)
        self.v = np.zeros(shp_r)
        self.uq = np.zeros(shp_r)
        self.vq = np.zeros(shp_r)
        self.uh = np.zeros(shp_c, np.complex128)
        self.vh = np.zeros(shp_c, np.complex128)
        self.uqh = np.zeros(shp_c, np.complex128)
        self.vqh = np.zeros(shp_c, np.complex128)
        self.dqhdt = np.zeros(shp_c, np.complex128)
        self.dqhdt_p = np.zeros(shp_c, np.complex128)
        self.dqhdt_pp = np.zeros(shp_c, np.complex128)

    # -- state setters (pyqg/kernel.pyx:576-591) --------------------------
    def set_q(self, q):
        self.q = np.array(q, dtype=np.float64, copy=True)
        self.qh = rfft2(self.q)

    def set_qh(self, qh):
        self.qh = np.array(qh, dtype=np.complex128, copy=True)
        self.q = irfft2(self.qh)

    # -- stages -------------------------------------------------------------
    def invert(self):
        """``pyqg/kernel.pyx:315-355``: ph = sum_k1 a[k2,k1] qh[k1];
        uh = -il ph; vh = ik ph; u, v = irfft2(uh), irfft2(vh)."""
        ph = np.zeros_like(self.qh)
        for k2 in range(self.nz):
            for k1 in range(self.nz):
                ph[k2] = ph[k2] + self.a[k2, k1] * self.qh[k1]
        self.ph = ph
        self.uh = -self._il[np.newaxis, :, np.newaxis] * ph
        self.vh = self._ik[np.newaxis, np.newaxis, :] * ph
        self.u = irfft2(self.uh)
        self.v = irfft2(self.vh)

    def do_advection(self):
        """``pyqg/kernel.pyx:360-395``: uq = (u+Ubg) q, vq = v q (no Vbg),
        dqhdt = -(ik uqh + il vqh + ikQy ph) (no Qx term)."""
        self.uq = (self.u + self.Ubg[:, np.newaxis, np.newaxis]) * self.q
        self.vq = self.v * self.q
        self.uqh = rfft2(self.uq)
        self.vqh = rfft2(self.vq)
        self.dqhdt = -(self._ik[np.newaxis, np.newaxis, :] * self.uqh
                       + self._il[np.newaxis, :, np.newaxis] * self.vqh
                       + self._ikQy[:, np.newaxis, :] * self.ph)

    def do_friction(self):
        """``pyqg/kernel.pyx:447-461``: bottom layer only, only if rek."""
        if self.rek:
            self.dqhdt[-1] = self.dqhdt[-1] + (self.rek * self._k2l2 * self.ph[-1])

    def do_q_subgrid_parameterization(self, dq):
        """``pyqg/kernel.pyx:427-442``."""
        dqh = rfft2(np.asarray(dq, dtype=np.float64))
        self.dqh = dqh
        self.dqhdt = self.dqhdt + dqh

    def do_uv_subgrid_parameterization(self, du, dv):
        """``pyqg/kernel.pyx:400-422``."""
        duh = rfft2(np.asarray(du, dtype=np.float64))
        dvh = rfft2(np.asarray(dv, dtype=np.float64))
        self.duh, self.dvh = duh, dvh
        self.dqhdt = self.dqhdt + (
            -self._il[np.newaxis, :, np.newaxis] * duh
            + self._ik[np.newaxis, np.newaxis, :] * dvh)

    def ab_coefficients(self):
        """``pyqg/kernel.pyx:479-495``: FE, then AB2, then AB3."""
        dt = self.dt
        if self.ablevel == 0:
            return dt, 0.0, 0.0
        if self.ablevel == 1:
            return 1.5 * dt, -0.5 * dt, 0.0
        return 23. / 12. * dt, -16. / 12. * dt, 5. / 12. * dt

    def forward_timestep(self):
        """``pyqg/kernel.pyx:467-526``: filtered AB update, history rotation,
        q = irfft2(qh), tc += 1, t += dt."""
        dt1, dt2, dt3 = self.ab_coefficients()
        self.ablevel = min(self.ablevel + 1, 2)
        qh_new = self.filtr * (self.qh + dt1 * self.dqhdt + dt2 * self.dqhdt_p
                               + dt3 * self.dqhdt_pp)
        self.dqhdt_pp = self.dqhdt_p.copy()
        self.dqhdt_p = self.dqhdt.copy()
        self.qh = qh_new
        self.q = irfft2(qh_new)
        self.tc += 1
        self.t += self.dt

    def step(self, q_param=None, uv_param=None):
        """One step in ``Model._step_forward`` order (``pyqg/model.py:406-436``),
        with the parameterization callbacks given as callables of the oracle."""
        self.invert()
        self.do_advection()
        self.do_friction()
        if uv_param is not None:
            du, dv = uv_param(self)
            self.do_uv_subgrid_parameterization(du, dv)
        if q_param is not None:
            self.do_q_subgrid_parameterization(q_param(self))
        self.forward_timestep()


def qg_constants(nx, L=1e6, W=None, beta=1.5e-11, rd=15000.0, delta=0.25,
                 H1=500.0, U1=0.025, U2=0.0, filterfac=23.6, ny=None):
    """Two-layer QGModel constants, restated from ``pyqg/model.py:446-503``
    (grid, filter) and ``pyqg/qg_model.py:110-161`` (background, inversion).
    Returns a dict with the OracleKernel constructor arguments (minus rek/dt)."""
    ny = nx if ny is None else ny
    W = L if W is None else W
    nk = nx // 2 + 1
    dk, dl = 2 * np.pi / L, 2 * np.pi / W
    ll = dl * np.append(np.arange(0., nx / 2), np.arange(-nx / 2, 0.))
    kk = dk * np.arange(0., nk)
    k, l = np.meshgrid(kk, ll)
    wv2 = k ** 2 + l ** 2
    dx, dy = L / nx, W / ny
    F1 = rd ** -2 / (1. + delta)
    F2 = delta * F1
    Qy = np.array([beta + F1 * (U1 - U2), beta - F2 * (U1 - U2)])
    a = np.zeros((2, 2, ny, nk))
    det = wv2 * (wv2 + F1 + F2)
    nz_ = det != 0
    det_inv = np.zeros_like(det)
    det_inv[nz_] = det[nz_] ** -1
    a[0, 0] = -(wv2 + F2) * det_inv
    a[0, 1] = -F1 * det_inv
    a[1, 0] = -F2 * det_inv
    a[1, 1] = -(wv2 + F1) * det_inv
    cphi = 0.65 * np.pi
    wvx = np.sqrt((k * dx) ** 2. + (l * dy) ** 2.)
    filtr = np.exp(-filterfac * (wvx - cphi) ** 4.)
    filtr[wvx <= cphi] = 1.
    return dict(nz=2, ny=ny, nx=nx, a=a, kk=kk, ll=ll,
                Ubg=np.array([U1, U2]), Qy=Qy, filtr=filtr)
