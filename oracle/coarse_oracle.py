"""CPU oracle of the spectral coarse-graining and subgrid forcing.

TEST INFRASTRUCTURE ONLY: imported by ``tests/`` to compare against, never
by the product path.

Parity unpinned: the reference has no coarse-graining (its
``Model.subgrid_forcing`` raises, ``pyqg/model.py:397-402``).  This numpy
restatement defines the operator the CUDA path must reproduce:

* sharp spectral truncation of a fine (ny_f, nx_f) grid to a coarse
  (ny_c, nx_c) grid keeping |k| < nx_c/2 and |l| < ny_c/2, amplitudes kept
  (spectral coefficients times (nx_c ny_c) / (nx_f ny_f)), the coarse
  Nyquist row and column zero;
* J(psi, q) = u q_x + v q_y evaluated as ik fft(u q) + il fft(v q), the
  reference's ``Model._advect`` (``pyqg/model.py:539-558``) with eddy
  velocities u = irfft(-il a qh), v = irfft(ik a qh) (``pyqg/kernel.pyx:
  312-355``);
* the forcing S = filtered(J(psi, q)) - J(filtered psi, filtered q).
"""
import numpy as np

from pyqg_oracle import irfft2, rfft2


def truncate(xh, nyc, nxc):
    nz, nyf, nkf = xh.shape
    nxf = 2 * (nkf - 1)
    nkc = nxc // 2 + 1
    out = np.zeros((nz, nyc, nkc), dtype=np.complex128)
    scale = (nxc * nyc) / (nxf * nyf)
    h = nyc // 2
    out[:, :h, :nkc - 1] = xh[:, :h, :nkc - 1] * scale
    out[:, h + 1:, :nkc - 1] = xh[:, nyf - (nyc - h - 1):, :nkc - 1] * scale
    return out


def velocities(qh, a, kk, ll):
    ph = np.einsum("ijlk,jlk->ilk", a, qh)
    uh = -1j * ll[:, None] * ph
    vh = 1j * kk[None, :] * ph
    return irfft2(uh), irfft2(vh)


def advect(f, u, v, kk, ll):
    return 1j * kk[None, :] * rfft2(u * f) + 1j * ll[:, None] * rfft2(v * f)


def coarse_forcing(qh_f, fine, coarse):
    """fine / coarse: dicts with 'a' (nz, nz, nl, nk), 'kk', 'll', 'ny', 'nx'.
    Returns (q_c, S), both (nz, ny_c, nx_c)."""
    uf, vf = velocities(qh_f, fine["a"], fine["kk"], fine["ll"])
    qf = irfft2(qh_f)
    Jf = advect(qf, uf, vf, fine["kk"], fine["ll"])
    Jbar = truncate(Jf, coarse["ny"], coarse["nx"])
    qbar = truncate(qh_f, coarse["ny"], coarse["nx"])
    qc = irfft2(qbar)
    uc, vc = velocities(qbar, coarse["a"], coarse["kk"], coarse["ll"])
    Jc = advect(qc, uc, vc, coarse["kk"], coarse["ll"])
    return qc, irfft2(Jbar - Jc)
