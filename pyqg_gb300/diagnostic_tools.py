"""Spectral post-processing utilities (same API as ``pyqg/diagnostic_tools.py``)."""
import numpy as np

__all__ = ["spec_var", "spec_sum", "calc_ispec", "diagnostic_differences",
           "diagnostic_similarities"]


def _half_plane_weights(x):
    """Weight 2 for interior k columns of a half-plane spectrum, 1 for the
    k = 0 and Nyquist columns (whose conjugates are not stored)."""
    w = 2. * x
    w[..., 0] = w[..., 0] / 2.
    w[..., -1] = w[..., -1] / 2.
    return w


def spec_var(model, ph):
    """Variance of p from its Fourier coefficients ``ph``."""
    return _half_plane_weights(np.abs(ph) ** 2 / model.M ** 2).sum(axis=(-1, -2))


def spec_sum(ph2):
    """Full-plane sum of a real half-plane spectral quantity ``ph2``."""
    return _half_plane_weights(ph2).sum(axis=(-1, -2))


def calc_ispec(model, _var_dens, averaging=True, truncate=True,
               nd_wavenumber=False, nfactor=1):
    """Isotropic spectrum of a 2-D (half-plane) spectral density.

    Bins of width ``nfactor * sqrt(dk^2 + dl^2)`` from 0 to the inner circle
    (``truncate``) or the corner of the spectral domain; with ``averaging``
    each bin is the ring mean times the ring circumference, otherwise the
    ring sum divided by the bin width.  Returns bin centres and spectrum.
    """
    var_dens = np.copy(_var_dens)
    var_dens[..., 0] /= 2
    var_dens[..., -1] /= 2
    ll_max = np.abs(model.ll).max()
    kk_max = np.abs(model.kk).max()
    kmax = np.minimum(ll_max, kk_max) if truncate else np.sqrt(ll_max ** 2 + kk_max ** 2)
    kmin = 0
    dkr = np.sqrt(model.dk ** 2 + model.dl ** 2) * nfactor
    kr = np.arange(kmin, kmax, dkr)
    phr = np.zeros(kr.size)
    for i in range(kr.size):
        if i == kr.size - 1:
            ring = (model.wv >= kr[i]) & (model.wv <= kr[i] + dkr)
        else:
            ring = (model.wv >= kr[i]) & (model.wv < kr[i + 1])
        if averaging:
            phr[i] = var_dens[ring].mean() * (kr[i] + dkr / 2) * np.pi / (model.dk * model.dl)
        else:
            phr[i] = var_dens[ring].sum() / dkr
        phr[i] *= 2
    kr = kr + dkr / 2
    if nd_wavenumber:
        kr = kr / kmin
        phr = phr * kmin
    return kr, phr


def diagnostic_differences(m1, m2, reduction='rmse', instantaneous=False):
    """Distances between the diagnostics of two models (possibly of different
    resolution); spectral diagnostics are compared as isotropic spectra over
    the common wavenumbers, multi-layer ones per layer."""
    kr1, _ = calc_ispec(m1, m1.diagnostics['KEspec']['function'](m1)[0])
    kr2, _ = calc_ispec(m2, m2.diagnostics['KEspec']['function'](m2)[0])
    nkr = min(len(kr1), len(kr2))

    def normalized(model, name, layer=None):
        attrs = model.diagnostics[name]
        diag = attrs['function'](model) if instantaneous else model.get_diagnostic(name)
        for other in attrs.get('sums_with', []):
            diag = diag + (model.diagnostics[other]['function'](model)
                           if instantaneous else model.get_diagnostic(other))
        if layer is not None:
            diag = diag[layer]
        if attrs['dims'][-2:] == ('l', 'k'):
            _, diag = calc_ispec(model, diag)
            diag = diag[:nkr]
        return diag

    diffs = {}
    for name, attrs in m1.diagnostics.items():
        if attrs.get('skip_comparison', False) or name not in m2.diagnostics:
            continue
        if attrs['dims'][0] == 'lev':
            layers = range(m1.nz)
        elif attrs['dims'][0] == 'lev_mid':
            layers = range(m1.nz - 1)
        else:
            layers = [None]
        for layer in layers:
            d1 = normalized(m1, name, layer)
            d2 = normalized(m2, name, layer)
            label = f"{name}{'' if layer is None else layer + 1}"
            if reduction == 'rmse':
                diffs[label] = np.sqrt(np.mean((d1 - d2) ** 2))
            else:
                diffs[label] = reduction(d1, d2)
    return diffs


def diagnostic_similarities(model, target, baseline, **kw):
    """1 - d(model, target) / d(baseline, target) per diagnostic."""
    d1 = diagnostic_differences(model, target, **kw)
    d2 = diagnostic_differences(baseline, target, **kw)
    return dict((k, 1 - d1[k] / d2[k]) for k in d1.keys())
