"""The learned-closure experiment: data, training and the online comparison.

No counterpart in the reference.  Steps (``python -m
pyqg_gb300.closure_experiment --help`` lists the sizes):

1. an FP64 ensemble of two-layer nx=256 runs (seeded 1e-7 N(0, 1) initial PV)
   is spun up and sampled; every snapshot is coarse-grained to nx=64 with
   the subgrid forcing S (:mod:`pyqg_gb300.coarsen`);
2. the convolutional net (:mod:`pyqg_gb300.closure`) is trained with Adam on
   the standardised (q, S) pairs;
3. from the coarse-grained final fine states, nx=64 ensembles with and
   without the closure and the nx=256 runs advance side by side; the time
   mean kinetic-energy spectra (isotropic, layer-weighted) are compared at
   the wavenumbers the coarse grid resolves, and every ensemble's simulated
   years per wall-clock hour is measured.

The result is one JSON document (stdout, and ``--out``).
"""
import argparse
import json
import time

import numpy as np

from .coarsen import PHYSICS, QUIET, channel_stats, generate_training_data

YEAR = 360 * 86400.0


def ke_spectrum(model, q):
    """Isotropic layer-weighted KE spectrum of PV q (nz, ny, nx) on the
    grid of `model` (host FP64): (wavenumbers, spectrum)."""
    from .diagnostic_tools import calc_ispec
    qh = np.fft.rfftn(q, axes=(-2, -1))
    a = np.asarray(model.a)
    ph = np.einsum("ijlk,jlk->ilk", a, qh)
    w = (np.asarray(model.Hi) / model.H)[:, None, None]
    dens = (w * np.asarray(model.wv2)[None] * np.abs(ph) ** 2 / model.M ** 2).sum(axis=0)
    k, s = calc_ispec(model, dens, averaging=False, truncate=True)
    return np.asarray(k), np.asarray(s)


def _truncate_physical(q, nc):
    """Sharp spectral truncation of physical PV to an nc x nc grid."""
    nz, nf, _ = q.shape
    qh = np.fft.rfftn(q, axes=(-2, -1))
    h = nc // 2
    out = np.zeros((nz, nc, h + 1), dtype=complex)
    out[:, :h, :h] = qh[:, :h, :h]
    out[:, h + 1:, :h] = qh[:, nf - h + 1:, :h]
    return np.fft.irfftn(out * (nc * nc) / (nf * nf), s=(nc, nc), axes=(-2, -1))


def train(net, X, Y, epochs, batch=64, lr=1e-3, seed=0, log=None, schedule="constant"):
    """Adam on standardised tensors X, Y (N, C, ny, nx); returns the mean
    loss of every epoch.  A network without normalisation layers can
    collapse at lr 1e-3 (all ReLUs dead: the loss jumps back to the variance
    of the target); the best parameters are kept, and after an epoch whose
    loss exceeds 1.5 times the best (or reaches 0.99) they are restored and
    the learning rate is halved.  schedule "cosine" decays the rate of every
    epoch as lr (1 + cos(pi e / epochs)) / 2 (times the halvings)."""
    import math
    import torch
    g = torch.Generator(device="cpu").manual_seed(seed)
    n = X.shape[0] - X.shape[0] % batch
    hist = []
    best, best_p = float("inf"), None
    for ep in range(epochs):
        perm = torch.randperm(X.shape[0], generator=g)[:n].to(X.device)
        tot = 0.0
        lr_ep = lr * (0.5 * (1.0 + math.cos(math.pi * ep / epochs)) if schedule == "cosine" else 1.0)
        for i in range(0, n, batch):
            idx = perm[i:i + batch]
            tot += net.train_step(X[idx].contiguous(), Y[idx].contiguous(), lr=lr_ep)
        hist.append(tot / (n // batch))
        if log:
            log("epoch %d loss %.4f lr %.2e" % (ep, hist[-1], lr_ep))
        if hist[-1] < best:
            best, best_p = hist[-1], net.params
        elif best_p is not None and (hist[-1] > 1.5 * best or hist[-1] >= 0.99):
            net.params = best_p
            lr *= 0.5
            if log:
                log("  restored the best parameters (loss %.4f), lr -> %.2e" % (best, lr))
    if best_p is not None:
        net.params = best_p
    return hist


def run(nruns=32, spinup_years=4.0, sample_years=1.0, sample_every=48, epochs=30, batch=64, lr=1e-3,
        eval_years=3.0, spectra_every=240, seed0=2000, scales=(1.0, 0.5), lr_schedule="cosine", log=print):
    import torch
    import pyqg_gb300 as P
    from .closure import CNNParameterization, ConvNet
    dt_f, dt_c = 3600.0, 7200.0
    t0 = time.time()
    report = {"config": dict(nruns=nruns, spinup_years=spinup_years, sample_years=sample_years,
                             sample_every_steps=sample_every, epochs=epochs, batch=batch, lr=lr,
                             eval_years=eval_years, seed0=seed0, dt_fine=dt_f, dt_coarse=dt_c,
                             closure_scales=list(scales), lr_schedule=lr_schedule)}
    spin = int(round(spinup_years * YEAR / dt_f))
    nsnap = max(1, int(round(sample_years * YEAR / dt_f / sample_every)))
    X, Y, ens_f = generate_training_data(nruns=nruns, nx_fine=256, nx_coarse=64, dt=dt_f, spinup_steps=spin,
                                         snapshot_interval=sample_every, nsnapshots=nsnap, seed0=seed0,
                                         return_ensemble=True)
    torch.cuda.synchronize()
    report["data"] = dict(samples=int(X.shape[0]), seconds=time.time() - t0)
    log("data: %d samples in %.1f s" % (X.shape[0], time.time() - t0))
    qm, qs = channel_stats(X)
    sm, ss = channel_stats(Y)
    Xs = ((X.double() - torch.tensor(qm, device=X.device)[None, :, None, None]) /
          torch.tensor(qs, device=X.device)[None, :, None, None]).float().contiguous()
    Ys = ((Y.double() - torch.tensor(sm, device=X.device)[None, :, None, None]) /
          torch.tensor(ss, device=X.device)[None, :, None, None]).float().contiguous()
    n_val = max(batch, X.shape[0] // 10)
    net = ConvNet(max_batch=max(batch, nruns), seed=seed0)
    t1 = time.time()
    hist = train(net, Xs[n_val:], Ys[n_val:], epochs, batch=batch, lr=lr, log=log, schedule=lr_schedule)
    torch.cuda.synchronize()
    # validation: relative MSE of the standardised forcing on held-out samples
    pred = torch.empty_like(Ys[:n_val])
    net.set_norm([0.0, 0.0], [1.0, 1.0], [0.0, 0.0], [1.0, 1.0])
    for i in range(0, n_val, batch):
        j = min(n_val, i + batch)
        net.forward(Xs[i:j].contiguous(), pred[i:j])
    val = float(((pred - Ys[:n_val]) ** 2).mean() / (Ys[:n_val] ** 2).mean())
    report["training"] = dict(seconds=time.time() - t1, loss_first=hist[0], loss_last=hist[-1],
                              loss_best=min(hist), validation_relative_mse=val)
    log("training: loss %.4f -> %.4f, validation relative MSE %.3f" % (hist[0], hist[-1], val))
    CNNParameterization(net, (qm, qs, sm, ss))
    params = net.params

    # ---- online comparison from the coarse-grained final fine states -----
    # one closure ensemble per amplitude (the forcing times `scale`), each
    # with its own copy of the network
    nm = nruns
    qf = ens_f.groups[0].get_q()
    q0c = [_truncate_physical(qf[j], 64) for j in range(nm)]
    coarse_members = [("qg", dict(nx=64, dt=dt_c, **PHYSICS)) for _ in range(nm)]
    runs = [("fine", ens_f, 2)]
    closure_names = []
    nets = []
    for sc in scales:
        nt = ConvNet(max_batch=max(batch, nruns), seed=seed0)
        nt.params = params
        CNNParameterization(nt, (qm, qs, sm * sc, ss * sc))
        e = P.Ensemble(coarse_members, precision="fp32")
        e.set_q(q0c)
        e.set_closure(nt)
        name = "closure" if sc == 1.0 else "closure_x%g" % sc
        closure_names.append(name)
        nets.append(nt)
        runs.append((name, e, 1))
    ens_nc = P.Ensemble(coarse_members, precision="fp32")
    ens_nc.set_q(q0c)
    runs.append(("no_closure", ens_nc, 1))
    m_f = P.QGModel(nx=256, dt=dt_f, **PHYSICS, **QUIET)
    m_c = P.QGModel(nx=64, dt=dt_c, **PHYSICS, **QUIET)
    n_c = int(round(eval_years * YEAR / dt_c))
    chunk = spectra_every
    spec = {name: 0.0 for name, _, _ in runs}
    count = 0
    wall = {name: 0.0 for name, _, _ in runs}
    blowup = {}
    done = 0
    while done < n_c:
        c = min(chunk, n_c - done)
        for name, ens, mult in runs:
            torch.cuda.synchronize()
            ts = time.perf_counter()
            ens.step(mult * c)
            torch.cuda.synchronize()
            wall[name] += time.perf_counter() - ts
        done += c
        for name, ens, _ in runs:
            if name not in blowup:
                ke_ = ens.energy()[0]
                if not all(np.all(np.isfinite(k)) for k in ke_):
                    blowup[name] = done * dt_c / YEAR
        if done * dt_c >= 0.5 * eval_years * YEAR:      # second half: statistics
            for name, ens, _ in runs:
                model = m_f if name == "fine" else m_c
                qs_ = ens.groups[0].get_q()
                s_ = 0.0
                for j in range(nm):
                    k, sp = ke_spectrum(model, qs_[j])
                    s_ = s_ + sp
                spec[name] = spec[name] + s_ / nm
            count += 1
    kc, _ = ke_spectrum(m_c, np.zeros((2, 64, 64)))
    nres = len(kc)            # isotropic bins inside the coarse grid's circle
    sf = spec["fine"] / count
    # bands: every isotropic bin the coarse grid resolves; the bins below the
    # coarse grid's exponential filter (kappa* dx < 0.65 pi, where it is 1);
    # the energy-containing bins (fine spectrum above 10 % of its peak)
    dkr = kc[1] - kc[0]
    k_filter = 0.65 * np.pi / m_c.dx
    unfiltered = (kc[:nres] + dkr / 2) <= k_filter
    energetic = sf[:nres] >= 0.1 * sf[:nres].max()
    out = {}
    for name in closure_names + ["no_closure"]:
        sc = spec[name] / count
        n = min(nres, len(sf))
        rel = np.abs(sc[:n] - sf[:n]) / np.maximum(np.abs(sf[:n]), 1e-300)
        finite = bool(np.all(np.isfinite(sc)))
        band = {}
        for bname, mask in (("resolved", np.ones(n, bool)), ("unfiltered", unfiltered[:n]),
                            ("energy_containing", energetic[:n])):
            band[bname] = dict(max_rel_error=float(np.nanmax(rel[mask])) if finite else None,
                               mean_rel_error=float(np.nanmean(rel[mask])) if finite else None,
                               bins=int(mask.sum()))
        out[name] = dict(bands=band, total_ke_ratio=float(sc[:n].sum() / sf[:n].sum()) if finite else None,
                         finite=finite, blew_up_after_years=blowup.get(name))
    sim_years = n_c * dt_c / YEAR
    thr = {name: nm * sim_years / (wall[name] / 3600.0) for name in wall}
    report["online"] = dict(members=nm, years=sim_years, spectra_samples=count, ke_spectrum=out,
                            sim_years_per_hour=thr, k_resolved=[float(x) for x in kc[:nres]],
                            spectrum_fine=[float(x) for x in sf[:nres]],
                            spectra={name: [float(x) for x in (spec[name] / count)[:nres]]
                                     for name in closure_names + ["no_closure"]})
    report["seconds"] = time.time() - t0
    return report


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--nruns", type=int, default=32)
    ap.add_argument("--spinup-years", type=float, default=4.0)
    ap.add_argument("--sample-years", type=float, default=1.0)
    ap.add_argument("--sample-every", type=int, default=48)
    ap.add_argument("--epochs", type=int, default=30)
    ap.add_argument("--eval-years", type=float, default=3.0)
    ap.add_argument("--scales", default="1.0,0.5", help="closure amplitudes to evaluate online")
    ap.add_argument("--lr-schedule", default="cosine", choices=["constant", "cosine"])
    ap.add_argument("--out", default=None)
    a = ap.parse_args(argv)
    rep = run(nruns=a.nruns, spinup_years=a.spinup_years, sample_years=a.sample_years,
              sample_every=a.sample_every, epochs=a.epochs, eval_years=a.eval_years,
              scales=tuple(float(x) for x in a.scales.split(",")), lr_schedule=a.lr_schedule)
    txt = json.dumps(rep)
    print(txt)
    if a.out:
        with open(a.out, "w") as f:
            f.write(txt + "\n")


if __name__ == "__main__":
    main()
