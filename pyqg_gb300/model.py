"""Generic pseudo-spectral model on the GB300 kernel.

Same constructor, loop and diagnostics API as ``pyqg.Model``
(``pyqg/model.py:22-862``); the time step runs in the CUDA library through
:class:`~pyqg_gb300.kernel.PseudoSpectralKernel`.

``_step_forward`` keeps the reference's stage order (``pyqg/model.py:406-436``).
When nothing observes the intermediate state of a step (no parameterization
hook, no diagnostics due, no subclass overriding a stage), the step runs as
the fused two-kernel step instead, and ``run`` / ``run_with_snapshots`` hand
whole stretches of such steps to the CUDA library at once.  Both paths give
bit-identical states.
"""
import logging
import warnings

import numpy as np

from .errors import DiagnosticNotFilledError
from .kernel import PseudoSpectralKernel

__all__ = ["Model"]

_MAX_BATCH = 4096


class _DiagEntry(dict):
    """A diagnostics entry.  Built-in diagnostics accumulate on the device
    (key '_acc'); reading 'value' returns the host copy of the sum, as the
    reference's entries hold it."""

    def __getitem__(self, key):
        if key == 'value' and '_acc' in self:
            acc = dict.__getitem__(self, '_acc').cpu().numpy()
            return acc[()] if acc.ndim == 0 else acc
        return dict.__getitem__(self, key)

    def __contains__(self, key):
        if key == 'value' and dict.__contains__(self, '_acc'):
            return True
        return dict.__contains__(self, key)

    def get(self, key, default=None):
        return self[key] if key in self else default


def grid_constants(nx, ny, L, W):
    """Spatial and spectral grids (``pyqg/model.py:446-482``).

    Note ``ll`` is built from ``nx`` as in the reference (square grids)."""
    g = {}
    g["x"], g["y"] = np.meshgrid(np.arange(0.5, nx, 1.) / nx * L,
                                 np.arange(0.5, ny, 1.) / ny * W)
    g["dk"] = 2. * np.pi / L
    g["dl"] = 2. * np.pi / W
    nk = int(nx / 2 + 1)
    g["ll"] = g["dl"] * np.append(np.arange(0., nx / 2), np.arange(-nx / 2, 0.))
    g["kk"] = g["dk"] * np.arange(0., nk)
    g["k"], g["l"] = np.meshgrid(g["kk"], g["ll"])
    g["ik"] = 1j * g["k"]
    g["il"] = 1j * g["l"]
    g["dx"] = L / nx
    g["dy"] = W / ny
    g["M"] = nx * ny
    g["wv2"] = g["k"] ** 2 + g["l"] ** 2
    g["wv"] = np.sqrt(g["wv2"])
    nonzero = g["wv2"] != 0.
    g["wv2i"] = np.zeros_like(g["wv2"])
    g["wv2i"][nonzero] = g["wv2"][nonzero] ** -1
    return g


def spectral_filter(k, l, dx, dy, filterfac):
    """Exponential filter of Arbic & Flierl (2003) (``pyqg/model.py:496-503``):
    1 below the cutoff 0.65 pi (grid units), exp(-filterfac (k* - c)^4) above."""
    cphi = 0.65 * np.pi
    wvx = np.sqrt((k * dx) ** 2. + (l * dy) ** 2.)
    filtr = np.exp(-filterfac * (wvx - cphi) ** 4.)
    filtr[wvx <= cphi] = 1.
    return filtr


class Model(PseudoSpectralKernel):
    """A generic pseudo-spectral inversion model (see ``pyqg.Model``).

    Subclasses provide ``_initialize_background``,
    ``_initialize_inversion_matrix``, ``_initialize_forcing``, ``_calc_cfl``
    and ``_calc_ke``.
    """

    def __init__(self, nz=1, nx=64, ny=None, L=1e6, W=None, dt=7200.,
                 twrite=1000., tmax=1576800000., tavestart=315360000.,
                 taveint=86400., useAB2=False, rek=5.787e-7, filterfac=23.6,
                 f=None, g=9.81, q_parameterization=None,
                 uv_parameterization=None, parameterization=None,
                 diagnostics_list='all', ntd=1, log_level=1, logfile=None):
        ny = nx if ny is None else ny
        W = L if W is None else W
        if ny != nx:
            # the reference builds the meridional wavenumbers from nx
            # (pyqg/model.py:459-460), so its models have wrong wavenumbers
            # (or index past them) when ny != nx; refuse instead.  The kernel
            # (PseudoSpectralKernel) itself takes any (ny, nx).
            raise ValueError("ny != nx is not supported by the model classes (the reference's "
                             "wavenumber grid assumes ny == nx); got nx=%d, ny=%d" % (nx, ny))

        # infer the hook of an explicit parameterization object
        # (pyqg/model.py:203-212)
        if parameterization is not None:
            kind = getattr(parameterization, "parameterization_type", None)
            if kind == "uv_parameterization":
                assert uv_parameterization is None
                uv_parameterization = parameterization
            elif kind == "q_parameterization":
                assert q_parameterization is None
                q_parameterization = parameterization
            else:
                raise ValueError(f"unknown parameterization type {kind}")

        PseudoSpectralKernel.__init__(
            self, nz, ny, nx, ntd,
            has_q_param=int(q_parameterization is not None),
            has_uv_param=int(uv_parameterization is not None))

        self.L, self.W = L, W
        self.dt = dt
        self.twrite = twrite
        self.tmax = tmax
        self.tavestart = tavestart
        self.taveint = taveint
        self.logfile = logfile
        self.log_level = log_level
        self.useAB2 = useAB2   # stored, unused by the step (as the reference)
        self.ntd = ntd
        self.rek = rek
        self.filterfac = filterfac
        self.g = g
        if f:
            self.f = f
            self.f2 = f ** 2
        self.q_parameterization = q_parameterization
        self.uv_parameterization = uv_parameterization

        self._initialize_logger()
        self._initialize_grid()
        self._initialize_background()
        self._initialize_forcing()
        self._initialize_filter()
        self._initialize_time()
        self._initialize_inversion_matrix()
        self._initialize_diagnostics(diagnostics_list)

    # ------------------------------------------------------------------
    # time loop
    # ------------------------------------------------------------------
    def run_with_snapshots(self, tsnapstart=0., tsnapint=432000.):
        """Run the model, yielding the time every `tsnapint` seconds of model
        time once ``t >= tsnapstart``."""
        tsnapints = np.ceil(tsnapint / self.dt)
        while self.t < self.tmax:
            stop = lambda t, tc: t >= tsnapstart and (tc % tsnapints) == 0
            self._advance(stop)
            if self.t >= tsnapstart and (self.tc % tsnapints) == 0:
                yield self.t

    def run(self):
        """Run the model until ``t >= tmax``."""
        while self.t < self.tmax:
            self._advance(lambda t, tc: False)

    def _advance(self, stop_after):
        """One step, or a batch of fusable steps ending before the next
        observation point (diagnostics, status output, `stop_after`)."""
        n = self._fusable_run_length(stop_after)
        if n <= 1:
            self._step_forward()
        else:
            self._step_fused(n)
            self._print_status()

    def _fusable(self):
        """True when no code outside this library observes the inside of a
        step: no hooks, and no stage overridden by a user subclass."""
        if self.q_parameterization is not None or self.uv_parameterization is not None:
            return False
        cls = type(self)
        for name in ("_invert", "_do_advection", "_do_friction",
                     "_forward_timestep", "_do_external_forcing",
                     "_step_forward", "_calc_diagnostics"):
            impl = getattr(cls, name)
            if getattr(impl, "__module__", "").split(".")[0] != "pyqg_gb300":
                return False
        return True

    def _diagnostics_due(self, t, tc):
        """Whether ``_calc_diagnostics`` fires at the start of a step at
        (t, tc) (``pyqg/model.py:577-580``)."""
        return (t >= self.dt) and (t >= self.tavestart) and (tc % self.taveints == 0)

    def _status_due(self, tc):
        return bool(self.log_level) and (tc % self.twrite) == 0

    def _fusable_run_length(self, stop_after=lambda t, tc: False):
        if not self._fusable():
            return 0
        t, tc, dt = self.t, self.tc, self.dt
        n = 0
        while t < self.tmax and n < _MAX_BATCH:
            if self._diagnostics_due(t, tc):
                break
            t = t + dt
            tc = tc + 1
            n += 1
            if self._status_due(tc) or stop_after(t, tc):
                break
        return n

    def _step_forward(self):
        if (self._fusable() and not self._diagnostics_due(self.t, self.tc)):
            self._step_fused(1)
            self._print_status()
            return
        # stage-by-stage path (pyqg/model.py:406-436)
        self._invert()
        self._do_advection()
        self._do_friction()
        self._do_external_forcing()
        if self.uv_parameterization is not None:
            self._do_uv_subgrid_parameterization()
        if self.q_parameterization is not None:
            self._do_q_subgrid_parameterization()
        self._calc_diagnostics()
        self._forward_timestep()
        self._print_status()

    # ------------------------------------------------------------------
    # initialization
    # ------------------------------------------------------------------
    def _initialize_time(self):
        self.taveints = np.ceil(self.taveint / self.dt)

    def _initialize_grid(self):
        g = grid_constants(self.nx, self.ny, self.L, self.W)
        self.x, self.y = g["x"], g["y"]
        self.dk, self.dl = g["dk"], g["dl"]
        self.ll = g["ll"]
        self.kk = g["kk"]
        self.k, self.l = g["k"], g["l"]
        self.ik, self.il = g["ik"], g["il"]
        self.dx, self.dy = g["dx"], g["dy"]
        self.M = g["M"]
        self.wv2, self.wv, self.wv2i = g["wv2"], g["wv"], g["wv2i"]

    def _initialize_background(self):
        raise NotImplementedError('needs to be implemented by Model subclass')

    def _initialize_inversion_matrix(self):
        raise NotImplementedError('needs to be implemented by Model subclass')

    def _initialize_forcing(self):
        raise NotImplementedError('needs to be implemented by Model subclass')

    def _initialize_filter(self):
        self.filtr = spectral_filter(self.k, self.l, self.dx, self.dy, self.filterfac)

    def _filter(self, q):
        return self.filtr * q

    def _do_external_forcing(self):
        pass

    def _initialize_logger(self):
        self.logger = logging.getLogger(__name__)
        if self.logfile is not None:
            handler = logging.FileHandler(filename=self.logfile, mode='w')
        else:
            handler = logging.StreamHandler()
        handler.setFormatter(logging.Formatter('%(levelname)s: %(message)s'))
        if not self.logger.handlers:
            self.logger.addHandler(handler)
        self.logger.setLevel(self.log_level * 10)
        self.logger.propagate = False
        self.logger.info(' Logger initialized')

    # ------------------------------------------------------------------
    # helpers used by diagnostics and parameterizations
    # ------------------------------------------------------------------
    def _advect(self, q, u=None, v=None):
        """Spectral advective tendency ik (uq)^ + il (vq)^ of real q
        (``pyqg/model.py:539-558``); 2-D inputs give a 2-D result.  The
        products, transforms and derivatives run on the GPU; numpy inputs
        give a numpy result, CUDA tensors a CUDA tensor."""
        import torch
        on_device = any(isinstance(x, torch.Tensor) for x in (q, u, v))
        if u is None:
            u = self.device_field("u") if on_device else self.u
        if v is None:
            v = self.device_field("v") if on_device else self.v
        arrs = [x if isinstance(x, torch.Tensor) else torch.from_numpy(np.asarray(x, dtype=np.float64))
                for x in (q, u, v)]
        shape = torch.broadcast_shapes(*(a.shape for a in arrs))
        flat = len(shape) == 2
        with torch.cuda.stream(self._stream):
            arrs = [a.to(self._device, torch.float64).broadcast_to(shape).reshape(-1, self.ny, self.nx)
                    for a in arrs]
            tend = self._device_advect(*arrs)
            if flat:
                tend = tend[0]
            return tend if on_device else tend.cpu().numpy()

    def _print_status(self):
        """Log KE and CFL every `twrite` steps; fail if CFL >= 1.  A state
        the step kernels flagged as non-finite gives CFL = NaN, so the
        assertion fails as the reference's does for a NaN velocity, without
        downloading the velocity fields."""
        if self.log_level and (self.tc % self.twrite) == 0:
            self._stream.synchronize()
            nonfinite = self.nonfinite
            self.ke = self._calc_ke()
            self.cfl = float("nan") if nonfinite else self._calc_cfl()
            self.logger.info('Step: %i, Time: %3.2e, KE: %3.2e, CFL: %4.3f',
                             self.tc, self.t, self.ke, self.cfl)
            assert self.cfl < 1., self.logger.error('CFL condition violated')

    def _calc_diagnostics(self):
        if self._diagnostics_due(self.t, self.tc):
            self._increment_diagnostics()

    def _calc_cfl(self):
        raise NotImplementedError('needs to be implemented by Model subclass')

    def _calc_ke(self):
        raise NotImplementedError('needs to be implemented by Model subclass')

    def spec_var(self, ph):
        """Variance of p from its half-plane Fourier coefficients."""
        var_dens = 2. * np.abs(ph) ** 2 / self.M ** 2
        var_dens[..., 0] = var_dens[..., 0] / 2.
        var_dens[..., -1] = var_dens[..., -1] / 2.
        return var_dens.sum()

    # ------------------------------------------------------------------
    # vertical structure (used by LayeredModel)
    # ------------------------------------------------------------------
    def vertical_modes(self):
        """Eigen-decomposition of the stretching matrix (baroclinic modes)."""
        evals, evecs = np.linalg.eig(-self.S)
        order = evals.argsort()
        self.kdi2 = evals[order]
        self.radii = np.zeros_like(self.kdi2)
        self.radii[0] = np.sqrt(self.g * self.H) / np.abs(self.f)
        self.radii[1:] = 1. / np.sqrt(self.kdi2[1:])
        self.pmodes = evecs[:, order]
        norm = (self.H / (self.Hi[:, np.newaxis] * (self.pmodes ** 2)).sum(axis=0)) ** 0.5
        self.pmodes = norm[np.newaxis, :] * self.pmodes

    def modal_projection(self, p, forward=True):
        """Project layer field p onto the vertical modes (or back)."""
        if forward:
            flat = p.reshape(p.shape[0], -1)
            return np.linalg.solve(self.pmodes, flat).reshape(p.shape)
        return np.einsum("ik,k...->i...", self.pmodes, p)

    def subgrid_forcing(self, **kwargs):
        raise ValueError(
            "This method was found to be buggy and removed for now. "
            "It will be re-added in a future release. "
            "See https://github.com/pyqg/pyqg/pull/308 for details. ")

    # ------------------------------------------------------------------
    # diagnostics registry (pyqg/model.py:630-820)
    # ------------------------------------------------------------------
    #: built-in diagnostics accumulate on the GPU (False: host functions)
    gpu_diagnostics = True

    def _initialize_diagnostics(self, diagnostics_list):
        self.diagnostics = dict()
        self._initialize_core_diagnostics()
        self._initialize_model_diagnostics()
        if diagnostics_list == 'all':
            pass
        elif diagnostics_list == 'none':
            self.set_active_diagnostics([])
        else:
            self.set_active_diagnostics(diagnostics_list)

    def set_active_diagnostics(self, diagnostics_list):
        for name, d in self.diagnostics.items():
            d['active'] = name in diagnostics_list

    _set_active_diagnostics = set_active_diagnostics

    def _ab_coefficients(self):
        dt = self.dt
        if self.ablevel == 0:
            return dt, 0.0, 0.0
        if self.ablevel == 1:
            return 1.5 * dt, -0.5 * dt, 0.0
        return 23. / 12. * dt, -16. / 12. * dt, 5. / 12. * dt

    def _filter_dissipation(self):
        """Change of qh the filter will make in the coming step."""
        dt1, dt2, dt3 = self._ab_coefficients()
        qh, dq, dqp, dqpp = self.qh, self.dqhdt, self.dqhdt_p, self.dqhdt_pp
        out = np.zeros_like(qh)
        for z in range(self.nz):
            out[z] = (self.filtr - 1.) * (qh[z] + dt1 * dq[z] + dt2 * dqp[z] + dt3 * dqpp[z])
        return out

    def _initialize_core_diagnostics(self):
        M2 = lambda m: m.M ** 2
        add = self.add_diagnostic
        add('Ensspec', gpu=True, description='enstrophy spectrum',
            function=lambda m: np.abs(m.qh) ** 2 / M2(m),
            units='s^-2', dims=('lev', 'l', 'k'))
        add('KEspec', gpu=True, description='kinetic energy spectrum',
            function=lambda m: m.wv2 * np.abs(m.ph) ** 2 / M2(m),
            units='m^2 s^-2', dims=('lev', 'l', 'k'))
        add('EKEdiss', gpu=True, description='total energy dissipation by bottom drag',
            function=lambda m: m.Hi[-1] / m.H * m.rek * (m.v[-1] ** 2 + m.u[-1] ** 2).mean(),
            units='m^2 s^-3', dims=('time',))
        add('KEfrictionspec', gpu=True, description='total energy dissipation spectrum by bottom drag',
            function=lambda m: -m.rek * m.Hi[-1] / m.H * m.wv2 * np.abs(m.ph[-1]) ** 2 / M2(m),
            units='m^2 s^-3', dims=('l', 'k'))
        add('EKE', gpu=True, description='mean eddy kinetic energy',
            function=lambda m: 0.5 * (m.v ** 2 + m.u ** 2).mean(axis=-1).mean(axis=-1),
            units='m^2 s^-2', dims=('lev',))
        add('Dissspec', gpu=True, description='Spectral contribution of filter dissipation to total energy',
            function=lambda m: -np.tensordot(m.Hi, np.conj(m.ph) * m._filter_dissipation(),
                                             axes=(0, 0)).real / m.H / m.dt / M2(m),
            units='m^2 s^-3', dims=('l', 'k'))
        add('ENSDissspec', gpu=True, description='Spectral contribution of filter dissipation to barotropic enstrophy',
            function=lambda m: np.tensordot(m.Hi, np.conj(m.qh) * m._filter_dissipation(),
                                            axes=(0, 0)).real / m.H / m.dt / M2(m),
            units='s^-3', dims=('l', 'k'))
        add('paramspec', gpu=True, description='Spectral contribution of subgrid parameterization to energy (if present)',
            function=lambda m: m._calc_parameterization_spectrum(),
            units='m^2 s^-3', dims=('l', 'k'), skip_comparison=True)
        add('ENSparamspec', gpu=True, description='Spectral contribution of subgrid parameterization to enstrophy',
            function=lambda m: m._calc_parameterization_enstrophy_spectrum(),
            units='s^-3', dims=('l', 'k'), skip_comparison=True)

    def _calc_parameterization_contribution(self):
        """Spectral dq/dt added by the hooks in the current step."""
        dqh = np.zeros_like(self.qh)
        if self.uv_parameterization is not None:
            ik = np.broadcast_to(np.asarray(self._ik)[np.newaxis, :], self.wv2.shape)
            il = np.broadcast_to(np.asarray(self._il)[:, np.newaxis], self.wv2.shape)
            dqh += -il * self.duh + ik * self.dvh
        if self.q_parameterization is not None:
            dqh += self.dqh
        return dqh

    def _height_ratios(self):
        return (self.Hi / self.H)[:, np.newaxis, np.newaxis]

    def _calc_parameterization_spectrum(self):
        dqh = self._calc_parameterization_contribution()
        return -np.real((self._height_ratios() * np.conj(self.ph) * dqh).sum(axis=0)) / self.M ** 2

    def _calc_parameterization_enstrophy_spectrum(self):
        dqh = self._calc_parameterization_contribution()
        return np.real((self._height_ratios() * np.conj(self.qh) * dqh).sum(axis=0)) / self.M ** 2

    def _calc_derived_fields(self):
        pass

    def _initialize_model_diagnostics(self):
        pass

    def add_diagnostic(self, diag_name, description=None, function=None,
                       units=None, dims=None, **kw):
        assert hasattr(function, '__call__')
        assert isinstance(diag_name, str)
        entry = _DiagEntry(description=description, units=units, dims=dims,
                           active=True, count=0, function=function)
        entry.update(**kw)
        self.diagnostics[diag_name] = entry

    def describe_diagnostics(self):
        print('NAME               | DESCRIPTION')
        print(80 * '-')
        for name in sorted(self.diagnostics):
            print('{:<10} | {:<54}'.format(name, self.diagnostics[name]['description']))

    def _increment_diagnostics(self):
        """Accumulate the active diagnostics.  Built-in diagnostics (those
        registered with a device kind) accumulate in FP64 on the GPU
        (``pqg_diag_accumulate``); the others run their host function."""
        device = [(n, d) for n, d in self.diagnostics.items()
                  if d['active'] and d.get('gpu') is not None and self.gpu_diagnostics]
        host = [(n, d) for n, d in self.diagnostics.items()
                if d['active'] and not (d.get('gpu') is not None and self.gpu_diagnostics)]
        if device:
            self._accumulate_device_diagnostics(device)
        if host:
            self._calc_derived_fields()
            for name, d in host:
                value = d['function'](self)
                if d['count'] == 0:
                    d['value'] = value
                else:
                    d['value'] += value
                d['count'] += 1

    # device kinds of the built-in diagnostics (enum order of the C ABI)
    _DIAG_KIND = {name: i for i, name in enumerate((
        'Ensspec', 'KEspec', 'EKE', 'EKEdiss', 'KEfrictionspec', 'Dissspec', 'ENSDissspec',
        'paramspec', 'ENSparamspec', 'entspec', 'paramspec_APEflux', 'paramspec_KEflux',
        'ENSflux', 'ENSgenspec', 'ENSfrictionspec', 'APEgenspec', 'APEflux', 'KEflux', 'APEgen',
        'KEspec_modal', 'PEspec_modal', 'APEspec', 'KEflux_div', 'APEflux_div'))}
    _DIAG_NEEDS = {'ENSflux': ('Jq',), 'KEflux': ('Jpxi',), 'KEflux_div': ('Jpxi',),
                   'APEflux': ('Jptpc',), 'APEflux_div': ('JSp',), 'ENSgenspec': ('Sph',),
                   'APEgenspec': ('Sph',), 'KEspec_modal': ('phn',), 'PEspec_modal': ('phn',)}

    def _diag_shape(self, name):
        nz, nl, nk = self.nz, self.nl, self.nk
        if name in ('Ensspec', 'KEspec', 'KEspec_modal'):
            return (nz, nl, nk)
        if name == 'PEspec_modal':
            return (nz - 1, nl, nk)
        if name == 'EKE':
            return (nz,)
        if name in ('EKEdiss', 'APEgen'):
            return ()
        return (nl, nk)

    def _device_derived(self, needs):
        """Derived fields of the diagnostics, on the device (the device
        counterpart of ``_calc_derived_fields``); layer combinations and
        spectral scalings by ``pqg_layer_mix`` and ``pqg_lap_power``."""
        import ctypes
        import torch
        from . import _lib
        from .parameterizations import _dev
        L = _lib.lib()

        def ptr(t):
            return ctypes.c_void_p(t.data_ptr())

        def mix(mat, x):
            """sum_j mat[i][j] x[j] for (n, ...) device x (the real part of a
            complex-typed layer matrix, whose values are real)."""
            mat = np.asarray(mat)
            if np.iscomplexobj(mat):
                mat = mat.real
            mat = np.ascontiguousarray(np.atleast_2d(mat.astype(np.float64)))
            x = x.contiguous()
            plane = x[0].numel() * (2 if x.is_complex() else 1)
            out = torch.empty((mat.shape[0],) + tuple(x.shape[1:]), dtype=x.dtype, device=self._device)
            _lib.check(L.pqg_layer_mix(mat.shape[0], mat.shape[1], plane, mat.ctypes.data, ptr(x), ptr(out),
                                       self._sp()))
            return out

        f = {}
        ph = self.device_field("ph")
        u, v = self.device_field("u"), self.device_field("v")
        with torch.cuda.stream(self._stream):
            if 'Jq' in needs:
                f['Jq'] = self._device_advect(self.device_field("q"), u, v)
            if 'Jpxi' in needs:
                # xi = ifft(-wv2 ph)
                neg_wv2_ph = torch.empty_like(ph)
                _lib.check(L.pqg_lap_power(ph.shape[0], self.nl, self.nk, ptr(_dev(self, "kk")),
                                           ptr(_dev(self, "ll")), 1, -1.0, ptr(ph), ptr(neg_wv2_ph), self._sp()))
                f['Jpxi'] = self._device_advect(self._device_irfft2(neg_wv2_ph), u, v)
            if 'Jptpc' in needs:
                p = self._device_irfft2(ph)
                w = [[self.del1, self.del2]]
                f['Jptpc'] = mix([[-1.0]], self._device_advect(mix([[1.0, -1.0]], p), mix(w, u), mix(w, v)))[0]
            if 'Sph' in needs or 'JSp' in needs:
                f['Sph'] = mix(self.S, ph)
                if 'JSp' in needs:
                    f['JSp'] = self._device_advect(self._device_irfft2(f['Sph']), u, v)
            if 'phn' in needs:
                f['phn'] = mix(np.linalg.inv(self.pmodes), ph)
        return f

    def _accumulate_device_diagnostics(self, items):
        import ctypes
        import torch
        from . import _lib
        needs = set()
        for name, _ in items:
            needs.update(self._DIAG_NEEDS.get(name, ()))
        derived = self._device_derived(needs)
        keep = []

        def ptr(t):
            if t is None:
                return None
            keep.append(t)
            return ctypes.cast(t.data_ptr(), ctypes.POINTER(ctypes.c_double))

        def harr(x, n):
            if x is None:
                return None
            x = np.asarray(x)
            if np.iscomplexobj(x):
                # eigenvalue-derived constants (kdi2 of the layered model)
                # are real numbers held in a complex array
                x = x.real
            a = np.ascontiguousarray(np.broadcast_to(np.asarray(x, dtype=np.float64).ravel(), (n,)))
            keep.append(a)
            return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))

        nz = self.nz
        dt1, dt2, dt3 = self._ab_coefficients()
        fl = _lib.DiagFields()
        fl.qh = ptr(self.device_field("qh"))
        fl.ph = ptr(self.device_field("ph"))
        fl.dqhdt = ptr(self.device_field("dqhdt"))
        fl.dqhdt_p = ptr(self.device_field("dqhdt_p"))
        fl.dqhdt_pp = ptr(self.device_field("dqhdt_pp"))
        fl.u = ptr(self.device_field("u"))
        fl.v = ptr(self.device_field("v"))
        for key in ('Jq', 'Jpxi', 'Jptpc', 'JSp', 'Sph', 'phn'):
            setattr(fl, key, ptr(derived.get(key)))
        if self.q_parameterization is not None:
            fl.dqh = ptr(self.device_field("dqh"))
        if self.uv_parameterization is not None:
            fl.duh = ptr(self.device_field("duh"))
            fl.dvh = ptr(self.device_field("dvh"))
        fl.H = float(getattr(self, 'H', 1.0))
        fl.dt, fl.c1, fl.c2, fl.c3 = float(self.dt), float(dt1), float(dt2), float(dt3)
        for key in ('rd', 'del1', 'del2', 'U'):
            val = getattr(self, key, None)
            setattr(fl, key, float(val) if np.isscalar(val) and val is not None else 0.0)
        fl.Hi = harr(getattr(self, 'Hi', np.ones(nz)), nz)
        fl.Qx = harr(getattr(self, 'Qx', 0.0) if np.ndim(getattr(self, 'Qx', 0.0)) <= 1 else 0.0, nz)
        fl.Qy = harr(self.Qy, nz)
        fl.Ubg = harr(self.Ubg, nz)
        fl.Vbg = harr(getattr(self, 'Vbg', 0.0), nz)
        if hasattr(self, 'f2gpi'):
            fl.f2gpi = harr(np.ravel(self.f2gpi), max(1, np.size(self.f2gpi)))
        if hasattr(self, 'kdi2'):
            fl.kdi2 = harr(self.kdi2, nz)
        if hasattr(type(self), 'S') or hasattr(self, 'S'):
            try:
                fl.S = harr(np.asarray(self.S, dtype=np.float64), nz * nz)
            except Exception:
                fl.S = None
        L = self._L
        for name, d in items:
            acc = d.get('_acc')
            if acc is None:
                acc = torch.zeros(self._diag_shape(name), dtype=torch.float64, device=self._device)
                dict.__setitem__(d, '_acc', acc)
            _lib.check(L.pqg_diag_accumulate(self._plan, self._DIAG_KIND[name], ctypes.byref(fl),
                                             acc.data_ptr(), self._sp()))
            d['count'] += 1
        if keep:
            torch.cuda.current_stream().wait_stream(self._stream)

    def get_diagnostic(self, dname):
        d = self.diagnostics[dname]
        if 'value' not in d:
            raise DiagnosticNotFilledError(dname)
        return d['value'] / d['count']

    def set_qh(self, qh):
        warnings.warn("Method deprecated. Set model.qh directly instead. ",
                      DeprecationWarning)
        self.qh = qh

    def set_q(self, q):
        warnings.warn("Method deprecated. Set model.q directly instead. ",
                      DeprecationWarning)
        self.q = q

    def to_dataset(self):
        """Convert the model state to an xarray Dataset (needs xarray)."""
        from .xarray_output import model_to_dataset
        return model_to_dataset(self)

    @property
    def parameterization(self):
        if self.q_parameterization and self.uv_parameterization:
            warnings.warn("Model has multiple parameterizations, "
                          "but only returning PV")
        return self.q_parameterization or self.uv_parameterization
