"""Benchmark of the FP64 pseudo-spectral step (two-layer QG, nx=ny=256,
dt=3600 s) in simulated years per wall-clock hour.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

One timed step = one call of the fused step over `--chunk` model steps
(default 100) with the state resident in HBM; L2 is flushed (a 256 MB
write) before every timed step.  Prints one JSON line on rank 0.

--impl reference times the reference's own CPU kernel (pyqg/kernel.pyx,
compiled by oracle/build_ref.py) on the host cores, falling back to the
numpy oracle port when that module cannot be built.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

YEAR = 360 * 86400.0          # pyqg/tests/test_reference_solns.py:12
METRIC = "sim-yr/hr, 1 GB300: nx64+learned closure vs nx256 plain at matched KE error"
TWO_LAYER = dict(L=1e6, beta=1.5e-11, rd=15000.0, delta=0.25, H1=500, U1=0.025,
          U2=0.0, rek=5.787e-7, filterfac=23.6)
QUIET = dict(tavestart=1e30, taveint=1e30, log_level=0)


def sim_yr_per_hr(model_steps, dt, seconds):
    return (model_steps * dt / YEAR) / (seconds / 3600.0)


def replica_value(local_s, model_steps, dt, world, device=None):
    """Replicas only: every rank advances its own model; the job's time is
    the slowest rank's (MAX over ranks) and the value sums the ranks'
    simulated years.  Returns (value, job seconds)."""
    total_s = local_s
    if world > 1:
        import torch
        t = torch.tensor([local_s], dtype=torch.float64, device=device)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        total_s = float(t.item())
    return world * sim_yr_per_hr(model_steps, dt, total_s), total_s


def peaks():
    try:
        with open(os.path.join(HERE, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


# --------------------------------------------------------------------------
# clocks sampled during the timed region
# --------------------------------------------------------------------------
class ClockSampler:
    """Streams `nvidia-smi -lms 50` for one GPU; summary() keeps the samples
    taken between mark_start() and mark_stop()."""
    FIELDS = ("clocks.sm,clocks.max.sm,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")
    NAMES = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]

    def __init__(self, index):
        self.index = index
        self.samples = []
        self.t0 = self.t1 = None
        self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            parts = [x.strip() for x in line.strip().split(",")]
            if len(parts) >= 6:
                self.samples.append((time.time(), parts))

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.FIELDS,
                 "--format=csv,noheader,nounits", "-lms", "50"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            threading.Thread(target=self._read, daemon=True).start()
            t_end = time.time() + 5.0
            while not self.samples and time.time() < t_end:
                time.sleep(0.05)
        except Exception:
            self.proc = None
        return self

    def mark_start(self):
        self.t0 = time.time()

    def mark_stop(self):
        self.t1 = time.time()
        time.sleep(0.12)   # let the sample covering the end arrive

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        inside = [p for t, p in self.samples if self.t0 is not None and self.t0 - 0.05 <= t <= self.t1 + 0.06]
        if not inside:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}

        def num(x):
            try:
                return float(x)
            except ValueError:
                return None
        sm = [v for v in (num(p[0]) for p in inside) if v is not None]
        mx = [v for v in (num(p[1]) for p in inside) if v is not None]
        reasons = sorted({self.NAMES[i] for p in inside for i in range(4)
                          if p[2 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "samples": len(inside)}


# --------------------------------------------------------------------------
# CPU baseline: the reference kernel (or the oracle port) on host cores
# --------------------------------------------------------------------------
def _ref_kernel(mod, fft_workers):
    """The reference's compiled kernel class, or (fft_workers > 0) a subclass
    whose FFT hooks (the Python-dispatched ``fft_*`` / ``ifft_*`` methods of
    ``pyqg/kernel.pyx:245-263``) call scipy.fft with that many workers: the
    reference's multithreaded-FFT path without pyfftw."""
    if not fft_workers:
        return mod.PseudoSpectralKernel
    import scipy.fft as sfft
    w = fft_workers

    # the getters return views of the kernel's buffers: writing through them
    # bypasses the q / qh setters, which would transform again
    class Kernel(mod.PseudoSpectralKernel):
        def fft_q_to_qh(self):
            self.qh[...] = sfft.rfftn(self.q, axes=(-2, -1), workers=w)

        def ifft_qh_to_q(self):
            self.q[...] = sfft.irfftn(self.qh, axes=(-2, -1), workers=w)

        def ifft_uh_to_u(self):
            self.u[...] = sfft.irfftn(self.uh, axes=(-2, -1), workers=w)

        def ifft_vh_to_v(self):
            self.v[...] = sfft.irfftn(self.vh, axes=(-2, -1), workers=w)

        def fft_uq_to_uqh(self):
            self.uqh[...] = sfft.rfftn(self.uq, axes=(-2, -1), workers=w)

        def fft_vq_to_vqh(self):
            self.vqh[...] = sfft.rfftn(self.vq, axes=(-2, -1), workers=w)
    return Kernel


def cpu_model_steps(nsteps, nx=256, dt=3600.0, seed=0, threads=None, fft_workers=0):
    """Run `nsteps` two-layer nx=256 steps on the CPU with the reference itself
    (kind 'reference': pyqg's unchanged QGModel and _step_forward over its
    compiled kernel, `threads` OpenMP threads for the kernel's loops,
    `fft_workers` > 0 for multithreaded transforms) or the numpy oracle
    (kind 'port').  Returns (seconds, kind, cores)."""
    sys.path.insert(0, os.path.join(HERE, "oracle"))
    import pyqg_oracle as O
    from pyqg_gb300.model import grid_constants, spectral_filter
    from pyqg_gb300.qg_model import qg_inversion_matrix
    threads = threads or 1
    g = grid_constants(nx, nx, TWO_LAYER["L"], TWO_LAYER["L"])
    F1 = TWO_LAYER["rd"] ** -2 / (1. + TWO_LAYER["delta"])
    F2 = TWO_LAYER["delta"] * F1
    a = qg_inversion_matrix(g["wv2"], F1, F2)
    filtr = spectral_filter(g["k"], g["l"], g["dx"], g["dy"], TWO_LAYER["filterfac"])
    Qy = np.array([TWO_LAYER["beta"] + F1 * (TWO_LAYER["U1"] - TWO_LAYER["U2"]),
                   TWO_LAYER["beta"] - F2 * (TWO_LAYER["U1"] - TWO_LAYER["U2"])])
    Ubg = np.array([TWO_LAYER["U1"], TWO_LAYER["U2"]])
    q0 = 1e-7 * np.random.default_rng(seed).standard_normal((2, nx, nx))
    try:
        import build_ref
        if not build_ref.available():
            build_ref.build(quiet=True)
        mod = build_ref.load()
        kernel_cls = _ref_kernel(mod, fft_workers)
        try:
            # the reference's own, unchanged QGModel over its compiled kernel:
            # its set-up, its _step_forward (pyqg/model.py:406-436)
            import types
            import ref_import
            kmod = types.ModuleType("pyqg_ref_kernel_threads")
            kmod.PseudoSpectralKernel = kernel_cls
            for name in ("tendency_forward_euler", "tendency_ab2", "tendency_ab3"):
                setattr(kmod, name, getattr(mod, name))
            ref = ref_import.import_reference_on(kmod)
            import warnings
            with warnings.catch_warnings():
                warnings.simplefilter("ignore")
                m = ref.QGModel(nx=nx, dt=dt, ntd=threads, **TWO_LAYER, **QUIET)
            m.q = q0
            step = m._step_forward
            kind = "reference"
        except ImportError:
            # staged reference package absent: the compiled kernel's stages
            # with the same constants
            k = kernel_cls(2, nx, nx, threads, 0, 0)
            k.ll = g["ll"]
            k.kk = g["kk"]
            k.a = a
            k.Ubg = Ubg
            k.Qy = Qy
            k.filtr = filtr
            k.rek = TWO_LAYER["rek"]
            k.dt = dt
            k.q = q0
            step = lambda: (k._invert(), k._do_advection(), k._do_friction(), k._forward_timestep())
            kind = "reference"
    except Exception:
        o = O.OracleKernel(2, nx, nx, a, g["kk"], g["ll"], Ubg, Qy, filtr, TWO_LAYER["rek"], dt)
        o.set_q(q0)
        step = o.step
        kind = "port"
        threads, fft_workers = 1, 0
    step()
    t0 = time.perf_counter()
    for _ in range(nsteps):
        step()
    return time.perf_counter() - t0, kind, max(threads, fft_workers)


def cpu_variant(dt, probe_steps=10, repeats=3):
    """The fastest CPU configuration of the reference kernel on this host:
    (OpenMP threads, FFT workers) among (1, 0), (all cores, 0) and (1, all
    cores), each timed `repeats` times over `probe_steps` steps (best of
    the repeats, so that a busy moment on the host does not decide);
    (1, 0) for the numpy port."""
    ncores = os.cpu_count() or 1
    best = None
    for th, fw in dict.fromkeys([(1, 0), (ncores, 0), (1, ncores)]):
        times = []
        for _ in range(repeats):
            try:
                secs, kind, _ = cpu_model_steps(probe_steps, dt=dt, threads=th, fft_workers=fw)
            except Exception:
                break
            if kind != "reference":
                return 1, 0
            times.append(secs)
        if times and (best is None or min(times) < best[0]):
            best = (min(times), th, fw)
    return (best[1], best[2]) if best else (1, 0)


def cpu_variant_name(th, fw):
    if fw:
        return "loops 1 thread, FFT %d scipy.fft workers" % fw
    return "%d OpenMP thread%s, numpy FFT" % (th, "" if th == 1 else "s")


def cpu_baseline(dt, sample_steps):
    th, fw = cpu_variant(dt)
    secs, kind, cores = cpu_model_steps(sample_steps, dt=dt, threads=th, fft_workers=fw)
    return {"value": sim_yr_per_hr(sample_steps, dt, secs), "unit": "sim-yr/hr",
            "cores": cores, "kind": kind,
            "sample": "%d two-layer steps (nx=256, dt=3600, FP64) on the host through pyqg's own QGModel._step_forward "
                      "over its compiled kernel, %.1f ms/step (%s, the fastest of "
                      "1 thread / all cores / multithreaded FFT)"
                      % (sample_steps, 1e3 * secs / sample_steps, cpu_variant_name(th, fw))}


def run_reference(args, rank, world):
    if rank != 0:
        return
    dt = 3600.0
    sample = min(args.chunk, 100)   # model steps per timed step on the CPU
    th, fw = cpu_variant(dt)
    secs, kind, cores = cpu_model_steps(max(1, args.warmup), threads=th, fft_workers=fw)  # warm-up steps
    times = []
    for _ in range(args.steps):
        s, kind, cores = cpu_model_steps(sample, dt=dt, threads=th, fft_workers=fw)
        times.append(s)
    total = sum(times)
    value = sim_yr_per_hr(args.steps * sample, dt, total)
    line = {"metric": METRIC, "value": value, "unit": "sim-yr/hr", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * total / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "impl": "reference",
            "config": {"workload": "two-layer QG nx=ny=256 dt=3600 FP64 (standard two-layer physics), "
                                   "%d model steps per timed step" % sample,
                       "model_steps_per_step": sample, "l2": "n/a (CPU)"},
            "cpu_baseline": {"value": value, "unit": "sim-yr/hr", "cores": cores, "kind": kind,
                             "sample": "%d x %d two-layer nx=256 steps through pyqg's own QGModel._step_forward "
                                       "over its compiled kernel (%s)"
                                       % (args.steps, sample, cpu_variant_name(th, fw))},
            "e2e": {"value": value, "unit": "sim-yr/hr", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0},
            "gpu_launches": 0}
    print(json.dumps(line), flush=True)


# --------------------------------------------------------------------------
# GPU arm
# --------------------------------------------------------------------------
def stored_traffic(name):
    """DRAM bytes of one launch of kernel `name` from the committed ncu
    capture (profiles/traffic.json), with the capture's command and date:
    ncu cannot run inside the timed region, so this figure is not measured
    by the run that prints it."""
    try:
        with open(os.path.join(HERE, "profiles", "traffic.json")) as f:
            e = json.load(f).get(name)
        if isinstance(e, dict):
            return e.get("bytes"), "stored ncu capture: %s (%s)" % (e.get("command"), e.get("date"))
        return e, "stored ncu capture (profiles/traffic.json)"
    except Exception:
        return None, None


def algorithmic_bytes(nz, ny, nx):
    """Compulsory HBM bytes of one FP64 model step with the state resident:
    read qh, dqhdt_p, dqhdt_pp and write qh, dqhdt (16 B each per spectral
    point) plus read and write q (8 B per grid point)."""
    S = nz * ny * (nx // 2 + 1)
    P = nz * ny * nx
    return 80 * S + 16 * P


def run_ours(args, rank, world, local_rank):
    import ctypes
    import torch
    import pyqg_gb300 as P
    from pyqg_gb300 import _lib
    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    nx, dt = args.nx, 3600.0
    m = P.QGModel(nx=nx, dt=dt, **TWO_LAYER, **QUIET)
    q0 = 1e-7 * np.random.default_rng(1000 + rank).standard_normal((2, nx, nx))
    m.q = q0
    stream = torch.cuda.current_stream(dev)
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device=dev)
    L = _lib.lib()

    def state():
        if m._role["dqhdt_p"] == m._role["dqhdt_pp"]:
            m._own("dqhdt_pp", copy=True)
        return _lib.State(m._ptr("q"), m._ptr("qh"), m._ptr("dqhdt"), m._ptr("dqhdt_p"),
                          m._ptr("dqhdt_pp"), m._ablevel, m._tc, m._t, m._dt)

    def commit(st):
        idx = {b.data_ptr(): i for i, b in enumerate(m._tend)}
        m._role = {"dqhdt": idx[st.dqhdt], "dqhdt_p": idx[st.dqhdt_p],
                   "dqhdt_pp": idx[st.dqhdt_pp]}
        m._ablevel, m._tc, m._t = st.ablevel, st.tc, st.t

    def device_step():
        st = state()
        _lib.check(L.pqg_step(m._plan, ctypes.byref(st), args.chunk, None,
                              ctypes.c_void_p(stream.cuda_stream)))
        commit(st)

    def timed(nsteps):
        evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
               for _ in range(nsteps)]
        for i in range(nsteps):
            flush.zero_()
            evs[i][0].record(stream)
            device_step()
            evs[i][1].record(stream)
        torch.cuda.synchronize()
        return [a.elapsed_time(b) for a, b in evs]

    # the other transform engine, measured beside the default one
    other = "fp64" if m.engine == "fixed" else "fixed"
    engine = m.engine
    alt = None
    try:
        m.engine = other
        for _ in range(args.warmup):
            device_step()
        torch.cuda.synchronize()
        alt_ms = timed(max(3, args.steps // 4))
        alt = sim_yr_per_hr(len(alt_ms) * args.chunk, dt, sum(alt_ms) / 1e3)
    except Exception:
        alt = None
    m.engine = engine

    # warm-up (also captures and caches the CUDA graphs)
    for _ in range(args.warmup):
        device_step()
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    with ClockSampler(local_rank) as clocks:
        torch.cuda.synchronize()
        clocks.mark_start()
        ms = timed(args.steps)
        clocks.mark_stop()
    if world > 1:
        torch.distributed.barrier()
    model_steps = args.steps * args.chunk
    value, total_s = replica_value(sum(ms) / 1e3, model_steps, dt, world, dev)

    # per-kernel durations (CUDA events around every launch, no graph)
    st = state()
    kms = (ctypes.c_double * 2)()
    kcnt = (ctypes.c_int * 2)()
    flush.zero_()
    _lib.check(L.pqg_step_profile(m._plan, ctypes.byref(st), args.chunk, kms, kcnt,
                                  ctypes.c_void_p(stream.cuda_stream)))
    commit(st)
    row_ev, col_ev = kms[0] / kcnt[0], kms[1] / kcnt[1]
    # Events around every launch add their own overhead (the two event-timed
    # durations sum to more than a graph-replayed model step), so each
    # kernel's in-step time is its share of the event-timed pair times the
    # graph-timed model step; the two in-step times sum to the step.
    step_ms = sum(ms) / (len(ms) * args.chunk)
    row_ms = step_ms * row_ev / (row_ev + col_ev)
    col_ms = step_ms * col_ev / (row_ev + col_ev)

    # end to end through the public model API with host buffers
    qhost = torch.from_numpy(q0.copy()).pin_memory().numpy()
    for _ in range(2):
        m.q = qhost
        m.tmax = m.t + args.chunk * dt
        m.run()
        _ = m.q
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        m.q = qhost                      # H2D of the step's input state
        m.tmax = m.t + args.chunk * dt
        m.run()
        qout = m.q                       # D2H of the result
    torch.cuda.synchronize()
    e2e_s = time.perf_counter() - t0
    e2e = world * sim_yr_per_hr(model_steps, dt, e2e_s)
    del qout

    if rank != 0:
        return
    hbm, peak_kind = peaks()
    nz = 2
    # dominant kernel: the larger of the two per-step kernels; its share of
    # the step's compulsory bytes (column kernel: spectral state 80 S,
    # row kernel: physical q 16 P)
    S = nz * nx * (nx // 2 + 1)
    Pn = nz * nx * nx
    sfx = "_fx" if engine == "fixed" else ""
    if col_ms >= row_ms:
        name, kms_, nbytes = "k_col_fused" + sfx, col_ms, 80 * S
    else:
        name, kms_, nbytes = "k_row_adv" + sfx, row_ms, 16 * Pn
    achieved = nbytes / (kms_ * 1e-3) / 1e9
    traffic, traffic_src = stored_traffic(name)
    step_bytes = algorithmic_bytes(nz, nx, nx)
    base = cpu_baseline(dt, args.cpu_sample)
    line = {
        "metric": METRIC, "value": value, "unit": "sim-yr/hr", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": sum(ms) / len(ms),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64" if engine == "fp64" else "f64+int64",
        "data": "synthetic (seeded 1e-7 N(0,1) initial PV)",
        "config": {"workload": "two-layer QG nx=ny=256 dt=3600 FP64 (standard two-layer physics), "
                               "%d model steps per timed step" % args.chunk,
                   "engine": engine if engine == "fp64" else
                   "fixed (FP64 state and pointwise physics; transforms in 64-bit block fixed point)",
                   "value_other_engine": {other: alt},
                   "model_steps_per_step": args.chunk,
                   "model_steps_per_s": model_steps * world / total_s,
                   "l2": "flushed (256 MB write) before every timed step",
                   "parallelism": "replicas" if world > 1 else "single"},
        "e2e": {"value": e2e, "unit": "sim-yr/hr", "h2d_bytes_per_step": int(q0.nbytes),
                "d2h_bytes_per_step": int(q0.nbytes),
                "api": "QGModel.q = host q; QGModel.run() for the chunk; QGModel.q"},
        "roofline": {"bound": "hbm", "kernel": name, "achieved": achieved, "peak": hbm,
                     "unit": "GB/s", "frac": achieved / hbm, "traffic": traffic,
                     "traffic_source": traffic_src,
                     "peak_source": peak_kind,
                     "kernel_ms": {"k_row_adv" + sfx: row_ms, "k_col_fused" + sfx: col_ms},
                     "kernel_ms_basis": "share of the event-timed launch pair (%.4f / %.4f ms) "
                                        "times the graph-timed model step (%.4f ms)"
                                        % (row_ev, col_ev, step_ms),
                     "algorithmic_bytes_per_launch": nbytes,
                     "step": {"ms": step_ms, "algorithmic_bytes": step_bytes,
                              "achieved": step_bytes / (step_ms * 1e-3) / 1e9,
                              "frac": step_bytes / (step_ms * 1e-3) / 1e9 / hbm},
                     "note": "single nx=256 model: latency-bound (FP64 pipe / integer ALU "
                             "under 55% busy, state L2-resident); see profiles/"},
        "cpu_baseline": base,
        "clocks": clocks.summary(),
        "gpu_launches": args.steps * (2 * args.chunk + 2),
    }
    if world == 1 and not args.no_ensemble:
        try:
            line["ensemble"] = ensemble_throughput(args)
        except Exception as exc:
            line["ensemble"] = {"error": "%s: %s" % (type(exc).__name__, exc)}
    if world == 1 and not args.no_closure:
        try:
            line["closure"] = closure_throughput(args, value, alt if other == "fp64" else value)
        except Exception as exc:      # reported, the main line stands
            line["closure"] = {"error": "%s: %s" % (type(exc).__name__, exc)}
    print(json.dumps(line), flush=True)


def closure_throughput(args, plain_value, plain_fp64_transforms=None):
    """Closure workload: two-layer nx=64 FP32 members with the 8-layer
    convolutional closure applied every step (and the same ensemble without
    it), aggregate simulated years per wall-clock hour over the members.
    The network is randomly initialised: its cost does not depend on the
    weights."""
    import torch
    import pyqg_gb300 as P
    from pyqg_gb300.closure import CNNParameterization, ConvNet
    from pyqg_gb300.coarsen import PHYSICS
    B, dt, chunk = args.closure_members, 7200.0, args.closure_chunk
    members = [("qg", dict(nx=64, dt=dt, **PHYSICS))] * B
    rng = np.random.default_rng(3000)
    qs = [1e-7 * rng.standard_normal((2, 64, 64)) for _ in range(B)]
    net = ConvNet(max_batch=B, seed=0)
    CNNParameterization(net, ([0.0, 0.0], [1e-6, 1e-7], [0.0, 0.0], [1e-12, 1e-13]))
    stream = torch.cuda.current_stream()
    res = {"workload": "%d two-layer QG members nx=64 dt=7200 FP32 (FP64-built matrices), "
                       "8-layer 5x5 CNN closure (2-128-64-32-32-32-32-32-2, BF16 tcgen05) every step; "
                       "%d steps per timed step" % (B, chunk)}
    for name, closure in (("closure", True), ("no_closure", False)):
        ens = P.Ensemble(members, precision="fp32")
        ens.set_q(qs)
        if closure:
            ens.set_closure(net)
        for _ in range(max(1, args.warmup)):
            ens.step(chunk)
        torch.cuda.synchronize()
        evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
               for _ in range(args.closure_steps)]
        for a, b in evs:
            a.record(stream)
            ens.step(chunk)
            b.record(stream)
        torch.cuda.synchronize()
        sec = sum(a.elapsed_time(b) for a, b in evs) / 1e3
        res[name] = {"value": sim_yr_per_hr(B * chunk * args.closure_steps, dt, sec),
                     "ms_per_model_step": 1e3 * sec / (chunk * args.closure_steps)}
        del ens
    x = torch.randn(B, 2, 64, 64, device="cuda")
    y = torch.empty_like(x)
    for _ in range(3):
        net.forward(x, y)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(10):
        net.forward(x, y)
    e1.record(stream)
    torch.cuda.synchronize()
    cnn_ms = e0.elapsed_time(e1) / 10
    flops = 2.0 * 366400 * B * 64 * 64
    bf16 = None
    pk = os.path.join(HERE, "MEASURED_PEAKS.json")
    if os.path.exists(pk):
        with open(pk) as f:
            bf16 = json.load(f).get("bf16_tflops")
    tfs = flops / (cnn_ms * 1e-3) / 1e12
    res["cnn_forward"] = {"ms": cnn_ms, "tflops": tfs, "peak_tflops": bf16,
                          "frac": (tfs / bf16) if bf16 else None, "unit": "TFLOP/s",
                          "bound": "tensor", "peak_source": "measured" if bf16 else None}
    res["unit"] = "sim-yr/hr (sum over members)"
    res["vs_nx256_plain_fp64"] = res["closure"]["value"] / plain_value if plain_value else None
    # the same ratio against the nx=256 run with FP64 transforms (the
    # default engine above transforms in 64-bit fixed point)
    res["vs_nx256_plain_fp64_transforms"] = (res["closure"]["value"] / plain_fp64_transforms
                                             if plain_fp64_transforms else None)
    # the closure's plain baseline: a 16-member FP64 nx=256 plain ensemble
    base = nx256_ensemble16(args)
    res["nx256_fp64_ensemble16"] = base
    agg = base["value"]
    res["vs_nx256_fp64_ensemble16"] = res["closure"]["value"] / agg
    res["per_member"] = {"closure_nx64": res["closure"]["value"] / B,
                         "nx256_fp64_ensemble16": agg / 16, "nx256_fp64_single": plain_value,
                         "ratio_vs_ensemble16": (res["closure"]["value"] / B) / (agg / 16)}
    res["claim"] = ("vs_nx256_fp64_ensemble16: aggregate over the 512 closure members against the "
                    "aggregate of the 16-member FP64 nx=256 ensemble, both filling one GPU")
    return res


def nx256_ensemble16(args, nmembers=16):
    """Aggregate sim-yr/hr of 16 FP64 nx=256 two-layer plain members (standard
    two-layer physics, dt = 3600 s), the faster of two ways of running them on one GPU:
    the batched FP64 ensemble (FP64 transforms, one launch pair per step for
    all members) and 16 independent single models, each with the fused step
    of the default engine on its own stream (their kernels overlap)."""
    import torch
    import pyqg_gb300 as P
    from pyqg_gb300.coarsen import PHYSICS
    dt, chunk, reps = 3600.0, args.closure_chunk, max(2, args.closure_steps)
    rng = np.random.default_rng(4000)
    qs = [1e-7 * rng.standard_normal((2, 256, 256)) for _ in range(nmembers)]
    stream = torch.cuda.current_stream()
    out = {"workload": "%d two-layer QG members nx=256 dt=3600 FP64 (standard two-layer physics), no closure"
                       % nmembers}
    # (a) batched FP64 ensemble
    ens = P.Ensemble([("qg", dict(nx=256, dt=dt, **PHYSICS))] * nmembers, precision="fp64")
    ens.set_q(qs)
    ens.step(8)
    ens.autotune()
    ens.step(chunk)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(reps):
        ens.step(chunk)
    e1.record(stream)
    torch.cuda.synchronize()
    sec = e0.elapsed_time(e1) / 1e3
    out["batched_ensemble"] = {"value": sim_yr_per_hr(nmembers * chunk * reps, dt, sec),
                               "ms_per_model_step": 1e3 * sec / (chunk * reps)}
    del ens
    # (b) independent fused single models on their own streams
    streams = [torch.cuda.Stream() for _ in range(nmembers)]
    models = []
    for q, st in zip(qs, streams):
        with torch.cuda.stream(st):
            m = P.QGModel(nx=256, dt=dt, **PHYSICS, **QUIET)
            m.q = q
            m._step_fused(chunk)
        models.append(m)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(reps):
        for m in models:
            m._step_fused(chunk)
    torch.cuda.synchronize()
    sec = time.perf_counter() - t0
    out["concurrent_single_models"] = {"value": sim_yr_per_hr(nmembers * chunk * reps, dt, sec),
                                       "ms_per_model_step": 1e3 * sec / (chunk * reps),
                                       "engine": models[0].engine,
                                       "timing": "host clock around all streams, synchronized on both sides"}
    del models
    best = max(("batched_ensemble", "concurrent_single_models"), key=lambda k: out[k]["value"])
    out["value"] = out[best]["value"]
    out["chosen"] = best
    out["unit"] = "sim-yr/hr (sum over members)"
    return out


def mixed_ensemble_1024(rng):
    """The 1024 mixed-size members (614 x nx=64, 307 x nx=128, 103 x nx=256; 20 %
    three-layer; beta and rek drawn per member) as an FP32 Ensemble with
    seeded initial PV."""
    import pyqg_gb300 as P
    members = []
    for nx, cnt in ((64, 614), (128, 307), (256, 103)):
        dt = 3600.0 if nx == 256 else 7200.0
        for i in range(cnt):
            beta = rng.uniform(0.5, 2) * 1.5e-11
            rek = rng.uniform(0.5, 2) * 5.787e-7
            if i < int(0.2 * cnt + 0.5):
                members.append(("layered", dict(nx=nx, dt=dt, nz=3, H=[500., 1000., 2500.],
                                                U=[0.05, 0.02, 0.0], V=[0., 0., 0.], beta=beta, rek=rek)))
            else:
                members.append(("qg", dict(nx=nx, dt=dt, beta=beta, rek=rek)))
    ens = P.Ensemble(members, precision="fp32")
    qs = [1e-7 * rng.standard_normal((3 if k == "layered" else 2, kw["nx"], kw["nx"])) for k, kw in members]
    ens.set_q(qs)
    return ens, members


def ensemble_throughput(args):
    """Mixed-size ensemble workload: 1024 FP32 members of uneven size, autotuned launch
    shapes, groups on concurrent branches and steady-state stretches
    replayed as CUDA graphs."""
    import torch
    rng = np.random.default_rng(1234)
    ens, members = mixed_ensemble_1024(rng)
    ens.step(4)
    ens.autotune()
    stream = torch.cuda.current_stream()
    nsteps = args.ensemble_steps
    ens.step(32)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    ens.step(nsteps)
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / nsteps
    S = sum(g.B * g.nz * g.nx * (g.nx // 2 + 1) for g in ens.groups)
    Pn = sum(g.B * g.nz * g.nx * g.nx for g in ens.groups)
    nbytes = 40 * S + 8 * Pn
    hbm, kind = peaks()
    ach = nbytes / (ms * 1e-3) / 1e9
    traffic, traffic_src = stored_traffic("ensemble_1024_mixed_step")
    return {"workload": "1024 FP32 members (614 x nx=64, 307 x nx=128, 103 x nx=256, "
                        "20 % three-layer), uneven beta / rek, autotuned, CUDA graphs",
            "ms_per_ensemble_step": ms, "member_steps_per_s": len(members) / (ms * 1e-3),
            "roofline": {"bound": "hbm", "achieved": ach, "peak": hbm, "unit": "GB/s", "frac": ach / hbm,
                         "algorithmic_bytes_per_step": nbytes, "peak_source": kind, "traffic": traffic,
                         "traffic_source": traffic_src,
                         "note": "compulsory bytes 40 S + 8 P (FP32) per ensemble step; traffic = measured "
                                 "DRAM bytes of one steady step (ncu, serialised launches)"}}


def profile_case(args):
    """Small workloads for profiler captures (no timing, no output line)."""
    import torch
    import pyqg_gb300 as P
    if args.profile_step:
        m = P.QGModel(nx=args.nx, dt=3600.0, **TWO_LAYER, **QUIET)
        m.q = 1e-7 * np.random.default_rng(0).standard_normal((2, args.nx, args.nx))
        m._step_fused(args.profile_step)
    if args.profile_ensemble:
        ens, _ = mixed_ensemble_1024(np.random.default_rng(1234))
        ens.step(4)
        ens.autotune()
        torch.cuda.synchronize()
        # the steps a profiler should see: ncu --nvtx --nvtx-include "ensemble_steps/"
        torch.cuda.nvtx.range_push("ensemble_steps")
        ens.step(args.profile_ensemble)
        torch.cuda.synchronize()
        torch.cuda.nvtx.range_pop()
    if args.profile_cnn:
        from pyqg_gb300.closure import ConvNet
        net = ConvNet(max_batch=args.profile_cnn, seed=0)
        x = torch.randn(args.profile_cnn, 2, 64, 64, device="cuda")
        y = torch.empty_like(x)
        for _ in range(2):
            net.forward(x, y)
    torch.cuda.synchronize()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--chunk", type=int, default=500)
    ap.add_argument("--nx", type=int, default=256)
    ap.add_argument("--cpu-sample", type=int, default=1000)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--closure-members", type=int, default=512)
    ap.add_argument("--closure-steps", type=int, default=5)
    ap.add_argument("--closure-chunk", type=int, default=100)
    ap.add_argument("--no-closure", action="store_true", help="skip the closure-ensemble measurement")
    ap.add_argument("--no-ensemble", action="store_true", help="skip the 1024-member mixed-size ensemble measurement")
    ap.add_argument("--ensemble-steps", type=int, default=200)
    ap.add_argument("--profile-step", type=int, default=0, metavar="N",
                    help="only run N fused nx=256 steps (a small case for profilers) and exit")
    ap.add_argument("--profile-cnn", type=int, default=0, metavar="B",
                    help="only run two closure-network forwards of a batch of B and exit")
    ap.add_argument("--profile-ensemble", type=int, default=0, metavar="N",
                    help="only run N steps of the 1024-member mixed-size FP32 ensemble and exit")
    args = ap.parse_args()
    if args.profile_step or args.profile_cnn or args.profile_ensemble:
        profile_case(args)
        return
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        run_reference(args, rank, world)
        return
    if world > 1:
        import torch
        torch.distributed.init_process_group("nccl")
    run_ours(args, rank, world, local_rank)
    if world > 1:
        import torch
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
