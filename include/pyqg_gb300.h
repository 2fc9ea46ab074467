/*
 * pyqg_gb300 — C ABI of the GB300 (sm_103a) pseudo-spectral time step.
 *
 * The entry points replace, one for one, the hot-path interface of pyqg's
 * Cython class `PseudoSpectralKernel` (pyqg/kernel.pyx:32-637): its
 * constructor, its constant setters, its transforms and its five stage
 * methods, plus a fused multi-step call that pyqg runs as a Python loop
 * (`Model.run` -> `Model._step_forward`, pyqg/model.py:280-283,406-436).
 *
 * Conventions
 *   - Shapes follow the reference: physical fields (nz, ny, nx) float64 and
 *     spectral fields (nz, nl, nk) complex128 with nl = ny, nk = nx/2 + 1,
 *     C order.  Complex arrays are interleaved (re, im) `double` pairs.
 *   - Pointers to fields are DEVICE pointers (16-byte aligned); pointers to
 *     constants (pqg_set_*) are HOST pointers, copied into the plan.
 *   - `stream` is a cudaStream_t passed as void* (NULL = legacy default).
 *     All compute calls are asynchronous on that stream.
 *   - Every function returns PQG_OK (0) or a PQG_ERR_* code; the message of
 *     the last error on the calling thread is returned by pqg_last_error().
 *   - Threads: like pyqg's kernel object, a plan, an ensemble or a network
 *     is not re-entrant: calls on one object must not overlap from several
 *     host threads.  The ensemble step calls (pqg_ens_step_many,
 *     pqg_ens_autotune, pqg_ens_set_constants) share one process-wide cache
 *     of CUDA graphs, so ensembles are stepped from one host thread at a
 *     time.
 *   - Transforms: pqg_rfft2 is unnormalised, pqg_irfft2 scales by 1/(nx ny)
 *     and ignores the imaginary parts of the k = 0 and k = nx/2 columns after
 *     the y transform, as numpy.fft.irfftn / FFTW c2r do.
 */
#ifndef PYQG_GB300_H
#define PYQG_GB300_H

#ifdef __cplusplus
extern "C" {
#endif

#define PQG_OK 0
#define PQG_ERR_INVALID 1      /* bad argument (NULL pointer, negative size) */
#define PQG_ERR_UNSUPPORTED 2  /* grid size the kernels do not handle       */
#define PQG_ERR_CUDA 3         /* CUDA runtime error (message has details)   */
#define PQG_ERR_NOMEM 4        /* device or host allocation failed           */
#define PQG_ERR_STATE 5        /* call out of order (e.g. constants unset)   */
#define PQG_ERR_TIMEOUT 6      /* a bounded device-side wait ran out        */

typedef struct pqg_plan pqg_plan;

/* Optional outputs of the last step of pqg_step (any may be NULL). These are
 * the intermediates the reference keeps as state after `_step_forward`:
 * ph, uh, vh (spectral) and u, v, uq, vq (physical), uqh, vqh (spectral). */
typedef struct pqg_aux {
    double *ph, *uh, *vh;
    double *u, *v, *uq, *vq;
    double *uqh, *vqh;
} pqg_aux;

/* Time-stepping state for pqg_step.  `dqhdt_p` and `dqhdt_pp` must be
 * distinct buffers.  pqg_step rotates the history pointers the way the
 * reference rotates the values (pyqg/kernel.pyx:509-510): on return
 * `dqhdt` and `dqhdt_p` point to the same buffer (the newest tendency). */
typedef struct pqg_state {
    double *q;          /* (nz, ny, nx) physical PV                    */
    double *qh;         /* (nz, nl, nk) spectral PV                    */
    double *dqhdt;      /* newest tendency (output only)               */
    double *dqhdt_p;    /* previous tendency                           */
    double *dqhdt_pp;   /* tendency before previous (overwritten)      */
    int ablevel;        /* 0: forward Euler next, 1: AB2, >=2: AB3     */
    long long tc;       /* step counter  (pyqg/kernel.pyx:98)          */
    double t;           /* model time    (pyqg/kernel.pyx:99)          */
    double dt;          /* time step     (pyqg/kernel.pyx:97)          */
} pqg_state;

/* Library version (major*10000 + minor*100 + patch). */
int pqg_version(void);

/* Message of the last failed call on this thread ("" if none). */
const char *pqg_last_error(void);

/* Create / destroy a plan for an (nz, ny, nx) grid: FFT descriptors,
 * twiddle tables, constants and the transposition scratch (device memory).
 * Replaces PseudoSpectralKernel.__init__ (pyqg/kernel.pyx:120-206).
 * nx and ny must be even; nx/2 and ny must factor into 2, 3 and 5 and be
 * at most 2048; 3*nz*ny*16 bytes must fit the per-block shared memory. */
int pqg_plan_create(pqg_plan **plan, int nz, int ny, int nx);
int pqg_plan_destroy(pqg_plan *plan);

/* Constants (host arrays, copied).  Setting the wavenumbers also sets
 * k2l2 = kk^2 + ll^2 and the ikQy table.
 *   kk (nk), ll (nl)          -> pyqg/kernel.pyx:536-556 (kk, ll setters)
 *   k2l2 (nl, nk)             -> pyqg/kernel.pyx:82 (public _k2l2)
 *   a (nz, nz, nl, nk) real   -> pyqg/kernel.pyx:557-563 (a setter)
 *   Ubg (nz)                  -> pyqg/kernel.pyx:564-568 (Ubg setter)
 *   Qy (nz)                   -> pyqg/kernel.pyx:569-575 (Qy setter, ikQy)
 *   filtr (nl, nk)            -> pyqg/kernel.pyx:90 (public filtr)
 *   rek                       -> pyqg/kernel.pyx:93 (public rek)         */
int pqg_set_wavenumbers(pqg_plan *plan, const double *kk, const double *ll);
int pqg_set_k2l2(pqg_plan *plan, const double *k2l2);
int pqg_set_inversion(pqg_plan *plan, const double *a);
int pqg_set_ubg(pqg_plan *plan, const double *Ubg);
int pqg_set_qy(pqg_plan *plan, const double *Qy);
int pqg_set_filter(pqg_plan *plan, const double *filtr);
int pqg_set_rek(pqg_plan *plan, double rek);

/* Transform engine of the fused step (pqg_step), no counterpart in the
 * reference: 0 = FP64 Stockham transforms (default); 1 = 64-bit block
 * fixed-point transforms (exact integer additions, Q62 twiddles rounded to
 * nearest, 50-52 bits below each sequence's largest element) with all
 * pointwise physics in FP64.  Engine 1 takes the transforms off GB300's
 * FP64 pipe; it needs power-of-two nx and ny.  pqg_get_engine returns the
 * current engine (-1 for a NULL plan). */
int pqg_set_engine(pqg_plan *plan, int engine);
int pqg_get_engine(const pqg_plan *plan);

/* Batched 2-D real transforms over `nplanes` (ny, nx) planes.
 * Replace the planned transforms and the fft/ifft helpers
 * (pyqg/kernel.pyx:208-267,291-309).  Always FP64, whatever the plan's
 * engine (which applies to the transforms inside the step). */
int pqg_rfft2(pqg_plan *plan, const double *x, double *xh, int nplanes,
              void *stream);
int pqg_irfft2(pqg_plan *plan, const double *xh, double *x, int nplanes,
               void *stream);

/* _invert (pyqg/kernel.pyx:312-355): ph = a qh, uh = -il ph, vh = ik ph,
 * u = irfft2(uh), v = irfft2(vh).  ph/uh/vh may be NULL (not stored). */
int pqg_invert(pqg_plan *plan, const double *qh, double *ph, double *uh,
               double *vh, double *u, double *v, void *stream);

/* _do_advection (pyqg/kernel.pyx:357-395): uq = (u + Ubg) q, vq = v q,
 * uqh, vqh = rfft2, dqhdt = -(ik uqh + il vqh + ikQy ph).  uq, vq, uqh and
 * vqh may be NULL (not stored). */
int pqg_do_advection(pqg_plan *plan, const double *q, const double *u,
                     const double *v, const double *ph, double *uq,
                     double *vq, double *uqh, double *vqh, double *dqhdt,
                     void *stream);

/* _do_friction (pyqg/kernel.pyx:444-461): if rek != 0,
 * dqhdt[nz-1] += rek k2l2 ph[nz-1]. */
int pqg_do_friction(pqg_plan *plan, const double *ph, double *dqhdt,
                    void *stream);

/* Spectral part of _do_q_subgrid_parameterization (pyqg/kernel.pyx:424-442):
 * dqh = rfft2(dq); dqhdt += dqh.  dqh may be NULL. */
int pqg_do_q_forcing(pqg_plan *plan, const double *dq, double *dqh,
                     double *dqhdt, void *stream);

/* Spectral part of _do_uv_subgrid_parameterization
 * (pyqg/kernel.pyx:397-422): duh, dvh = rfft2(du, dv);
 * dqhdt += -il duh + ik dvh.  duh and dvh may be NULL. */
int pqg_do_uv_forcing(pqg_plan *plan, const double *du, const double *dv,
                      double *duh, double *dvh, double *dqhdt, void *stream);

/* _forward_timestep (pyqg/kernel.pyx:463-526): FE/AB2/AB3 by `ablevel`,
 * qh = filtr (qh + dt1 dqhdt + dt2 dqhdt_p + dt3 dqhdt_pp), q = irfft2(qh).
 * With rotate != 0 the history is also shifted in place
 * (dqhdt_pp <- dqhdt_p, dqhdt_p <- dqhdt) exactly as the reference does;
 * with rotate == 0 the caller rotates its buffer roles instead. */
int pqg_forward_timestep(pqg_plan *plan, int ablevel, double dt, double *qh,
                         const double *dqhdt, double *dqhdt_p,
                         double *dqhdt_pp, double *q, int rotate,
                         void *stream);

/* `nsteps` whole steps without parameterization hooks, in the order of
 * pyqg/model.py:406-436 (_invert, _do_advection, _do_friction,
 * _forward_timestep), fused into two kernels per step and replayed from a
 * cached CUDA graph.  Updates *state (q, qh, history pointers, ablevel, tc,
 * t).  `aux` (may be NULL) receives the intermediates of the last step. */
int pqg_step(pqg_plan *plan, pqg_state *state, int nsteps,
             const pqg_aux *aux, void *stream);

/* ---------------------------------------------------------------------
 * Ensembles (no counterpart in the reference): B independent members of
 * one shape (nz, ny, nx), physics shared except beta (Qy), bottom drag and
 * background flow per member, advanced together by the fused step in FP32
 * (precision 4) or FP64 (precision 8).  The ensemble owns its device
 * state.  Grids: powers of two, 16..1024.
 * ------------------------------------------------------------------- */
typedef struct pqg_ens pqg_ens;

const char *pqg_ens_last_error(void);
int pqg_ens_create(pqg_ens **ens, int nmembers, int nz, int ny, int nx,
                   int precision);
int pqg_ens_destroy(pqg_ens *ens);
/* shared constants (host, FP64; rounded once to the ensemble precision):
 * a (nz, nz, nl, nk), kk (nk), ll (nl), filtr (nl, nk), time step dt */
int pqg_ens_set_constants(pqg_ens *ens, const double *a, const double *kk,
                          const double *ll, const double *filtr, double dt);
/* per member (host, FP64): Ubg (B, nz), Qy (B, nz), rek (B) */
int pqg_ens_set_members(pqg_ens *ens, const double *Ubg, const double *Qy,
                        const double *rek);
/* q (B, nz, ny, nx) FP64 host in/out; set_q also resets the AB3 history */
int pqg_ens_set_q(pqg_ens *ens, const double *q, void *stream);
int pqg_ens_get_q(pqg_ens *ens, double *q, void *stream);
int pqg_ens_step(pqg_ens *ens, int nsteps, void *stream);
/* several ensembles (e.g. one per grid size), each on its own stream
 * branch so that they overlap on the GPU.  Steady-state stretches of 16
 * steps are captured once into a CUDA graph and replayed (environment
 * PQG_ENS_NO_GRAPHS=1 disables this). */
int pqg_ens_step_many(pqg_ens **ens, int count, int nsteps, void *stream);
/* autotuner: times the row kernel over (rows per CTA, threads) and the
 * fused column kernel over (columns per CTA, threads) on the ensemble's own
 * state, keeps the fastest, then, for square grids of 16 to 64 points (FP64:
 * up to 32) and at most 4 layers, times four whole steps of the per-member
 * kernel (one CTA per member, the member's mixed planes resident in shared
 * memory; 128 or 256 threads) against four steps of the row and column
 * kernels and keeps the faster schedule.  The state is restored.  out (may
 * be NULL, else 10 values) gets {rows per CTA, row threads, row ms, columns
 * per CTA, column threads, column ms, per-member kernel chosen (0 / 1), its
 * threads, its ms for four steps, the two-kernel ms for four steps}.
 * Without the autotuner the row and column kernels run; PQG_ENS_FUSED=1 /
 * 0 forces the per-member kernel on / off where the shape allows it.
 * Ensembles with a closure always use the row and column kernels.
 * Synchronizes `stream`. */
int pqg_ens_autotune(pqg_ens *ens, double *out, void *stream);
/* FP64 sums per (member, layer): ke = 0.5 sum |kappa ph|^2 / M^2 and
 * enstrophy 0.5 sum |qh|^2 / M^2 over the full spectral plane (host out) */
int pqg_ens_energy(pqg_ens *ens, double *ke, double *enstrophy, void *stream);
/* learned closure for every member: each step adds the spectral transform
 * of net(q) to dq/dt after the bottom drag (the q_parameterization hook of
 * the single-model step).  The network's input and output channels must be
 * nz, its image (ny, nx) and its batch capacity at least the member count.
 * NULL detaches.  The ensemble keeps the pointer: destroy the network
 * after the ensemble or after detaching it.  Synchronizes the device. */
typedef struct pqg_cnn pqg_cnn;
int pqg_ens_set_closure(pqg_ens *ens, pqg_cnn *net);
/* device pointers of the state and the step counter / time: q is
 * (B, nz, ny, nx) and qh is (B, nz, nk, ny) -- column-contiguous, the
 * transpose of the single-model layout -- both in the ensemble precision */
int pqg_ens_state(pqg_ens *ens, void **q, void **qh, long long *tc,
                  double *t);

/* Non-finite state flag (no counterpart in the reference, whose status
 * output finds a NaN state only through its CFL assertion,
 * pyqg/model.py:564-574).  The step kernels set it when a new spectral PV
 * value is Inf or NaN; it lives in host-mapped memory, so pqg_nonfinite
 * reads it without synchronizing: it reflects the kernels that have
 * completed.  pqg_clear_nonfinite resets it (between kernels). */
int pqg_nonfinite(const pqg_plan *plan, int *flag);
int pqg_clear_nonfinite(pqg_plan *plan);

/* Instrumentation for the profile / bench tooling (no counterpart in the
 * reference): `nsteps` fused steps like pqg_step but launched one by one
 * (no graph) with CUDA events around each kernel.  On return ms[0] / ms[1]
 * hold the summed durations of the row / column kernels and counts[0] /
 * counts[1] their launch counts.  Synchronizes `stream`. */
int pqg_step_profile(pqg_plan *plan, pqg_state *state, int nsteps,
                     double *ms, int *counts, void *stream);

/* Forward 2-D real transform for callers that cannot allocate device
 * memory (no counterpart in the reference).  Same result as pqg_rfft2, but
 * needs no plan: the transposition scratch and twiddle tables are static
 * device arrays of the library (about 8.1 MiB per device, kept until the
 * process exits).  Intended for code whose device memory belongs to another
 * allocator (a framework's caching allocator or a fixed arena) and for code
 * that must not stall the device, as cudaMalloc / cudaFree can.
 *   - nplanes * ny * (nx/2 + 1) must not exceed PQG_NOALLOC_MAX_COMPLEX;
 *     larger requests fail with PQG_ERR_UNSUPPORTED and a message.
 *   - The first call on a device looks up the arrays' device addresses and
 *     a call whose (ny, nx) differs from the previous call's on that device
 *     uploads twiddle tables; make such calls before any stream capture.
 *   - All calls on a device share the arrays: calls that can overlap on the
 *     GPU (different streams without ordering) race.  Calls on one stream
 *     are safe; no state carries over between calls. */
#define PQG_NOALLOC_MAX_COMPLEX (1 << 19)
int pqg_rfft2_noalloc(const double *x, double *xh, int nplanes, int ny,
                      int nx, void *stream);

/* Inversion matrices built in FP64 on the device (the FP32 precision form
 * builds its matrices here and rounds them once):
 * a (nz, nz, nl, nk) = (S - kappa^2 I)^-1 per wavenumber, kappa^2 =
 * kk[k]^2 + ll[l]^2, 0 where singular (kappa = 0).  S is a HOST nz x nz
 * row-major array; kk (nk), ll (nl) and a are DEVICE arrays.
 *   form 0: two-layer QG, F1 = S[0][1], F2 = S[1][0]
 *           (replaces QGModel._initialize_inversion_matrix,
 *           pyqg/qg_model.py:146-161), bit-identical to the host build;
 *   form 1: layered, nz = 2..8 (replaces LayeredModel.
 *           _initialize_inversion_matrix, pyqg/layered_model.py:211-229);
 *           nz = 2 bit-identical, nz > 2 by Gauss-Jordan elimination. */
int pqg_inversion_matrix(int form, int nz, int nl, int nk, const double *S,
                         const double *kk, const double *ll, double *a,
                         void *stream);

/* Spectral advective tendency of nplanes physical fields f by (u, v):
 * out_h = ik fft(u f) + il fft(v f), FP64 transforms
 * (replaces Model._advect, pyqg/model.py:539-558). */
int pqg_advect(pqg_plan *plan, const double *f, const double *u,
               const double *v, int nplanes, double *out_h, void *stream);

/* ---------------------------------------------------------------------
 * Pointwise stages of the physical parameterizations
 * (pyqg/parameterizations.py:132-366).  Device arrays: spectral fields
 * (n, nl, nk) complex (re, im), physical fields (n, ny, nx), wavenumbers
 * kk (nk) and ll (nl); "3n" = three fields of n planes one after the
 * other.  The transforms between these stages are pqg_rfft2 /
 * pqg_irfft2.
 * Smagorinsky (pyqg/parameterizations.py:165-189):
 *   pqg_smag_strain:     out3 = [ik uh, il vh, (il uh + ik vh) / 2]
 *   pqg_smag_stress:     nu = c2dx2 sqrt(2 (Sxx^2 + Syy^2 + 2 Sxy^2)) and
 *                        p3 = [nu Sxx, nu Sxy, nu Syy] from s3 = [Sxx, Syy,
 *                        Sxy]; either output may be NULL
 *   pqg_smag_divergence: out2 = [2 (ik nSxx + il nSxy), 2 (ik nSxy + il nSyy)]
 * ZannaBolton2020 (pyqg/parameterizations.py:266-285):
 *   pqg_zb_gradients:    out4 = [ik vh, il vh, ik uh, il uh]
 *   pqg_zb_products:     from g4 = [vx, vy, ux, uy]: rv = vx - uy,
 *                        sh = vx + uy, st = ux - vy;
 *                        out3 = [rv st, rv sh, rv^2 + sh^2 + st^2]
 *   pqg_zb_combine:      from f3 = fft of those: ss = f3[2] / 2,
 *                        out2 = kappa [ik (ss - rsh) + il rs,
 *                                      il (ss + rsh) + ik rs]
 * BackscatterBiharmonic (pyqg/parameterizations.py:226-236):
 *   pqg_lap_power:       out = scale (k^2 + l^2)^power in, power 1 or 2
 *   pqg_mul_scaled:      out = (a s) b over `count` values
 *   pqg_backscatter:     out = diss - Cb llp num / (den + eps) with
 *                        num = sum_z Hi mean(psi diss), den = sum_z Hi
 *                        mean(psi llp); sums: 2n doubles of device scratch
 * RingForcing (pyqg/parameterizations.py:338-362):
 *   pqg_ring_normalize:  out[z] = mag (x - mean x) / mean|x - mean x| for
 *                        layers with keep[z] != 0, NaN for the others (the
 *                        reference's 0 / 0); x one plane, moments 2 doubles
 *                        of device scratch. */
int pqg_smag_strain(int n, int nl, int nk, const double *kk, const double *ll,
                    const double *uh, const double *vh, double *out3,
                    void *stream);
int pqg_smag_stress(int n, int ny, int nx, const double *s3, double c2dx2,
                    double *nu, double *p3, void *stream);
int pqg_smag_divergence(int n, int nl, int nk, const double *kk,
                        const double *ll, const double *n3, double *out2,
                        void *stream);
int pqg_zb_gradients(int n, int nl, int nk, const double *kk, const double *ll,
                     const double *uh, const double *vh, double *out4,
                     void *stream);
int pqg_zb_products(int n, int ny, int nx, const double *g4, double *out3,
                    void *stream);
int pqg_zb_combine(int n, int nl, int nk, const double *kk, const double *ll,
                   const double *f3, double kappa, double *out2, void *stream);
int pqg_lap_power(int n, int nl, int nk, const double *kk, const double *ll,
                  int power, double scale, const double *in, double *out,
                  void *stream);
/* out[i] = sum_j m[i][j] in[j] (j in order) for planes of `plane` doubles
 * (a complex plane counts re and im); m is a host nout x nin row-major
 * matrix, at most 8 x 8.  The layer combinations of the device
 * diagnostics: S ph, the modal projection, p1 - p2 and del1 u1 + del2 u2
 * (pyqg/qg_model.py:231-263, pyqg/layered_model.py:261-300). */
int pqg_layer_mix(int nout, int nin, long long plane, const double *m,
                  const double *in, double *out, void *stream);
int pqg_mul_scaled(long long count, const double *a, double s, const double *b,
                   double *out, void *stream);
int pqg_backscatter(int n, int ny, int nx, const double *psi,
                    const double *diss, const double *llp, const double *Hi,
                    double cb, double eps, double *sums, double *out,
                    void *stream);
int pqg_ring_normalize(int n, int ny, int nx, const double *x, const int *keep,
                       double mag, double *moments, double *out, void *stream);

/* Coarse-graining of one state (no counterpart in the reference): the fine
 * spectral PV qh_f (nz, ny_f, nx_f/2+1) is truncated sharply to the coarse
 * plan's grid (|k| < nx_c/2, |l| < ny_c/2, amplitudes kept) giving q_c
 * (nz, ny_c, nx_c), and the subgrid forcing
 *   S = filtered(J(psi, q)) - J(filtered psi, filtered q)
 * with J(psi, q) = u q_x + v q_y evaluated spectrally on each grid.  Both
 * plans need their wavenumbers and inversion matrices; FP64 transforms. */
int pqg_coarse_forcing(pqg_plan *fine, pqg_plan *coarse, const double *qh_f,
                       double *q_c, double *S, void *stream);

/* ---------------------------------------------------------------------
 * Diagnostics on the device (replaces the host accumulation loop,
 * pyqg/model.py:802-814): pqg_diag_accumulate adds one step's value of a
 * built-in diagnostic to a device FP64 accumulator (acc += value), with the
 * formulas of pyqg/model.py:640-760, pyqg/qg_diagnostics.py,
 * pyqg/qg_model.py:231-263 and pyqg/layered_model.py:261-300.
 * Accumulator shapes: (nz, nl, nk) for ENSSPEC, KESPEC, KESPEC_MODAL;
 * (nz-1, nl, nk) for PESPEC_MODAL; (nz) for EKE; scalar for EKEDISS and
 * APEGEN; (nl, nk) otherwise.  Spectral fields are complex (re, im) device
 * arrays of (nz, nl, nk) (Jptpc: one plane); u, v are physical (nz, ny, nx).
 * Unused fields may be NULL; a missing required field is PQG_ERR_INVALID.
 * --------------------------------------------------------------------- */
#define PQG_DIAG_MAXZ 8
enum {
  PQG_DIAG_ENSSPEC = 0, PQG_DIAG_KESPEC, PQG_DIAG_EKE, PQG_DIAG_EKEDISS,
  PQG_DIAG_KEFRICTIONSPEC, PQG_DIAG_DISSSPEC, PQG_DIAG_ENSDISSSPEC,
  PQG_DIAG_PARAMSPEC, PQG_DIAG_ENSPARAMSPEC, PQG_DIAG_ENTSPEC,
  PQG_DIAG_PARAMSPEC_APEFLUX, PQG_DIAG_PARAMSPEC_KEFLUX, PQG_DIAG_ENSFLUX,
  PQG_DIAG_ENSGENSPEC, PQG_DIAG_ENSFRICTIONSPEC, PQG_DIAG_APEGENSPEC,
  PQG_DIAG_APEFLUX, PQG_DIAG_KEFLUX, PQG_DIAG_APEGEN, PQG_DIAG_KESPEC_MODAL,
  PQG_DIAG_PESPEC_MODAL, PQG_DIAG_APESPEC, PQG_DIAG_KEFLUX_DIV,
  PQG_DIAG_APEFLUX_DIV, PQG_DIAG_COUNT
};
typedef struct pqg_diag_fields {
  const double *qh, *ph, *dqhdt, *dqhdt_p, *dqhdt_pp; /* spectral state  */
  const double *u, *v;                                /* physical        */
  const double *Jq, *Jpxi, *Jptpc, *JSp, *Sph, *phn;  /* derived fields  */
  const double *dqh, *duh, *dvh;                      /* hook outputs    */
  /* host scalars / per-layer arrays */
  double H, dt, c1, c2, c3;        /* depth, dt, AB coefficients of the step */
  double rd, del1, del2, U;        /* two-layer constants                    */
  const double *Hi, *Qx, *Qy, *Ubg, *Vbg, *f2gpi, *kdi2, *S; /* S: nz x nz  */
} pqg_diag_fields;
int pqg_diag_accumulate(pqg_plan *plan, int kind, const pqg_diag_fields *f,
                        double *acc, void *stream);

/* ---------------------------------------------------------------------
 * Learned subgrid closure (no counterpart in the reference): a fully
 * convolutional network of 5x5 periodic convolutions with ReLU between
 * layers, BF16 weights and activations, FP32 accumulation on the tcgen05
 * tensor cores, trained with Adam.  It reaches a model through the
 * q_parameterization hook (pyqg/model.py:203-212, pyqg/kernel.pyx:424-442).
 *
 * Parameters are one FP32 vector: for each layer, weights w[co][ky][kx][ci]
 * followed by biases b[co].  Image arrays are NCHW (batch, channels, ny,
 * nx) device arrays; nx must be 64 and batch * ny * nx a multiple of 128;
 * hidden channel counts are multiples of 8, all counts at most 128.
 * --------------------------------------------------------------------- */
const char *pqg_cnn_last_error(void);
/* channels: nlayers + 1 counts (input, hidden..., output) */
int pqg_cnn_create(pqg_cnn **net, int nlayers, const int *channels, int ny,
                   int nx, int max_batch);
int pqg_cnn_destroy(pqg_cnn *net);
int pqg_cnn_nparams(pqg_cnn *net, long long *n);
/* input / output channels, image size and batch capacity (any may be NULL) */
int pqg_cnn_shape(pqg_cnn *net, int *cin, int *cout, int *ny, int *nx,
                  int *max_batch);
/* host parameter vector in / out (set also resets the Adam moments) */
int pqg_cnn_set_params(pqg_cnn *net, const float *params, void *stream);
int pqg_cnn_get_params(pqg_cnn *net, float *params, void *stream);
int pqg_cnn_get_grads(pqg_cnn *net, float *grads, void *stream);
/* per-channel standardisation used by pqg_cnn_forward (host arrays) */
int pqg_cnn_set_norm(pqg_cnn *net, const float *in_mean, const float *in_std,
                     const float *out_mean, const float *out_std);
/* y = net((x - in_mean) / in_std) * out_std + out_mean; x and y are FP32
 * (flag 0) or FP64 (flag 1) device arrays */
int pqg_cnn_forward(pqg_cnn *net, const void *x, int x_f64, void *y,
                    int y_f64, int batch, void *stream);
/* gradient of the mean squared error of net(x) against t (standardised FP32
 * device arrays) into the gradient vector; the loss before the update is
 * written to *loss (host) if loss is not NULL */
int pqg_cnn_backward(pqg_cnn *net, const float *x, const float *t, int batch,
                     float *loss, void *stream);
/* one Adam update from the gradient vector */
int pqg_cnn_adam(pqg_cnn *net, float lr, float beta1, float beta2, float eps,
                 void *stream);
/* backward + Adam (beta1 0.9, beta2 0.999, eps 1e-8) */
int pqg_cnn_train_step(pqg_cnn *net, const float *x, const float *t,
                       int batch, float lr, float *loss, void *stream);
/* Pipeline status: synchronizes `stream` and returns PQG_ERR_TIMEOUT if a
 * bounded wait of the network's tensor-core pipelines gave up since the
 * last check (forward calls are asynchronous and do not check). */
int pqg_cnn_status(pqg_cnn *net, void *stream);
/* Failure tests (no counterpart in the reference): from pipeline unit
 * `stop_unit` on (< 0: never) the producer of the halo-tile convolutions
 * issues no more copies, so the other warps' bounded waits run out after
 * `wait_ns` (0: one second); the kernel then waits (bounded) for its own
 * MMAs and copies in flight, frees its tensor memory and returns, and the
 * error is reported by pqg_cnn_status. */
int pqg_cnn_set_fault(pqg_cnn *net, int stop_unit, unsigned long long wait_ns);

#ifdef __cplusplus
}
#endif

#endif /* PYQG_GB300_H */
