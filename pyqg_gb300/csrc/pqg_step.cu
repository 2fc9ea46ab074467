// GB300 (sm_103a) FP64 pseudo-spectral time step of pyqg, behind a C ABI.
//
// Data layout in device memory (C order, complex = interleaved double2):
//   physical  (nz, ny, nx) double          q, u, v, uq, vq
//   spectral  (nz, nl, nk) double2         qh, ph, uh, vh, uqh, vqh, dqhdt*
//   mixed     (plane, ny, nk) double2      plan-owned scratch between the row
//             pass (x transforms) and the column pass (y transforms)
//
// A 2-D real transform is split into a row pass (length-nx real FFT of every
// row, done as a length-nx/2 complex FFT plus packing) and a column pass
// (length-ny complex FFT of every column k).  The row pass runs first on the
// forward transform, the column pass first on the inverse, matching
// numpy.fft.rfftn / irfftn axis order.  A whole time step is two kernels:
//   row kernel    C2R of (u, v, q) -> products (u+Ubg)q, vq -> R2C
//   column kernel FFT_y of (uq, vq) -> tendency, drag, filtered AB3 update ->
//                 inversion of the new qh -> IFFT_y of (uh, vh, qh)
// The column kernel runs one CTA per (layer, column); the nz CTAs of a
// column form a thread-block cluster and exchange the per-layer qh values
// the layer coupling needs through distributed shared memory.
// Transform engines (a plan setting): FP64 Stockham transforms, or, the
// default on power-of-two grids, the same transforms in 64-bit block fixed
// point (pqg_fixed.cuh).  The pointwise physics is FP64 under both.
#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/pyqg_gb300.h"
#include "pqg_fft.cuh"
#include "pqg_fixed.cuh"

namespace cg = cooperative_groups;
using namespace pqg;

// ===========================================================================
// error reporting
// ===========================================================================
static thread_local std::string g_last_error;

static int fail(int code, const std::string& msg) {
  g_last_error = msg;
  return code;
}

#define PQG_CUDA(call)                                                    \
  do {                                                                    \
    cudaError_t e_ = (call);                                              \
    if (e_ != cudaSuccess)                                                \
      return fail(PQG_ERR_CUDA, std::string(#call) + ": " +               \
                                    cudaGetErrorString(e_));              \
  } while (0)

// ===========================================================================
// kernel argument blocks
// ===========================================================================
struct Geo {
  int nz, ny, nx, nk, M;  // M = nx / 2
  double scale;           // 1 / (nx * ny)
  FftDesc fx;             // complex length M
  FftDesc fy;             // complex length ny
  const double2* twx;     // nx entries exp(-2 pi i m / nx)
  const double2* twy;     // ny entries exp(-2 pi i m / ny)
};

struct Consts {
  const double* a;      // (nz, nz, nl, nk)
  const double* kk;     // (nk)
  const double* ll;     // (nl)
  const double* k2l2;   // (nl, nk)
  const double* kQy;    // (nz, nk)   kk * Qy
  const double* Ubg;    // (nz)
  const double* filtr;  // (nl, nk)
  double rek;
  int* nonfinite;       // host-mapped flag, set when a new qh value is Inf or NaN
};

// Sets the plan's non-finite flag (host-mapped memory: the host reads it
// without synchronizing) when a new spectral PV value is Inf or NaN.
__device__ __forceinline__ void flag_nonfinite(int* nf, double2 v) {
  if (nf && !(isfinite(v.x) && isfinite(v.y))) *reinterpret_cast<volatile int*>(nf) = 1;
}

// load a twiddle table into shared memory
__device__ __forceinline__ void load_tw(double2* s, const double2* __restrict__ g, int n) {
  for (int i = threadIdx.x; i < n; i += blockDim.x) s[i] = g[i];
}

// ===========================================================================
// ROW PASS
// ===========================================================================
// Row kernel: one CTA handles `rb` consecutive rows r = z*ny + y of all
// fields it touches.  Shared layout: [tw_x (nx)] [field][row][M].
//
// mode ROW_ADV  (advection, reference _do_advection first half, fused step):
//   U, V from mixed (C2R) or physical; Q from mixed (C2R) or physical;
//   optional stores of u, v, q, uq, vq; R2C of uq, vq -> mixed UQ, VQ.
// mode ROW_C2R  (nf fields mixed -> physical)
// mode ROW_R2C  (nf fields physical -> mixed)
struct RowAdvArgs {
  const double2* mixU; const double2* mixV; const double2* mixQ;
  const double* physU; const double* physV; const double* physQ;
  double* outU; double* outV; double* outQ; double* outUQ; double* outVQ;
  double2* mixUQ; double2* mixVQ;
  const double* Ubg;
  int rb;
};

// Programmatic dependent launch: a step kernel lets the next one launch as
// soon as all its CTAs have started (launch_dependents), and waits for the
// previous kernel's completion and memory (wait) after loading constant
// tables and before touching any data the previous kernel wrote or reads.
// Without the launch attribute both are no-ops.
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

template <class FX>
__global__ void k_row_adv(Geo g, RowAdvArgs A) {
  extern __shared__ double2 sm[];
  const int M = g.M, nk = g.nk, nx = g.nx;
  const int nrows = g.nz * g.ny;
  const int r0 = blockIdx.x * A.rb;
  const int rb = min(A.rb, nrows - r0);
  double2* tw = sm;
  double2* bU = sm + nx;
  double2* bV = bU + A.rb * M;
  double2* bQ = bV + A.rb * M;
  load_tw(tw, g.twx, nx);
  pdl_trigger();
  pdl_wait();
  __syncthreads();

  // -- load / C2R pre-processing --------------------------------------------
  const int half = M / 2 + 1;
  for (int t = threadIdx.x; t < 3 * rb * half; t += blockDim.x) {
    const int f = t / (rb * half);
    const int rem = t - f * rb * half;
    const int rr = rem / half, k = rem - rr * half;
    const int r = r0 + rr;
    const double2* mix = f == 0 ? A.mixU : (f == 1 ? A.mixV : A.mixQ);
    const double* phys = f == 0 ? A.physU : (f == 1 ? A.physV : A.physQ);
    double2* b = (f == 0 ? bU : (f == 1 ? bV : bQ)) + rr * M;
    if (mix) {
      c2r_pre(mix + (size_t)r * nk, b, M, k, tw);
    } else {
      const double2* row = reinterpret_cast<const double2*>(phys + (size_t)r * nx);
      // k-th task copies complex slots k and M-1-k
      if (k < M - k) b[k] = row[k];
      if (k < M - k && M - 1 - k != k) b[M - 1 - k] = row[M - 1 - k];
    }
  }
  __syncthreads();

  // -- inverse transforms of the mixed inputs (U, V[, Q] are a prefix) -------
  // Buffers of a field hold A.rb rows; rows past `rb` (last CTA) are unused.
  {
    const int nmix = (A.mixU ? 1 : 0) + (A.mixV ? 1 : 0) + (A.mixQ ? 1 : 0);
    if (nmix) FX::template run<true>(bU, M, nmix * A.rb, g.fx, tw, 2);
  }

  // -- unpack, products, optional stores -------------------------------------
  const double s = g.scale;
  for (int t = threadIdx.x; t < rb * M; t += blockDim.x) {
    const int rr = t / M, m = t - rr * M;
    const int r = r0 + rr;
    const int z = r / g.ny;
    double2 u = bU[rr * M + m], v = bV[rr * M + m], q = bQ[rr * M + m];
    if (A.mixU) u = cscale(u, s);
    if (A.mixV) v = cscale(v, s);
    if (A.mixQ) q = cscale(q, s);
    const size_t po = (size_t)r * nx + 2 * m;
    if (A.outU) *reinterpret_cast<double2*>(A.outU + po) = u;
    if (A.outV) *reinterpret_cast<double2*>(A.outV + po) = v;
    if (A.outQ) *reinterpret_cast<double2*>(A.outQ + po) = q;
    // uq = (u + Ubg) q, vq = v q (pyqg/kernel.pyx:377-378)
    const double ub = A.Ubg[z];
    const double2 uq = make_double2(__dmul_rn(__dadd_rn(u.x, ub), q.x),
                                    __dmul_rn(__dadd_rn(u.y, ub), q.y));
    const double2 vq = make_double2(__dmul_rn(v.x, q.x), __dmul_rn(v.y, q.y));
    if (A.outUQ) *reinterpret_cast<double2*>(A.outUQ + po) = uq;
    if (A.outVQ) *reinterpret_cast<double2*>(A.outVQ + po) = vq;
    bU[rr * M + m] = uq;
    bV[rr * M + m] = vq;
  }
  __syncthreads();

  // -- forward transforms of uq, vq and R2C post-processing -------------------
  FX::template run<false>(bU, M, 2 * A.rb, g.fx, tw, 2);
  for (int t = threadIdx.x; t < 2 * rb * half; t += blockDim.x) {
    const int f = t / (rb * half);
    const int rem = t - f * rb * half;
    const int rr = rem / half, k = rem - rr * half;
    const int r = r0 + rr;
    double2* X = (f == 0 ? A.mixUQ : A.mixVQ) + (size_t)r * nk;
    r2c_post((f == 0 ? bU : bV) + rr * M, X, M, k, tw);
  }
}

// nf planes-of-fields: mixed -> physical (second half of irfft2)
struct RowBatchArgs {
  const double2* mix; double* phys;   // plane-major, nplanes planes
  const double2* mixsrc; const double* physsrc;
  double2* mixdst;
  int nrows;                          // nplanes * ny
  int rb;
};

__global__ void k_row_c2r(Geo g, RowBatchArgs A) {
  extern __shared__ double2 sm[];
  const int M = g.M, nk = g.nk, nx = g.nx;
  const int r0 = blockIdx.x * A.rb;
  const int rb = min(A.rb, A.nrows - r0);
  double2* tw = sm;
  double2* b = sm + nx;
  load_tw(tw, g.twx, nx);
  __syncthreads();
  const int half = M / 2 + 1;
  for (int t = threadIdx.x; t < rb * half; t += blockDim.x) {
    const int rr = t / half, k = t - rr * half;
    c2r_pre(A.mixsrc + (size_t)(r0 + rr) * nk, b + rr * M, M, k, tw);
  }
  __syncthreads();
  fft_run<true>(b, M, rb, g.fx, tw, 2);
  for (int t = threadIdx.x; t < rb * M; t += blockDim.x) {
    const int rr = t / M, m = t - rr * M;
    const double2 x = cscale(b[rr * M + m], g.scale);
    *reinterpret_cast<double2*>(A.phys + (size_t)(r0 + rr) * nx + 2 * m) = x;
  }
}

__global__ void k_row_r2c(Geo g, RowBatchArgs A) {
  extern __shared__ double2 sm[];
  const int M = g.M, nk = g.nk, nx = g.nx;
  const int r0 = blockIdx.x * A.rb;
  const int rb = min(A.rb, A.nrows - r0);
  double2* tw = sm;
  double2* b = sm + nx;
  load_tw(tw, g.twx, nx);
  for (int t = threadIdx.x; t < rb * M; t += blockDim.x) {
    const int rr = t / M, m = t - rr * M;
    b[rr * M + m] = reinterpret_cast<const double2*>(A.physsrc + (size_t)(r0 + rr) * nx)[m];
  }
  __syncthreads();
  fft_run<false>(b, M, rb, g.fx, tw, 2);
  const int half = M / 2 + 1;
  for (int t = threadIdx.x; t < rb * half; t += blockDim.x) {
    const int rr = t / half, k = t - rr * half;
    r2c_post(b + rr * M, A.mixdst + (size_t)(r0 + rr) * nk, M, k, tw);
  }
}

// ===========================================================================
// COLUMN PASS
// ===========================================================================
// One CTA per (plane or layer z = blockIdx.x, column k = blockIdx.y).
// Shared layout: [tw_y (ny)] [sequence][ny].

// column of a (plane, ny, nk) array
__device__ __forceinline__ size_t cidx(int plane, int l, int k, int ny, int nk) {
  return ((size_t)plane * ny + l) * nk + k;
}

// Column engines: how a CTA transforms `nseq` columns of length ny held in
// shared memory (contiguous, stride ny).  ColRT: FP64 Stockham with the
// runtime plan.  ColFx<LOGN>: 64-bit block fixed point (pqg_fixed.cuh).
// `tw` is the shared twiddle table the engine loaded, `ws` 8 shared ints.
struct ColRT {
  static __device__ __forceinline__ void load(void* tw, const Geo& g, const longlong2*) {
    load_tw(reinterpret_cast<double2*>(tw), g.twy, g.ny);
  }
  template <bool INV>
  static __device__ __forceinline__ void run(double2* buf, int nseq, const Geo& g, const void* tw, int*) {
    fft_run<INV>(buf, g.ny, nseq, g.fy, reinterpret_cast<const double2*>(tw), 1);
  }
};

template <int LOGN>
struct ColFx {
  static constexpr int N = 1 << LOGN;
  static constexpr int G = LOGN + 2;   // growth headroom of a length-N transform
  static __device__ __forceinline__ void load(void* tw, const Geo&, const longlong2* twq) {
    longlong2* t = reinterpret_cast<longlong2*>(tw);
    for (int i = threadIdx.x; i < N; i += blockDim.x) t[i] = twq[i];
  }
  template <bool INV>
  static __device__ __forceinline__ void run(double2* buf, int nseq, const Geo&, const void* tw, int* ws) {
    int* ex = ws;
    int* sh = ws + 4;
    fx::seq_max_exp(buf, N, nseq, N, ex);
    if (threadIdx.x < nseq) sh[threadIdx.x] = fx::block_shift(ex[threadIdx.x], G);
    __syncthreads();
    fx::seq_to_fixed(buf, N, nseq, N, sh);
    fx::FPow2Fft<N, 1, INV>::run(reinterpret_cast<longlong2*>(buf), N, nseq,
                             reinterpret_cast<const longlong2*>(tw), 1);
    fx::seq_from_fixed(buf, N, nseq, N, sh, 0);
  }
};

// shared layout of the column kernels: [tw (ny)] [nseq sequences (ny)] [8 ints]
__device__ __forceinline__ int* col_ws(double2* sm, int ny, int nseq) {
  return reinterpret_cast<int*>(sm + (size_t)ny * (1 + nseq));
}

// generic column FFT over planes: spectral <- mixed (forward, rfft2 2nd half)
// or mixed <- spectral (inverse, irfft2 1st half)
template <class CE, bool INV>
__global__ void k_col_batch(Geo g, const double2* __restrict__ src,
                            double2* __restrict__ dst, const longlong2* __restrict__ twq) {
  extern __shared__ double2 sm[];
  const int ny = g.ny, nk = g.nk;
  const int p = blockIdx.x, k = blockIdx.y;
  double2* b = sm + ny;
  CE::load(sm, g, twq);
  for (int l = threadIdx.x; l < ny; l += blockDim.x) b[l] = src[cidx(p, l, k, ny, nk)];
  __syncthreads();
  CE::template run<INV>(b, 1, g, sm, col_ws(sm, ny, 1));
  for (int l = threadIdx.x; l < ny; l += blockDim.x) dst[cidx(p, l, k, ny, nk)] = b[l];
}

// _invert, column part: ph = a qh; uh = -il ph; vh = ik ph (optionally
// stored); inverse y transforms of uh, vh -> mixed U, V.
template <class CE>
__global__ void k_col_invert(Geo g, Consts c, const double2* __restrict__ qh,
                             double2* ph, double2* uh, double2* vh,
                             double2* mixU, double2* mixV, const longlong2* __restrict__ twq) {
  extern __shared__ double2 sm[];
  const int ny = g.ny, nk = g.nk, nz = g.nz;
  const int z = blockIdx.x, k = blockIdx.y;
  double2* bU = sm + ny;
  double2* bV = bU + ny;
  CE::load(sm, g, twq);
  const double kk = c.kk[k];
  for (int l = threadIdx.x; l < ny; l += blockDim.x) {
    double2 p = make_double2(0.0, 0.0);
    for (int z1 = 0; z1 < nz; z1++)
      p = ph_acc(p, c.a[cidx(z * nz + z1, l, k, ny, nk)], qh[cidx(z1, l, k, ny, nk)]);
    const double2 u = uh_of(c.ll[l], p), v = vh_of(kk, p);
    const size_t o = cidx(z, l, k, ny, nk);
    if (ph) ph[o] = p;
    if (uh) uh[o] = u;
    if (vh) vh[o] = v;
    bU[l] = u;
    bV[l] = v;
  }
  __syncthreads();
  CE::template run<true>(bU, 2, g, sm, col_ws(sm, ny, 2));
  for (int l = threadIdx.x; l < ny; l += blockDim.x) {
    mixU[cidx(z, l, k, ny, nk)] = bU[l];
    mixV[cidx(z, l, k, ny, nk)] = bV[l];
  }
}

// _do_advection, column part: y transforms of mixed UQ, VQ -> uqh, vqh
// (optionally stored); dqhdt = -(ik uqh + il vqh + ikQy ph).
template <class CE>
__global__ void k_col_adv(Geo g, Consts c, const double2* __restrict__ mixUQ,
                          const double2* __restrict__ mixVQ,
                          const double2* __restrict__ ph, double2* uqh,
                          double2* vqh, double2* dqhdt, const longlong2* __restrict__ twq) {
  extern __shared__ double2 sm[];
  const int ny = g.ny, nk = g.nk;
  const int z = blockIdx.x, k = blockIdx.y;
  double2* bU = sm + ny;
  double2* bV = bU + ny;
  CE::load(sm, g, twq);
  for (int l = threadIdx.x; l < ny; l += blockDim.x) {
    bU[l] = mixUQ[cidx(z, l, k, ny, nk)];
    bV[l] = mixVQ[cidx(z, l, k, ny, nk)];
  }
  __syncthreads();
  CE::template run<false>(bU, 2, g, sm, col_ws(sm, ny, 2));
  const double kk = c.kk[k], kQy = c.kQy[z * nk + k];
  for (int l = threadIdx.x; l < ny; l += blockDim.x) {
    const size_t o = cidx(z, l, k, ny, nk);
    const double2 a = bU[l], b = bV[l];
    if (uqh) uqh[o] = a;
    if (vqh) vqh[o] = b;
    dqhdt[o] = tendency(kk, c.ll[l], kQy, a, b, ph[o]);
  }
}

// _forward_timestep, column part: filtered AB update of qh (stored), optional
// in-place history shift, inverse y transform of the new qh -> mixed Q.
template <class CE>
__global__ void k_col_ab3(Geo g, Consts c, double2* qh,
                          const double2* __restrict__ dq, double2* dqp,
                          double2* dqpp, double c1, double c2, double c3,
                          int rotate, double2* mixQ, const longlong2* __restrict__ twq) {
  extern __shared__ double2 sm[];
  const int ny = g.ny, nk = g.nk;
  const int z = blockIdx.x, k = blockIdx.y;
  double2* b = sm + ny;
  CE::load(sm, g, twq);
  for (int l = threadIdx.x; l < ny; l += blockDim.x) {
    const size_t o = cidx(z, l, k, ny, nk);
    const double2 d = dq[o], p = dqp[o], pp = dqpp[o];
    const double2 qn = ab_update(c.filtr[(size_t)l * nk + k], qh[o], d, p, pp, c1, c2, c3);
    flag_nonfinite(c.nonfinite, qn);
    qh[o] = qn;
    if (rotate) {
      dqpp[o] = p;
      dqp[o] = d;
    }
    b[l] = qn;
  }
  __syncthreads();
  CE::template run<true>(b, 1, g, sm, col_ws(sm, ny, 1));
  for (int l = threadIdx.x; l < ny; l += blockDim.x) mixQ[cidx(z, l, k, ny, nk)] = b[l];
}

// _do_friction (pyqg/kernel.pyx:447-461), bottom layer only
__global__ void k_friction(Geo g, Consts c, const double2* __restrict__ ph, double2* dqhdt) {
  const int n = g.ny * g.nk;
  const size_t off = (size_t)(g.nz - 1) * n;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const double rk2 = __dmul_rn(c.rek, c.k2l2[i]);
    dqhdt[off + i] = friction(dqhdt[off + i], rk2, ph[off + i]);
  }
}

// dqhdt += dqh (pyqg/kernel.pyx:436-441)
__global__ void k_add_q(Geo g, const double2* __restrict__ dqh, double2* dqhdt) {
  const size_t n = (size_t)g.nz * g.ny * g.nk;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const double2 a = dqhdt[i], b = dqh[i];
    dqhdt[i] = cadd(a, b);
  }
}

// dqhdt += -il duh + ik dvh (pyqg/kernel.pyx:412-421)
__global__ void k_add_uv(Geo g, Consts c, const double2* __restrict__ duh,
                         const double2* __restrict__ dvh, double2* dqhdt) {
  const size_t n = (size_t)g.nz * g.ny * g.nk;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const int k = (int)(i % g.nk);
    const int l = (int)((i / g.nk) % g.ny);
    dqhdt[i] = uv_curl_add(dqhdt[i], c.kk[k], c.ll[l], duh[i], dvh[i]);
  }
}

// products u f and v f of physical planes (pyqg/model.py:546-547)
__global__ void k_products(size_t n, const double* __restrict__ f, const double* __restrict__ u,
                           const double* __restrict__ v, double* __restrict__ uf, double* __restrict__ vf) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const double x = f[i];
    uf[i] = __dmul_rn(u[i], x);
    vf[i] = __dmul_rn(v[i], x);
  }
}

// spectral advective tendency ik A + il B of A = fft(u f), B = fft(v f)
// (pyqg/model.py:553); (0 + ik)(a + ib) = -k b + i k a exactly
__global__ void k_adv_combine(int nplanes, int ny, int nk, const double* __restrict__ kk,
                              const double* __restrict__ ll, const double2* __restrict__ A,
                              const double2* __restrict__ B, double2* __restrict__ out) {
  const size_t n = (size_t)nplanes * ny * nk;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const int k = (int)(i % nk);
    const int l = (int)((i / nk) % ny);
    const double2 a = A[i], b = B[i];
    const double kx = kk[k], ly = ll[l];
    out[i] = make_double2(__dadd_rn(-__dmul_rn(kx, a.y), -__dmul_rn(ly, b.y)),
                          __dadd_rn(__dmul_rn(kx, a.x), __dmul_rn(ly, b.x)));
  }
}

// sharp spectral truncation of (nplanes, nyf, nkf) to (nplanes, nyc, nkc):
// wavenumbers |k| < nxc / 2 and |l| < nyc / 2 are kept (times `scale`, the
// ratio of the grids' point counts, so that physical amplitudes are kept);
// the coarse grid's Nyquist row and column are zero.
__global__ void k_truncate(int nplanes, int nyf, int nkf, const double2* __restrict__ in, int nyc, int nkc,
                           double2* __restrict__ out, double scale) {
  const size_t n = (size_t)nplanes * nyc * nkc;
  const int nyc2 = nyc / 2;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const int k = (int)(i % nkc);
    const int l = (int)((i / nkc) % nyc);
    const size_t pl = i / ((size_t)nkc * nyc);
    double2 v = make_double2(0.0, 0.0);
    if (k < nkc - 1 && l != nyc2) {
      const int lf = l < nyc2 ? l : nyf - (nyc - l);
      const double2 x = in[(pl * nyf + lf) * nkf + k];
      v = make_double2(__dmul_rn(x.x, scale), __dmul_rn(x.y, scale));
    }
    out[i] = v;
  }
}

__global__ void k_csub(size_t n, const double2* __restrict__ a, const double2* __restrict__ b,
                       double2* __restrict__ out) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const double2 x = a[i], y = b[i];
    out[i] = make_double2(__dsub_rn(x.x, y.x), __dsub_rn(x.y, y.y));
  }
}

// ---------------------------------------------------------------------------
// Fused column kernel of one time step.  Grid (nz, nk), cluster (nz, 1, 1):
// the CTA of layer z = cluster rank z handles column k of that layer.
//   1. load mixed UQ, VQ and the current qh of this layer; FFT_y of UQ, VQ
//   2. ph = sum a qh (qh of other layers read from their CTAs' shared memory)
//      tendency + drag (+ optional spectral forcing), filtered AB update
//   3. ph_new = sum a qh_new (other layers via shared memory), uh, vh
//   4. IFFT_y of uh, vh, qh_new -> mixed U, V, Q for the next step
// Mixed UQ/VQ alias mixed U/V: a CTA reads its column before writing it and
// no other CTA touches that column.
struct FusedColArgs {
  double2* qh;                 // in: current, out: new
  const double2* dqp;          // previous tendency
  double2* dqpp;               // tendency before previous (read)
  double2* dqout;              // new tendency (may equal dqpp)
  const double2* forcing;      // optional spectral forcing added to dqhdt
  double2* mixUQ; double2* mixVQ;   // in
  double2* mixU; double2* mixV; double2* mixQ;  // out
  double2* ph; double2* uh; double2* vh; double2* uqh; double2* vqh;  // aux
  double c1, c2, c3;
};

template <class FY>
__global__ void k_col_fused(Geo g, Consts c, FusedColArgs A) {
  extern __shared__ double2 sm[];
  cg::cluster_group cluster = cg::this_cluster();
  const int ny = g.ny, nk = g.nk, nz = g.nz;
  const int z = blockIdx.x, k = blockIdx.y;
  double2* tw = sm;
  double2* bU = sm + ny;      // UQ, later U
  double2* bV = bU + ny;      // VQ, later V
  double2* bQN = bV + ny;     // qh (new) of this layer
  double2* bQO = bQN + ny;    // qh (old) of this layer
  load_tw(tw, g.twy, ny);
  pdl_trigger();
  pdl_wait();
  for (int l = threadIdx.x; l < ny; l += blockDim.x) {
    const size_t o = cidx(z, l, k, ny, nk);
    bU[l] = A.mixUQ[o];
    bV[l] = A.mixVQ[o];
    bQO[l] = A.qh[o];
  }
  __syncthreads();
  FY::template run<false>(bU, ny, 2, g.fy, tw, 1);
  cluster.sync();  // qh(old) of every layer is in shared memory

  const double kk = c.kk[k], kQy = c.kQy[z * nk + k];
  const bool drag = (c.rek != 0.0) && (z == nz - 1);
  for (int l = threadIdx.x; l < ny; l += blockDim.x) {
    const size_t o = cidx(z, l, k, ny, nk);
    double2 p = make_double2(0.0, 0.0);
    for (int z1 = 0; z1 < nz; z1++) {
      const double2* rq = cluster.map_shared_rank(bQO, z1);
      p = ph_acc(p, c.a[cidx(z * nz + z1, l, k, ny, nk)], rq[l]);
    }
    const double2 uqh = bU[l], vqh = bV[l];
    const double ll = c.ll[l];
    if (A.ph) A.ph[o] = p;
    if (A.uh) A.uh[o] = uh_of(ll, p);
    if (A.vh) A.vh[o] = vh_of(kk, p);
    if (A.uqh) A.uqh[o] = uqh;
    if (A.vqh) A.vqh[o] = vqh;
    double2 d = tendency(kk, ll, kQy, uqh, vqh, p);
    if (drag) d = friction(d, __dmul_rn(c.rek, c.k2l2[(size_t)l * nk + k]), p);
    if (A.forcing) d = cadd(d, A.forcing[o]);
    const double2 pv = A.dqp[o], ppv = A.dqpp[o];
    const double2 qn = ab_update(c.filtr[(size_t)l * nk + k], bQO[l], d, pv, ppv, A.c1, A.c2, A.c3);
    flag_nonfinite(c.nonfinite, qn);
    A.qh[o] = qn;
    A.dqout[o] = d;
    bQN[l] = qn;
  }
  cluster.sync();  // qh(new) of every layer is in shared memory

  for (int l = threadIdx.x; l < ny; l += blockDim.x) {
    double2 p = make_double2(0.0, 0.0);
    for (int z1 = 0; z1 < nz; z1++) {
      const double2* rq = cluster.map_shared_rank(bQN, z1);
      p = ph_acc(p, c.a[cidx(z * nz + z1, l, k, ny, nk)], rq[l]);
    }
    bU[l] = uh_of(c.ll[l], p);
    bV[l] = vh_of(kk, p);
  }
  cluster.sync();  // remote reads of bQN done before it is transformed
  FY::template run<true>(bU, ny, 3, g.fy, tw, 1);  // U, V, qh(new): contiguous
  for (int l = threadIdx.x; l < ny; l += blockDim.x) {
    const size_t o = cidx(z, l, k, ny, nk);
    A.mixU[o] = bU[l];
    A.mixV[o] = bV[l];
    A.mixQ[o] = bQN[l];
  }
}

// ===========================================================================
// FIXED-POINT ENGINE (power-of-two grids): the same two fused kernels with
// the transforms in 64-bit block fixed point (pqg_fixed.cuh); all pointwise
// physics stays FP64.
// ===========================================================================

// C2R pre-processing in fixed point from a double half spectrum (shift S).
__device__ __forceinline__ void c2r_pre_fx(const double2* __restrict__ X, longlong2* z, int M, int k,
                                           const longlong2* __restrict__ twq, int S) {
  using namespace fx;
  if (k == 0) {
    const i64 x0 = to_fixed(X[0].x, S), xm = to_fixed(X[M].x, S);
    z[0] = make_longlong2(x0 + xm, x0 - xm);
    return;
  }
  const double2 ad = X[k], bd = X[M - k];
  const longlong2 a = make_longlong2(to_fixed(ad.x, S), to_fixed(ad.y, S));
  const longlong2 b = make_longlong2(to_fixed(bd.x, S), -to_fixed(bd.y, S));
  const longlong2 A = fadd(a, b), B = fsub(a, b);
  const longlong2 D = fcmulc(B, twq[k]);
  z[k] = make_longlong2(A.x - D.y, A.y + D.x);
  if (k != M - k) z[M - k] = make_longlong2(A.x + D.y, D.x - A.y);
}

// R2C post-processing in fixed point, writing the double half spectrum.
// Interior entries are formed as 2X and converted with one more bit of shift.
__device__ __forceinline__ void r2c_post_fx(const longlong2* z, double2* __restrict__ X, int M, int k,
                                            const longlong2* __restrict__ twq, int S) {
  using namespace fx;
  if (k == 0) {
    const longlong2 z0 = z[0];
    X[0] = make_double2(from_fixed(z0.x + z0.y, S), 0.0);
    X[M] = make_double2(from_fixed(z0.x - z0.y, S), 0.0);
    return;
  }
  const longlong2 a = z[k], bb = z[M - k];
  const longlong2 b = make_longlong2(bb.x, -bb.y);
  const longlong2 A = fadd(a, b), B = fsub(a, b);
  const longlong2 C = fcmul(B, twq[k]);
  const int S1 = S == kNanShift ? S : S + 1;
  X[k] = make_double2(from_fixed(A.x + C.y, S1), from_fixed(A.y - C.x, S1));
  if (k != M - k) X[M - k] = make_double2(from_fixed(A.x - C.y, S1), from_fixed(-(A.y + C.x), S1));
}

template <int LOGM>
__global__ void k_row_adv_fx(Geo g, RowAdvArgs A, const longlong2* __restrict__ twq_g, int log2_nxny) {
  using namespace fx;
  constexpr int M = 1 << LOGM;
  constexpr int G_C2R = LOGM + 4;   // growth: packing (3 bits) + length-M transform
  constexpr int G_R2C = LOGM + 4;
  extern __shared__ double2 sm[];
  const int nk = M + 1, nx = 2 * M;
  const int nrows = g.nz * g.ny;
  const int r0 = blockIdx.x * A.rb;
  const int rb = min(A.rb, nrows - r0);
  longlong2* tw = reinterpret_cast<longlong2*>(sm);
  double2* bU = sm + nx;
  double2* bV = bU + A.rb * M;
  double2* bQ = bV + A.rb * M;
  int* ex = reinterpret_cast<int*>(bQ + A.rb * M);
  int* sh = ex + 3 * A.rb;
  for (int i = threadIdx.x; i < nx; i += blockDim.x) tw[i] = twq_g[i];
  pdl_trigger();
  pdl_wait();
  const int nmix = (A.mixU ? 1 : 0) + (A.mixV ? 1 : 0) + (A.mixQ ? 1 : 0);
  for (int i = threadIdx.x; i < 3 * A.rb; i += blockDim.x) ex[i] = 0;
  __syncthreads();
  // block exponents of the mixed half spectra (imaginary parts of k = 0 and
  // k = M are ignored by the C2R and do not count)
  for (int t = threadIdx.x; t < nmix * rb * nk; t += blockDim.x) {
    const int f = t / (rb * nk);
    const int rem = t - f * rb * nk;
    const int rr = rem / nk, k = rem - rr * nk;
    const double2* mix = f == 0 ? A.mixU : (f == 1 ? A.mixV : A.mixQ);
    const double2 v = mix[(size_t)(r0 + rr) * nk + k];
    atomicMax(&ex[f * A.rb + rr], (k == 0 || k == M) ? bexp1(v.x) : bexp(v));
  }
  __syncthreads();
  for (int i = threadIdx.x; i < 3 * A.rb; i += blockDim.x) sh[i] = block_shift(ex[i], G_C2R);
  __syncthreads();
  const int half = M / 2 + 1;
  for (int t = threadIdx.x; t < 3 * rb * half; t += blockDim.x) {
    const int f = t / (rb * half);
    const int rem = t - f * rb * half;
    const int rr = rem / half, k = rem - rr * half;
    const int r = r0 + rr;
    const double2* mix = f == 0 ? A.mixU : (f == 1 ? A.mixV : A.mixQ);
    const double* phys = f == 0 ? A.physU : (f == 1 ? A.physV : A.physQ);
    double2* b = (f == 0 ? bU : (f == 1 ? bV : bQ)) + rr * M;
    if (mix) {
      c2r_pre_fx(mix + (size_t)r * nk, reinterpret_cast<longlong2*>(b), M, k, tw, sh[f * A.rb + rr]);
    } else {
      const double2* row = reinterpret_cast<const double2*>(phys + (size_t)r * nx);
      if (k < M - k) b[k] = row[k];
      if (k < M - k && M - 1 - k != k) b[M - 1 - k] = row[M - 1 - k];
    }
  }
  __syncthreads();
  if (nmix) FPow2Fft<M, 1, true>::run(reinterpret_cast<longlong2*>(bU), M, nmix * A.rb, tw, 2);

  for (int t = threadIdx.x; t < rb * M; t += blockDim.x) {
    const int rr = t / M, m = t - rr * M;
    const int r = r0 + rr;
    const int z = r / g.ny;
    double2 u = bU[rr * M + m], v = bV[rr * M + m], q = bQ[rr * M + m];
    if (A.mixU) {
      const longlong2 f = *reinterpret_cast<const longlong2*>(&bU[rr * M + m]);
      const int S = sh[rr] == kNanShift ? kNanShift : sh[rr] + log2_nxny;
      u = make_double2(from_fixed(f.x, S), from_fixed(f.y, S));
    }
    if (A.mixV) {
      const longlong2 f = *reinterpret_cast<const longlong2*>(&bV[rr * M + m]);
      const int S = sh[A.rb + rr] == kNanShift ? kNanShift : sh[A.rb + rr] + log2_nxny;
      v = make_double2(from_fixed(f.x, S), from_fixed(f.y, S));
    }
    if (A.mixQ) {
      const longlong2 f = *reinterpret_cast<const longlong2*>(&bQ[rr * M + m]);
      const int S = sh[2 * A.rb + rr] == kNanShift ? kNanShift : sh[2 * A.rb + rr] + log2_nxny;
      q = make_double2(from_fixed(f.x, S), from_fixed(f.y, S));
    }
    const size_t po = (size_t)r * nx + 2 * m;
    if (A.outU) *reinterpret_cast<double2*>(A.outU + po) = u;
    if (A.outV) *reinterpret_cast<double2*>(A.outV + po) = v;
    if (A.outQ) *reinterpret_cast<double2*>(A.outQ + po) = q;
    const double ub = A.Ubg[z];
    const double2 uq = make_double2(__dmul_rn(__dadd_rn(u.x, ub), q.x),
                                    __dmul_rn(__dadd_rn(u.y, ub), q.y));
    const double2 vq = make_double2(__dmul_rn(v.x, q.x), __dmul_rn(v.y, q.y));
    if (A.outUQ) *reinterpret_cast<double2*>(A.outUQ + po) = uq;
    if (A.outVQ) *reinterpret_cast<double2*>(A.outVQ + po) = vq;
    bU[rr * M + m] = uq;
    bV[rr * M + m] = vq;
  }
  __syncthreads();
  seq_max_exp(bU, M, 2 * A.rb, M, ex);
  for (int i = threadIdx.x; i < 2 * A.rb; i += blockDim.x) sh[i] = block_shift(ex[i], G_R2C);
  __syncthreads();
  seq_to_fixed(bU, M, 2 * A.rb, M, sh);
  FPow2Fft<M, 1, false>::run(reinterpret_cast<longlong2*>(bU), M, 2 * A.rb, tw, 2);
  for (int t = threadIdx.x; t < 2 * rb * half; t += blockDim.x) {
    const int f = t / (rb * half);
    const int rem = t - f * rb * half;
    const int rr = rem / half, k = rem - rr * half;
    const int r = r0 + rr;
    double2* X = (f == 0 ? A.mixUQ : A.mixVQ) + (size_t)r * nk;
    r2c_post_fx(reinterpret_cast<const longlong2*>((f == 0 ? bU : bV) + rr * M), X, M, k, tw,
                sh[f * A.rb + rr]);
  }
}

// Fixed-point counterparts of k_row_c2r / k_row_r2c: the same block
// exponent rule, packing and transform as k_row_adv_fx, so that results
// match the fused kernels bit for bit.
template <int LOGM>
__global__ void k_row_c2r_fx(Geo g, RowBatchArgs A, const longlong2* __restrict__ twq_g, int log2_nxny) {
  using namespace fx;
  constexpr int M = 1 << LOGM;
  constexpr int G_C2R = LOGM + 4;
  extern __shared__ double2 sm[];
  const int nk = M + 1, nx = 2 * M;
  const int r0 = blockIdx.x * A.rb;
  const int rb = min(A.rb, A.nrows - r0);
  longlong2* tw = reinterpret_cast<longlong2*>(sm);
  double2* b = sm + nx;
  int* ex = reinterpret_cast<int*>(b + A.rb * M);
  int* sh = ex + A.rb;
  for (int i = threadIdx.x; i < nx; i += blockDim.x) tw[i] = twq_g[i];
  for (int i = threadIdx.x; i < A.rb; i += blockDim.x) ex[i] = 0;
  __syncthreads();
  for (int t = threadIdx.x; t < rb * nk; t += blockDim.x) {
    const int rr = t / nk, k = t - rr * nk;
    const double2 v = A.mixsrc[(size_t)(r0 + rr) * nk + k];
    atomicMax(&ex[rr], (k == 0 || k == M) ? bexp1(v.x) : bexp(v));
  }
  __syncthreads();
  for (int i = threadIdx.x; i < A.rb; i += blockDim.x) sh[i] = block_shift(ex[i], G_C2R);
  __syncthreads();
  const int half = M / 2 + 1;
  for (int t = threadIdx.x; t < rb * half; t += blockDim.x) {
    const int rr = t / half, k = t - rr * half;
    c2r_pre_fx(A.mixsrc + (size_t)(r0 + rr) * nk, reinterpret_cast<longlong2*>(b + rr * M), M, k, tw, sh[rr]);
  }
  __syncthreads();
  FPow2Fft<M, 1, true>::run(reinterpret_cast<longlong2*>(b), M, A.rb, tw, 2);
  for (int t = threadIdx.x; t < rb * M; t += blockDim.x) {
    const int rr = t / M, m = t - rr * M;
    const longlong2 f = *reinterpret_cast<const longlong2*>(&b[rr * M + m]);
    const int S = sh[rr] == kNanShift ? kNanShift : sh[rr] + log2_nxny;
    *reinterpret_cast<double2*>(A.phys + (size_t)(r0 + rr) * nx + 2 * m) =
        make_double2(from_fixed(f.x, S), from_fixed(f.y, S));
  }
}

template <int LOGM>
__global__ void k_row_r2c_fx(Geo g, RowBatchArgs A, const longlong2* __restrict__ twq_g) {
  using namespace fx;
  constexpr int M = 1 << LOGM;
  constexpr int G_R2C = LOGM + 4;
  extern __shared__ double2 sm[];
  const int nk = M + 1, nx = 2 * M;
  const int r0 = blockIdx.x * A.rb;
  const int rb = min(A.rb, A.nrows - r0);
  longlong2* tw = reinterpret_cast<longlong2*>(sm);
  double2* b = sm + nx;
  int* ex = reinterpret_cast<int*>(b + A.rb * M);
  int* sh = ex + A.rb;
  for (int i = threadIdx.x; i < nx; i += blockDim.x) tw[i] = twq_g[i];
  for (int t = threadIdx.x; t < A.rb * M; t += blockDim.x) {
    const int rr = t / M, m = t - rr * M;
    b[rr * M + m] = rr < rb ? reinterpret_cast<const double2*>(A.physsrc + (size_t)(r0 + rr) * nx)[m]
                            : make_double2(0.0, 0.0);
  }
  __syncthreads();
  seq_max_exp(b, M, A.rb, M, ex);
  for (int i = threadIdx.x; i < A.rb; i += blockDim.x) sh[i] = block_shift(ex[i], G_R2C);
  __syncthreads();
  seq_to_fixed(b, M, A.rb, M, sh);
  FPow2Fft<M, 1, false>::run(reinterpret_cast<longlong2*>(b), M, A.rb, tw, 2);
  const int half = M / 2 + 1;
  for (int t = threadIdx.x; t < rb * half; t += blockDim.x) {
    const int rr = t / half, k = t - rr * half;
    r2c_post_fx(reinterpret_cast<const longlong2*>(b + rr * M), A.mixdst + (size_t)(r0 + rr) * nk, M, k,
                tw, sh[rr]);
  }
}

template <int LOGN>
__global__ void k_col_fused_fx(Geo g, Consts c, FusedColArgs A, const longlong2* __restrict__ twq_g) {
  using namespace fx;
  constexpr int N = 1 << LOGN;
  extern __shared__ double2 sm[];
  cg::cluster_group cluster = cg::this_cluster();
  const int ny = N, nk = g.nk, nz = g.nz;
  const int z = blockIdx.x, k = blockIdx.y;
  longlong2* tw = reinterpret_cast<longlong2*>(sm);
  double2* bU = sm + ny;      // UQ, later U
  double2* bV = bU + ny;      // VQ, later V
  double2* bQN = bV + ny;     // qh (new) of this layer
  double2* bQO = bQN + ny;    // qh (old) of this layer
  int* ex = reinterpret_cast<int*>(bQO + ny);
  ColFx<LOGN>::load(tw, g, twq_g);
  pdl_trigger();
  pdl_wait();
  for (int l = threadIdx.x; l < ny; l += blockDim.x) {
    const size_t o = cidx(z, l, k, ny, nk);
    bU[l] = A.mixUQ[o];
    bV[l] = A.mixVQ[o];
    bQO[l] = A.qh[o];
  }
  __syncthreads();
  ColFx<LOGN>::template run<false>(bU, 2, g, tw, ex);
  cluster.sync();  // qh(old) of every layer is in shared memory

  const double kk = c.kk[k], kQy = c.kQy[z * nk + k];
  const bool drag = (c.rek != 0.0) && (z == nz - 1);
  for (int l = threadIdx.x; l < ny; l += blockDim.x) {
    const size_t o = cidx(z, l, k, ny, nk);
    double2 p = make_double2(0.0, 0.0);
    for (int z1 = 0; z1 < nz; z1++) {
      const double2* rq = cluster.map_shared_rank(bQO, z1);
      p = ph_acc(p, c.a[cidx(z * nz + z1, l, k, ny, nk)], rq[l]);
    }
    const double2 uqh = bU[l], vqh = bV[l];
    const double ll = c.ll[l];
    if (A.ph) A.ph[o] = p;
    if (A.uh) A.uh[o] = uh_of(ll, p);
    if (A.vh) A.vh[o] = vh_of(kk, p);
    if (A.uqh) A.uqh[o] = uqh;
    if (A.vqh) A.vqh[o] = vqh;
    double2 d = tendency(kk, ll, kQy, uqh, vqh, p);
    if (drag) d = friction(d, __dmul_rn(c.rek, c.k2l2[(size_t)l * nk + k]), p);
    if (A.forcing) d = cadd(d, A.forcing[o]);
    const double2 pv = A.dqp[o], ppv = A.dqpp[o];
    const double2 qn = ab_update(c.filtr[(size_t)l * nk + k], bQO[l], d, pv, ppv, A.c1, A.c2, A.c3);
    flag_nonfinite(c.nonfinite, qn);
    A.qh[o] = qn;
    A.dqout[o] = d;
    bQN[l] = qn;
  }
  cluster.sync();  // qh(new) of every layer is in shared memory

  for (int l = threadIdx.x; l < ny; l += blockDim.x) {
    double2 p = make_double2(0.0, 0.0);
    for (int z1 = 0; z1 < nz; z1++) {
      const double2* rq = cluster.map_shared_rank(bQN, z1);
      p = ph_acc(p, c.a[cidx(z * nz + z1, l, k, ny, nk)], rq[l]);
    }
    bU[l] = uh_of(c.ll[l], p);
    bV[l] = vh_of(kk, p);
  }
  cluster.sync();  // remote reads of bQN done before it is transformed
  ColFx<LOGN>::template run<true>(bU, 3, g, tw, ex);
  for (int l = threadIdx.x; l < ny; l += blockDim.x) {
    const size_t o = cidx(z, l, k, ny, nk);
    A.mixU[o] = bU[l];
    A.mixV[o] = bV[l];
    A.mixQ[o] = bQN[l];
  }
}

// ===========================================================================
// plan
// ===========================================================================
struct GraphEntry {
  std::vector<const void*> key;
  double c[3];
  int nsteps;
  cudaGraphExec_t exec;
};

struct pqg_plan {
  int nz, ny, nx, nk, M;
  FftDesc fx, fy;
  double2* twx = nullptr;
  double2* twy = nullptr;
  double* a = nullptr;
  double* kk = nullptr;
  double* ll = nullptr;
  double* k2l2 = nullptr;
  double* kQy = nullptr;
  double* Ubg = nullptr;
  double* filtr = nullptr;
  double rek = 0.0;
  std::vector<double> h_kk, h_ll, h_Qy;
  bool have_kk = false, have_ll = false, have_qy = false;
  longlong2* twx_q = nullptr;  // Q62 twiddles for the fixed-point engine
  longlong2* twy_q = nullptr;
  int engine = 0;              // 0: FP64 transforms, 1: fixed-point transforms
  int log2_nxny = 0;
  double2* scratch = nullptr;  // mixed planes
  int scratch_planes = 0;
  bool pdl = false;             // programmatic dependent launch of the step kernels (PQG_PDL=1;
                                // measured slower at nx=256: 8.3k vs 10.3k sim-yr/hr)
  double2* work = nullptr;     // planes for advection / coarse-graining temporaries
  int work_planes = 0;
  int T_row = 128, rb = 1, T_col = 256;
  int T_row_batch = 128, rb_batch = 1;
  cudaStream_t cap_stream = nullptr;
  int* nf_host = nullptr;      // non-finite flag (pinned, mapped) and its device address
  int* nf_dev = nullptr;
  std::vector<GraphEntry> graphs;
  bool use_graphs = true;
};

static bool factor(int n, FftDesc& d) {
  d.n = n;
  d.nst = 0;
  d.code = 0;
  int m = n;
  auto push = [&](int r) { d.code |= (unsigned long long)r << (4 * d.nst); d.nst++; m /= r; };
  // power-of-two part: radix 8 where possible, radix 4 instead of a final
  // radix 2 (radix 2 costs more FP64 operations per point), then 3 and 5
  int a = 0;
  while (m % 2 == 0) { m /= 2; a++; }
  m = n;
  int eights = pow2_eights(a), fours = pow2_fours(a);
  int twos = a - 3 * eights - 2 * fours;
  if (const char* e = getenv("PQG_RADIX4")) {  // tuning: radix 4/2 only
    if (e[0] == '1') { eights = 0; fours = a / 2; twos = a % 2; }
  }
  for (int i = 0; i < eights && d.nst < kMaxStages; i++) push(8);
  for (int i = 0; i < fours && d.nst < kMaxStages; i++) push(4);
  for (int i = 0; i < twos && d.nst < kMaxStages; i++) push(2);
  while (m % 3 == 0 && d.nst < kMaxStages) push(3);
  while (m % 5 == 0 && d.nst < kMaxStages) push(5);
  return m == 1;
}

// Smallest block size for which every Stockham stage of `d` fits:
// blockDim * MaxIt<R> >= n / R.
static int min_threads(const FftDesc& d) {
  int t = 1;
  for (int s = 0; s < d.nst; s++) {
    const int r = d.radix(s);
    const int it = r == 2 ? MaxIt<2>::value : r == 3 ? MaxIt<3>::value : r == 4 ? MaxIt<4>::value
                 : r == 5 ? MaxIt<5>::value : MaxIt<8>::value;
    const int nb = d.n / r;
    t = std::max(t, (nb + it - 1) / it);
  }
  return t;
}

// cos and sin of 2 pi m / n in long double, with the angle folded into
// [0, pi/4] so that the tables are accurate to the last bit in practice.
static void cos_sin_ld(int n, int m, long double& cr, long double& sr) {
  const long double pi = 3.141592653589793238462643383279502884L;
  long long num = 8LL * m;          // angle = 2 pi m / n = (pi/4) * (8m/n)
  long long oct = num / n;          // octant 0..7
  long long rem = num - oct * n;    // angle within octant = (pi/4) rem / n
  long double x = pi / 4 * (long double)rem / (long double)n;
  long double c = cosl(x), s = sinl(x);
  switch (oct) {
    case 0: cr = c; sr = s; break;
    case 1: { long double y = pi / 4 - x; cr = sinl(y); sr = cosl(y); break; }
    case 2: cr = -s; sr = c; break;
    case 3: { long double y = pi / 4 - x; cr = -cosl(y); sr = sinl(y); break; }
    case 4: cr = -c; sr = -s; break;
    case 5: { long double y = pi / 4 - x; cr = -sinl(y); sr = -cosl(y); break; }
    case 6: cr = s; sr = -c; break;
    default: { long double y = pi / 4 - x; cr = cosl(y); sr = -sinl(y); break; }
  }
}

// exp(-2 pi i m / n) for m = 0..n-1 (FP64 table)
static void twiddles(int n, std::vector<double2>& w) {
  w.resize(n);
  for (int m = 0; m < n; m++) {
    long double cr, sr;
    cos_sin_ld(n, m, cr, sr);
    w[m] = make_double2((double)cr, -(double)sr);
  }
}

// the same table as Q62 integers (round(2^62 cos), round(-2^62 sin))
static void twiddles_q62(int n, std::vector<longlong2>& w) {
  w.resize(n);
  const long double one = 4611686018427387904.0L;  // 2^62
  for (int m = 0; m < n; m++) {
    long double cr, sr;
    cos_sin_ld(n, m, cr, sr);
    w[m] = make_longlong2(llroundl(cr * one), llroundl(-sr * one));
  }
}

static size_t row_adv_smem(const pqg_plan* p, int rb) {
  return sizeof(double2) * ((size_t)p->nx + 3 * (size_t)rb * p->M);
}
static size_t row_batch_smem(const pqg_plan* p, int rb) {
  return sizeof(double2) * ((size_t)p->nx + (size_t)rb * p->M);
}
static size_t col_smem(const pqg_plan* p, int nseq) {
  return sizeof(double2) * ((size_t)p->ny * (1 + nseq)) + 8 * sizeof(int);
}

static Geo geo(const pqg_plan* p) {
  Geo g;
  g.nz = p->nz; g.ny = p->ny; g.nx = p->nx; g.nk = p->nk; g.M = p->M;
  g.scale = 1.0 / ((double)p->nx * (double)p->ny);
  g.fx = p->fx; g.fy = p->fy;
  g.twx = p->twx; g.twy = p->twy;
  return g;
}
static Consts consts(const pqg_plan* p) {
  Consts c;
  c.a = p->a; c.kk = p->kk; c.ll = p->ll; c.k2l2 = p->k2l2; c.kQy = p->kQy;
  c.Ubg = p->Ubg; c.filtr = p->filtr; c.rek = p->rek;
  c.nonfinite = p->nf_dev;
  return c;
}

static int ensure_scratch(pqg_plan* p, int planes) {
  if (planes <= p->scratch_planes) return PQG_OK;
  if (p->scratch) return fail(PQG_ERR_STATE, "scratch already allocated");
  const size_t bytes = sizeof(double2) * (size_t)planes * p->ny * p->nk;
  if (cudaMalloc(&p->scratch, bytes) != cudaSuccess)
    return fail(PQG_ERR_NOMEM, "cudaMalloc scratch failed");
  p->scratch_planes = planes;
  return PQG_OK;
}

// work planes are grown on demand (between calls; never inside a capture)
static int ensure_work(pqg_plan* p, int planes) {
  if (planes <= p->work_planes) return PQG_OK;
  cudaFree(p->work);
  p->work = nullptr;
  p->work_planes = 0;
  const size_t bytes = sizeof(double2) * (size_t)planes * p->ny * p->nk;
  if (cudaMalloc(&p->work, bytes) != cudaSuccess) return fail(PQG_ERR_NOMEM, "cudaMalloc work planes failed");
  p->work_planes = planes;
  return PQG_OK;
}

static void drop_graphs(pqg_plan* p) {
  for (auto& e : p->graphs) cudaGraphExecDestroy(e.exec);
  p->graphs.clear();
}

static double2* dc(double* x) { return reinterpret_cast<double2*>(x); }
static const double2* dc(const double* x) { return reinterpret_cast<const double2*>(x); }

#define CHECK_LAUNCH() PQG_CUDA(cudaGetLastError())

// ---------------------------------------------------------------------------
// kernel selection: compile-time power-of-two plans for the hot kernels
// ---------------------------------------------------------------------------
typedef void (*RowAdvFn)(Geo, RowAdvArgs);
typedef void (*ColFusedFn)(Geo, Consts, FusedColArgs);

static bool is_pow2(int n) { return n > 0 && (n & (n - 1)) == 0; }

static RowAdvFn row_adv_kernel(int M) {
  if (is_pow2(M) && !getenv("PQG_GENERIC_FFT")) {
    switch (ilog2(M)) {
      case 3: return k_row_adv<FftPow2<3>>;
      case 4: return k_row_adv<FftPow2<4>>;
      case 5: return k_row_adv<FftPow2<5>>;
      case 6: return k_row_adv<FftPow2<6>>;
      case 7: return k_row_adv<FftPow2<7>>;
      case 8: return k_row_adv<FftPow2<8>>;
      case 9: return k_row_adv<FftPow2<9>>;
      case 10: return k_row_adv<FftPow2<10>>;
      default: break;
    }
  }
  return k_row_adv<FftRuntime>;
}

static ColFusedFn col_fused_kernel(int ny) {
  if (is_pow2(ny) && !getenv("PQG_GENERIC_FFT")) {
    switch (ilog2(ny)) {
      case 4: return k_col_fused<FftPow2<4>>;
      case 5: return k_col_fused<FftPow2<5>>;
      case 6: return k_col_fused<FftPow2<6>>;
      case 7: return k_col_fused<FftPow2<7>>;
      case 8: return k_col_fused<FftPow2<8>>;
      case 9: return k_col_fused<FftPow2<9>>;
      case 10: return k_col_fused<FftPow2<10>>;
      default: break;
    }
  }
  return k_col_fused<FftRuntime>;
}

typedef void (*RowAdvFxFn)(Geo, RowAdvArgs, const longlong2*, int);
typedef void (*ColFusedFxFn)(Geo, Consts, FusedColArgs, const longlong2*);

static RowAdvFxFn row_adv_fx_kernel(int M) {
  switch (is_pow2(M) ? ilog2(M) : -1) {
    case 3: return k_row_adv_fx<3>;
    case 4: return k_row_adv_fx<4>;
    case 5: return k_row_adv_fx<5>;
    case 6: return k_row_adv_fx<6>;
    case 7: return k_row_adv_fx<7>;
    case 8: return k_row_adv_fx<8>;
    case 9: return k_row_adv_fx<9>;
    case 10: return k_row_adv_fx<10>;
    default: return nullptr;
  }
}

static ColFusedFxFn col_fused_fx_kernel(int ny) {
  switch (is_pow2(ny) ? ilog2(ny) : -1) {
    case 4: return k_col_fused_fx<4>;
    case 5: return k_col_fused_fx<5>;
    case 6: return k_col_fused_fx<6>;
    case 7: return k_col_fused_fx<7>;
    case 8: return k_col_fused_fx<8>;
    case 9: return k_col_fused_fx<9>;
    case 10: return k_col_fused_fx<10>;
    default: return nullptr;
  }
}

typedef void (*ColBatchFn)(Geo, const double2*, double2*, const longlong2*);
typedef void (*ColInvertFn)(Geo, Consts, const double2*, double2*, double2*, double2*, double2*, double2*,
                            const longlong2*);
typedef void (*ColAdvFn)(Geo, Consts, const double2*, const double2*, const double2*, double2*, double2*,
                         double2*, const longlong2*);
typedef void (*ColAb3Fn)(Geo, Consts, double2*, const double2*, double2*, double2*, double, double, double, int,
                         double2*, const longlong2*);
typedef void (*RowC2rFxFn)(Geo, RowBatchArgs, const longlong2*, int);
typedef void (*RowR2cFxFn)(Geo, RowBatchArgs, const longlong2*);

#define PQG_LOGN_CASES(X) X(4) X(5) X(6) X(7) X(8) X(9) X(10)
#define PQG_LOGM_CASES(X) X(3) X(4) X(5) X(6) X(7) X(8) X(9) X(10)

// The plan's engine selects every column transform: FP64 with the runtime
// plan, or fixed point with the compile-time plan of length ny.
template <bool INV>
static ColBatchFn col_batch_kernel(int engine, int ny) {
  if (engine == 1) switch (ilog2(ny)) {
#define C(L) case L: return k_col_batch<ColFx<L>, INV>;
      PQG_LOGN_CASES(C)
#undef C
    }
  return k_col_batch<ColRT, INV>;
}
static ColInvertFn col_invert_kernel(int engine, int ny) {
  if (engine == 1) switch (ilog2(ny)) {
#define C(L) case L: return k_col_invert<ColFx<L>>;
      PQG_LOGN_CASES(C)
#undef C
    }
  return k_col_invert<ColRT>;
}
static ColAdvFn col_adv_kernel(int engine, int ny) {
  if (engine == 1) switch (ilog2(ny)) {
#define C(L) case L: return k_col_adv<ColFx<L>>;
      PQG_LOGN_CASES(C)
#undef C
    }
  return k_col_adv<ColRT>;
}
static ColAb3Fn col_ab3_kernel(int engine, int ny) {
  if (engine == 1) switch (ilog2(ny)) {
#define C(L) case L: return k_col_ab3<ColFx<L>>;
      PQG_LOGN_CASES(C)
#undef C
    }
  return k_col_ab3<ColRT>;
}
static RowC2rFxFn row_c2r_fx_kernel(int M) {
  switch (is_pow2(M) ? ilog2(M) : -1) {
#define C(L) case L: return k_row_c2r_fx<L>;
    PQG_LOGM_CASES(C)
#undef C
    default: return nullptr;
  }
}
static RowR2cFxFn row_r2c_fx_kernel(int M) {
  switch (is_pow2(M) ? ilog2(M) : -1) {
#define C(L) case L: return k_row_r2c_fx<L>;
    PQG_LOGM_CASES(C)
#undef C
    default: return nullptr;
  }
}

// ---------------------------------------------------------------------------
// launch helpers (stage kernels)
// ---------------------------------------------------------------------------
static int launch_row_adv(pqg_plan* p, const RowAdvArgs& A0, cudaStream_t st) {
  RowAdvArgs A = A0;
  A.rb = p->rb;
  A.Ubg = p->Ubg;
  const int nrows = p->nz * p->ny;
  const int grid = (nrows + A.rb - 1) / A.rb;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid, 1, 1);
  cfg.blockDim = dim3(p->T_row, 1, 1);
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = p->pdl ? 1 : 0;
  if (p->engine == 1) {
    cfg.dynamicSmemBytes = row_adv_smem(p, A.rb) + sizeof(int) * 6 * A.rb;
    PQG_CUDA(cudaLaunchKernelEx(&cfg, row_adv_fx_kernel(p->M), geo(p), A, (const longlong2*)p->twx_q,
                                p->log2_nxny));
  } else {
    cfg.dynamicSmemBytes = row_adv_smem(p, A.rb);
    PQG_CUDA(cudaLaunchKernelEx(&cfg, row_adv_kernel(p->M), geo(p), A));
  }
  CHECK_LAUNCH();
  return PQG_OK;
}

static int launch_row_c2r(pqg_plan* p, const double2* mix, double* phys, int nplanes, cudaStream_t st,
                          int engine) {
  RowBatchArgs A{};
  A.mixsrc = mix;
  A.phys = phys;
  A.nrows = nplanes * p->ny;
  A.rb = p->rb_batch;
  const int grid = (A.nrows + A.rb - 1) / A.rb;
  if (engine == 1) {
    const size_t smem = row_batch_smem(p, A.rb) + sizeof(int) * 2 * A.rb;
    row_c2r_fx_kernel(p->M)<<<grid, p->T_row_batch, smem, st>>>(geo(p), A, p->twx_q, p->log2_nxny);
  } else {
    k_row_c2r<<<grid, p->T_row_batch, row_batch_smem(p, A.rb), st>>>(geo(p), A);
  }
  CHECK_LAUNCH();
  return PQG_OK;
}

static int launch_row_r2c(pqg_plan* p, const double* phys, double2* mix, int nplanes, cudaStream_t st,
                          int engine) {
  RowBatchArgs A{};
  A.physsrc = phys;
  A.mixdst = mix;
  A.nrows = nplanes * p->ny;
  A.rb = p->rb_batch;
  const int grid = (A.nrows + A.rb - 1) / A.rb;
  if (engine == 1) {
    const size_t smem = row_batch_smem(p, A.rb) + sizeof(int) * 2 * A.rb;
    row_r2c_fx_kernel(p->M)<<<grid, p->T_row_batch, smem, st>>>(geo(p), A, p->twx_q);
  } else {
    k_row_r2c<<<grid, p->T_row_batch, row_batch_smem(p, A.rb), st>>>(geo(p), A);
  }
  CHECK_LAUNCH();
  return PQG_OK;
}

template <bool INV>
static int launch_col_batch(pqg_plan* p, const double2* src, double2* dst, int nplanes, cudaStream_t st,
                            int engine) {
  dim3 grid(nplanes, p->nk);
  col_batch_kernel<INV>(engine, p->ny)<<<grid, p->T_col, col_smem(p, 1), st>>>(geo(p), src, dst, p->twy_q);
  CHECK_LAUNCH();
  return PQG_OK;
}

static int launch_col_fused(pqg_plan* p, const FusedColArgs& A, cudaStream_t st) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(p->nz, p->nk, 1);
  cfg.blockDim = dim3(p->T_col, 1, 1);
  cfg.dynamicSmemBytes = col_smem(p, 4);
  cfg.stream = st;
  cudaLaunchAttribute attr[2];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = p->nz;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  attr[1].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[1].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = p->pdl ? 2 : 1;
  if (p->engine == 1) {
    cfg.dynamicSmemBytes = col_smem(p, 4) + sizeof(int) * 8;
    PQG_CUDA(cudaLaunchKernelEx(&cfg, col_fused_fx_kernel(p->ny), geo(p), consts(p), A, (const longlong2*)p->twy_q));
  } else {
    PQG_CUDA(cudaLaunchKernelEx(&cfg, col_fused_kernel(p->ny), geo(p), consts(p), A));
  }
  return PQG_OK;
}

static void ab_coeffs(int ablevel, double dt, double& c1, double& c2, double& c3) {
  // pyqg/kernel.pyx:479-495
  if (ablevel <= 0) { c1 = dt; c2 = 0.0; c3 = 0.0; }
  else if (ablevel == 1) { c1 = 1.5 * dt; c2 = -0.5 * dt; c3 = 0.0; }
  else { c1 = 23. / 12. * dt; c2 = -16. / 12. * dt; c3 = 5. / 12. * dt; }
}

// cudaFuncSetAttribute acts on the current device only, so the limits are
// raised once per device ordinal (under a lock: plans may be created from
// several host threads).
static std::mutex g_smem_mutex;
static bool g_smem_done[64];

static int set_smem_limits_current();

static int set_smem_limits() {
  int dev = 0;
  PQG_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) return fail(PQG_ERR_UNSUPPORTED, "device ordinal out of range");
  std::lock_guard<std::mutex> lock(g_smem_mutex);
  if (g_smem_done[dev]) return PQG_OK;
  const int rc = set_smem_limits_current();
  if (rc == PQG_OK) g_smem_done[dev] = true;
  return rc;
}

static int set_smem_limits_current() {
  const int big = 200 * 1024;
  for (int m = 8; m <= 1024; m *= 2)
    PQG_CUDA(cudaFuncSetAttribute(row_adv_kernel(m), cudaFuncAttributeMaxDynamicSharedMemorySize, big));
  PQG_CUDA(cudaFuncSetAttribute(row_adv_kernel(3), cudaFuncAttributeMaxDynamicSharedMemorySize, big));
  PQG_CUDA(cudaFuncSetAttribute(k_row_c2r, cudaFuncAttributeMaxDynamicSharedMemorySize, big));
  PQG_CUDA(cudaFuncSetAttribute(k_row_r2c, cudaFuncAttributeMaxDynamicSharedMemorySize, big));
  for (int engine = 0; engine < 2; engine++)
    for (int n = 16; n <= 1024; n *= 2) {
      PQG_CUDA(cudaFuncSetAttribute(col_batch_kernel<true>(engine, n), cudaFuncAttributeMaxDynamicSharedMemorySize, big));
      PQG_CUDA(cudaFuncSetAttribute(col_batch_kernel<false>(engine, n), cudaFuncAttributeMaxDynamicSharedMemorySize, big));
      PQG_CUDA(cudaFuncSetAttribute(col_invert_kernel(engine, n), cudaFuncAttributeMaxDynamicSharedMemorySize, big));
      PQG_CUDA(cudaFuncSetAttribute(col_adv_kernel(engine, n), cudaFuncAttributeMaxDynamicSharedMemorySize, big));
      PQG_CUDA(cudaFuncSetAttribute(col_ab3_kernel(engine, n), cudaFuncAttributeMaxDynamicSharedMemorySize, big));
    }
  for (int m = 8; m <= 1024; m *= 2) {
    PQG_CUDA(cudaFuncSetAttribute(row_c2r_fx_kernel(m), cudaFuncAttributeMaxDynamicSharedMemorySize, big));
    PQG_CUDA(cudaFuncSetAttribute(row_r2c_fx_kernel(m), cudaFuncAttributeMaxDynamicSharedMemorySize, big));
  }
  for (int n = 16; n <= 1024; n *= 2) {
    PQG_CUDA(cudaFuncSetAttribute(col_fused_kernel(n), cudaFuncAttributeMaxDynamicSharedMemorySize, big));
    PQG_CUDA(cudaFuncSetAttribute(col_fused_kernel(n), cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
  }
  for (int m = 8; m <= 1024; m *= 2)
    PQG_CUDA(cudaFuncSetAttribute(row_adv_fx_kernel(m), cudaFuncAttributeMaxDynamicSharedMemorySize, big));
  for (int n = 16; n <= 1024; n *= 2) {
    PQG_CUDA(cudaFuncSetAttribute(col_fused_fx_kernel(n), cudaFuncAttributeMaxDynamicSharedMemorySize, big));
    PQG_CUDA(cudaFuncSetAttribute(col_fused_fx_kernel(n), cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
  }
  PQG_CUDA(cudaFuncSetAttribute(col_fused_kernel(3), cudaFuncAttributeMaxDynamicSharedMemorySize, big));
  PQG_CUDA(cudaFuncSetAttribute(col_fused_kernel(3), cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
  return PQG_OK;
}

// ===========================================================================
// C ABI
// ===========================================================================
#define PQG_API __attribute__((visibility("default")))

extern "C" {

PQG_API int pqg_version(void) { return 100; }

PQG_API const char* pqg_last_error(void) { return g_last_error.c_str(); }

// error status for the library's other translation units (not part of the C API)
int pqg_report_error(int code, const char* msg) { return fail(code, msg); }

PQG_API int pqg_plan_create(pqg_plan** out, int nz, int ny, int nx) {
  if (!out) return fail(PQG_ERR_INVALID, "plan output pointer is NULL");
  *out = nullptr;
  if (nz < 1 || ny < 2 || nx < 2) return fail(PQG_ERR_INVALID, "grid sizes must be positive");
  if (nx % 2 || ny % 2) return fail(PQG_ERR_UNSUPPORTED, "nx and ny must be even");
  if (nx / 2 > 2048 || ny > 2048) return fail(PQG_ERR_UNSUPPORTED, "nx/2 and ny must be <= 2048");
  if (nz > 8) return fail(PQG_ERR_UNSUPPORTED, "nz must be <= 8");
  pqg_plan* p = new pqg_plan();
  p->nz = nz; p->ny = ny; p->nx = nx; p->nk = nx / 2 + 1; p->M = nx / 2;
  if (!factor(p->M, p->fx) || !factor(ny, p->fy)) {
    delete p;
    return fail(PQG_ERR_UNSUPPORTED, "nx/2 and ny must factor into 2, 3 and 5");
  }
  if (col_smem(p, 4) > 200 * 1024 || row_adv_smem(p, 1) > 200 * 1024) {
    delete p;
    return fail(PQG_ERR_UNSUPPORTED, "grid too large for the shared-memory kernels");
  }
  // block shapes: the Stockham stages need blockDim * MaxIt >= n / R
  p->T_col = std::max(64, std::min(256, ny));
  p->T_row = std::max(64, std::min(256, p->M));
  if (p->T_col < min_threads(p->fy)) p->T_col = std::min(1024, (min_threads(p->fy) + 31) / 32 * 32);
  if (p->T_row < min_threads(p->fx)) p->T_row = std::min(1024, (min_threads(p->fx) + 31) / 32 * 32);
  p->rb = std::max(1, std::min(4, 128 / p->M));
  p->T_row_batch = p->T_row;
  p->rb_batch = std::max(1, std::min(8, 256 / p->M));
  // tuning overrides (block shapes only; results do not depend on them)
  if (const char* e = getenv("PQG_T_ROW")) p->T_row = atoi(e);
  if (const char* e = getenv("PQG_RB")) p->rb = atoi(e);
  if (const char* e = getenv("PQG_T_COL")) p->T_col = atoi(e);
  if (p->T_col < min_threads(p->fy) || p->T_row < min_threads(p->fx) || p->rb < 1 ||
      p->T_row > 1024 || p->T_col > 1024) {
    delete p;
    return fail(PQG_ERR_UNSUPPORTED, "transform too long for the block size");
  }
  if (const char* e = getenv("PQG_NO_GRAPHS")) p->use_graphs = (e[0] == '0');
  if (const char* e = getenv("PQG_PDL")) p->pdl = (e[0] == '1');
  int rc = set_smem_limits();
  if (rc) { delete p; return rc; }

  std::vector<double2> w;
  const size_t nl = ny, nk = p->nk;
  auto alloc = [&](void** ptr, size_t bytes) {
    return cudaMalloc(ptr, bytes) == cudaSuccess && cudaMemset(*ptr, 0, bytes) == cudaSuccess;
  };
  bool ok = alloc((void**)&p->twx, sizeof(double2) * nx) &&
            alloc((void**)&p->twy, sizeof(double2) * ny) &&
            alloc((void**)&p->a, sizeof(double) * nz * nz * nl * nk) &&
            alloc((void**)&p->kk, sizeof(double) * nk) &&
            alloc((void**)&p->ll, sizeof(double) * nl) &&
            alloc((void**)&p->k2l2, sizeof(double) * nl * nk) &&
            alloc((void**)&p->kQy, sizeof(double) * nz * nk) &&
            alloc((void**)&p->Ubg, sizeof(double) * nz) &&
            alloc((void**)&p->filtr, sizeof(double) * nl * nk);
  if (!ok) { pqg_plan_destroy(p); return fail(PQG_ERR_NOMEM, "cudaMalloc failed in plan_create"); }
  twiddles(nx, w);
  cudaMemcpy(p->twx, w.data(), sizeof(double2) * nx, cudaMemcpyHostToDevice);
  twiddles(ny, w);
  cudaMemcpy(p->twy, w.data(), sizeof(double2) * ny, cudaMemcpyHostToDevice);
  // fixed-point engine: power-of-two grids within the compiled plans
  if (is_pow2(nx) && is_pow2(ny) && row_adv_fx_kernel(p->M) && col_fused_fx_kernel(ny) &&
      row_c2r_fx_kernel(p->M) && row_r2c_fx_kernel(p->M)) {
    std::vector<longlong2> wq;
    ok = alloc((void**)&p->twx_q, sizeof(longlong2) * nx) && alloc((void**)&p->twy_q, sizeof(longlong2) * ny);
    if (!ok) { pqg_plan_destroy(p); return fail(PQG_ERR_NOMEM, "cudaMalloc failed in plan_create"); }
    twiddles_q62(nx, wq);
    cudaMemcpy(p->twx_q, wq.data(), sizeof(longlong2) * nx, cudaMemcpyHostToDevice);
    twiddles_q62(ny, wq);
    cudaMemcpy(p->twy_q, wq.data(), sizeof(longlong2) * ny, cudaMemcpyHostToDevice);
    p->log2_nxny = ilog2(nx) + ilog2(ny);
  }
  rc = ensure_scratch(p, 5 * nz);
  if (rc) { pqg_plan_destroy(p); return rc; }
  if (cudaStreamCreateWithFlags(&p->cap_stream, cudaStreamNonBlocking) != cudaSuccess) {
    pqg_plan_destroy(p);
    return fail(PQG_ERR_CUDA, "cudaStreamCreate failed");
  }
  if (cudaHostAlloc((void**)&p->nf_host, sizeof(int), cudaHostAllocMapped) != cudaSuccess ||
      cudaHostGetDevicePointer((void**)&p->nf_dev, p->nf_host, 0) != cudaSuccess) {
    pqg_plan_destroy(p);
    return fail(PQG_ERR_NOMEM, "mapped host flag allocation failed");
  }
  *p->nf_host = 0;
  PQG_CUDA(cudaDeviceSynchronize());
  *out = p;
  return PQG_OK;
}

PQG_API int pqg_nonfinite(const pqg_plan* p, int* flag) {
  if (!p || !flag) return fail(PQG_ERR_INVALID, "NULL argument to pqg_nonfinite");
  *flag = *reinterpret_cast<volatile const int*>(p->nf_host);
  return PQG_OK;
}

PQG_API int pqg_clear_nonfinite(pqg_plan* p) {
  if (!p) return fail(PQG_ERR_INVALID, "NULL plan");
  *reinterpret_cast<volatile int*>(p->nf_host) = 0;
  return PQG_OK;
}

PQG_API int pqg_plan_destroy(pqg_plan* p) {
  if (!p) return PQG_OK;
  drop_graphs(p);
  cudaFree(p->twx); cudaFree(p->twy); cudaFree(p->a); cudaFree(p->kk);
  cudaFree(p->ll); cudaFree(p->k2l2); cudaFree(p->kQy); cudaFree(p->Ubg);
  cudaFree(p->filtr); cudaFree(p->scratch); cudaFree(p->twx_q); cudaFree(p->twy_q);
  cudaFree(p->work);
  if (p->cap_stream) cudaStreamDestroy(p->cap_stream);
  if (p->nf_host) cudaFreeHost(p->nf_host);
  delete p;
  return PQG_OK;
}

static int upload(double* dst, const double* src, size_t n) {
  PQG_CUDA(cudaMemcpy(dst, src, sizeof(double) * n, cudaMemcpyHostToDevice));
  return PQG_OK;
}

static int refresh_kqy(pqg_plan* p) {
  if (!(p->have_kk && p->have_qy)) return PQG_OK;
  std::vector<double> t((size_t)p->nz * p->nk);
  for (int z = 0; z < p->nz; z++)
    for (int i = 0; i < p->nk; i++) t[(size_t)z * p->nk + i] = p->h_kk[i] * p->h_Qy[z];
  return upload(p->kQy, t.data(), t.size());
}

PQG_API int pqg_set_wavenumbers(pqg_plan* p, const double* kk, const double* ll) {
  if (!p || !kk || !ll) return fail(PQG_ERR_INVALID, "NULL argument");
  drop_graphs(p);
  p->h_kk.assign(kk, kk + p->nk);
  p->h_ll.assign(ll, ll + p->ny);
  p->have_kk = p->have_ll = true;
  int rc = upload(p->kk, kk, p->nk);
  if (!rc) rc = upload(p->ll, ll, p->ny);
  if (rc) return rc;
  // k2l2 = kk^2 + ll^2 (pyqg/kernel.pyx:544-546), evaluated without
  // contraction (the library is built with -ffp-contract=off)
  std::vector<double> t((size_t)p->ny * p->nk);
  for (int j = 0; j < p->ny; j++)
    for (int i = 0; i < p->nk; i++) {
      const double a = kk[i] * kk[i];
      const double b = ll[j] * ll[j];
      t[(size_t)j * p->nk + i] = a + b;
    }
  rc = upload(p->k2l2, t.data(), t.size());
  if (rc) return rc;
  return refresh_kqy(p);
}

PQG_API int pqg_set_k2l2(pqg_plan* p, const double* k2l2) {
  if (!p || !k2l2) return fail(PQG_ERR_INVALID, "NULL argument");
  drop_graphs(p);
  return upload(p->k2l2, k2l2, (size_t)p->ny * p->nk);
}

PQG_API int pqg_set_inversion(pqg_plan* p, const double* a) {
  if (!p || !a) return fail(PQG_ERR_INVALID, "NULL argument");
  drop_graphs(p);
  return upload(p->a, a, (size_t)p->nz * p->nz * p->ny * p->nk);
}

PQG_API int pqg_set_ubg(pqg_plan* p, const double* Ubg) {
  if (!p || !Ubg) return fail(PQG_ERR_INVALID, "NULL argument");
  drop_graphs(p);
  return upload(p->Ubg, Ubg, p->nz);
}

PQG_API int pqg_set_qy(pqg_plan* p, const double* Qy) {
  if (!p || !Qy) return fail(PQG_ERR_INVALID, "NULL argument");
  drop_graphs(p);
  p->h_Qy.assign(Qy, Qy + p->nz);
  p->have_qy = true;
  return refresh_kqy(p);
}

PQG_API int pqg_set_filter(pqg_plan* p, const double* filtr) {
  if (!p || !filtr) return fail(PQG_ERR_INVALID, "NULL argument");
  drop_graphs(p);
  return upload(p->filtr, filtr, (size_t)p->ny * p->nk);
}

PQG_API int pqg_set_engine(pqg_plan* p, int engine) {
  if (!p) return fail(PQG_ERR_INVALID, "NULL argument");
  if (engine != 0 && engine != 1) return fail(PQG_ERR_INVALID, "engine must be 0 (FP64) or 1 (fixed point)");
  if (engine == 1 && !p->twx_q) return fail(PQG_ERR_UNSUPPORTED, "the fixed-point engine needs power-of-two nx, ny (16..2048)");
  if (engine != p->engine) drop_graphs(p);
  p->engine = engine;
  return PQG_OK;
}

PQG_API int pqg_get_engine(const pqg_plan* p) { return p ? p->engine : -1; }

PQG_API int pqg_set_rek(pqg_plan* p, double rek) {
  if (!p) return fail(PQG_ERR_INVALID, "NULL argument");
  if (rek != p->rek) drop_graphs(p);
  p->rek = rek;
  return PQG_OK;
}

PQG_API int pqg_rfft2(pqg_plan* p, const double* x, double* xh, int nplanes, void* stream) {
  if (!p || !x || !xh || nplanes < 0) return fail(PQG_ERR_INVALID, "bad argument to pqg_rfft2");
  cudaStream_t st = (cudaStream_t)stream;
  const int chunk = p->scratch_planes;
  const size_t pr = (size_t)p->ny * p->nx, pc = (size_t)p->ny * p->nk;
  for (int p0 = 0; p0 < nplanes; p0 += chunk) {
    const int n = std::min(chunk, nplanes - p0);
    int rc = launch_row_r2c(p, x + p0 * pr, p->scratch, n, st, 0);
    if (!rc) rc = launch_col_batch<false>(p, p->scratch, dc(xh) + p0 * pc, n, st, 0);
    if (rc) return rc;
  }
  return PQG_OK;
}

PQG_API int pqg_irfft2(pqg_plan* p, const double* xh, double* x, int nplanes, void* stream) {
  if (!p || !x || !xh || nplanes < 0) return fail(PQG_ERR_INVALID, "bad argument to pqg_irfft2");
  cudaStream_t st = (cudaStream_t)stream;
  const int chunk = p->scratch_planes;
  const size_t pr = (size_t)p->ny * p->nx, pc = (size_t)p->ny * p->nk;
  for (int p0 = 0; p0 < nplanes; p0 += chunk) {
    const int n = std::min(chunk, nplanes - p0);
    int rc = launch_col_batch<true>(p, dc(xh) + p0 * pc, p->scratch, n, st, 0);
    if (!rc) rc = launch_row_c2r(p, p->scratch, x + p0 * pr, n, st, 0);
    if (rc) return rc;
  }
  return PQG_OK;
}

PQG_API int pqg_invert(pqg_plan* p, const double* qh, double* ph, double* uh, double* vh,
               double* u, double* v, void* stream) {
  if (!p || !qh || !u || !v) return fail(PQG_ERR_INVALID, "NULL argument to pqg_invert");
  cudaStream_t st = (cudaStream_t)stream;
  const size_t pc = (size_t)p->ny * p->nk;
  double2* mU = p->scratch;
  double2* mV = p->scratch + p->nz * pc;
  dim3 grid(p->nz, p->nk);
  col_invert_kernel(p->engine, p->ny)<<<grid, p->T_col, col_smem(p, 2), st>>>(geo(p), consts(p), dc(qh), dc(ph), dc(uh), dc(vh), mU, mV, p->twy_q);
  CHECK_LAUNCH();
  int rc = launch_row_c2r(p, mU, u, p->nz, st, p->engine);
  if (!rc) rc = launch_row_c2r(p, mV, v, p->nz, st, p->engine);
  return rc;
}

PQG_API int pqg_do_advection(pqg_plan* p, const double* q, const double* u, const double* v,
                     const double* ph, double* uq, double* vq, double* uqh, double* vqh,
                     double* dqhdt, void* stream) {
  if (!p || !q || !u || !v || !ph || !dqhdt) return fail(PQG_ERR_INVALID, "NULL argument to pqg_do_advection");
  cudaStream_t st = (cudaStream_t)stream;
  const size_t pc = (size_t)p->ny * p->nk;
  RowAdvArgs A{};
  A.physU = u; A.physV = v; A.physQ = q;
  A.outUQ = uq; A.outVQ = vq;
  A.mixUQ = p->scratch;
  A.mixVQ = p->scratch + p->nz * pc;
  int rc = launch_row_adv(p, A, st);
  if (rc) return rc;
  dim3 grid(p->nz, p->nk);
  col_adv_kernel(p->engine, p->ny)<<<grid, p->T_col, col_smem(p, 2), st>>>(geo(p), consts(p), A.mixUQ, A.mixVQ, dc(ph), dc(uqh), dc(vqh), dc(dqhdt), p->twy_q);
  CHECK_LAUNCH();
  return PQG_OK;
}

PQG_API int pqg_do_friction(pqg_plan* p, const double* ph, double* dqhdt, void* stream) {
  if (!p || !ph || !dqhdt) return fail(PQG_ERR_INVALID, "NULL argument to pqg_do_friction");
  if (p->rek == 0.0) return PQG_OK;  // `if self.rek:` (pyqg/kernel.pyx:451)
  const int n = p->ny * p->nk;
  k_friction<<<(n + 255) / 256, 256, 0, (cudaStream_t)stream>>>(geo(p), consts(p), dc(ph), dc(dqhdt));
  CHECK_LAUNCH();
  return PQG_OK;
}

PQG_API int pqg_do_q_forcing(pqg_plan* p, const double* dq, double* dqh, double* dqhdt, void* stream) {
  if (!p || !dq || !dqhdt) return fail(PQG_ERR_INVALID, "NULL argument to pqg_do_q_forcing");
  cudaStream_t st = (cudaStream_t)stream;
  const size_t pc = (size_t)p->ny * p->nk;
  int rc = ensure_scratch(p, 4 * p->nz);
  if (rc) return rc;
  double2* tmp = dqh ? dc(dqh) : p->scratch + 3 * p->nz * pc;
  rc = launch_row_r2c(p, dq, p->scratch, p->nz, st, p->engine);
  if (!rc) rc = launch_col_batch<false>(p, p->scratch, tmp, p->nz, st, p->engine);
  if (rc) return rc;
  const size_t n = p->nz * pc;
  k_add_q<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(geo(p), tmp, dc(dqhdt));
  CHECK_LAUNCH();
  return PQG_OK;
}

PQG_API int pqg_do_uv_forcing(pqg_plan* p, const double* du, const double* dv, double* duh,
                      double* dvh, double* dqhdt, void* stream) {
  if (!p || !du || !dv || !dqhdt) return fail(PQG_ERR_INVALID, "NULL argument to pqg_do_uv_forcing");
  cudaStream_t st = (cudaStream_t)stream;
  const size_t pc = (size_t)p->ny * p->nk;
  int rc = ensure_scratch(p, 5 * p->nz);
  if (rc) return rc;
  double2* tu = duh ? dc(duh) : p->scratch + 3 * p->nz * pc;
  double2* tv = dvh ? dc(dvh) : p->scratch + 4 * p->nz * pc;
  rc = launch_row_r2c(p, du, p->scratch, p->nz, st, p->engine);
  if (!rc) rc = launch_col_batch<false>(p, p->scratch, tu, p->nz, st, p->engine);
  if (!rc) rc = launch_row_r2c(p, dv, p->scratch, p->nz, st, p->engine);
  if (!rc) rc = launch_col_batch<false>(p, p->scratch, tv, p->nz, st, p->engine);
  if (rc) return rc;
  const size_t n = p->nz * pc;
  k_add_uv<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(geo(p), consts(p), tu, tv, dc(dqhdt));
  CHECK_LAUNCH();
  return PQG_OK;
}

PQG_API int pqg_forward_timestep(pqg_plan* p, int ablevel, double dt, double* qh, const double* dqhdt,
                         double* dqhdt_p, double* dqhdt_pp, double* q, int rotate, void* stream) {
  if (!p || !qh || !dqhdt || !dqhdt_p || !dqhdt_pp || !q)
    return fail(PQG_ERR_INVALID, "NULL argument to pqg_forward_timestep");
  cudaStream_t st = (cudaStream_t)stream;
  double c1, c2, c3;
  ab_coeffs(ablevel, dt, c1, c2, c3);
  dim3 grid(p->nz, p->nk);
  col_ab3_kernel(p->engine, p->ny)<<<grid, p->T_col, col_smem(p, 1), st>>>(
      geo(p), consts(p), dc(qh), dc(dqhdt), dc(dqhdt_p), dc(dqhdt_pp), c1, c2, c3, rotate, p->scratch, p->twy_q);
  CHECK_LAUNCH();
  return launch_row_c2r(p, p->scratch, q, p->nz, st, p->engine);
}

// one fused step: row kernel (+ column kernel); `first` reads physical q.
// `ev` (optional, 3 events) is recorded before the row kernel, between the
// two kernels and after the column kernel.
static int fused_step(pqg_plan* p, pqg_state* s, bool first, const pqg_aux* aux, cudaStream_t st,
                      cudaEvent_t* ev = nullptr) {
  const size_t pc = (size_t)p->ny * p->nk;
  double2* mU = p->scratch;
  double2* mV = p->scratch + p->nz * pc;
  double2* mQ = p->scratch + 2 * p->nz * pc;
  RowAdvArgs R{};
  R.mixU = mU; R.mixV = mV;
  if (first) R.physQ = s->q; else R.mixQ = mQ;
  R.mixUQ = mU; R.mixVQ = mV;
  if (aux) { R.outU = aux->u; R.outV = aux->v; R.outUQ = aux->uq; R.outVQ = aux->vq; }
  if (ev) PQG_CUDA(cudaEventRecord(ev[0], st));
  int rc = launch_row_adv(p, R, st);
  if (rc) return rc;
  if (ev) PQG_CUDA(cudaEventRecord(ev[1], st));
  FusedColArgs C{};
  C.qh = dc(s->qh);
  C.dqp = dc(s->dqhdt_p);
  C.dqpp = dc(s->dqhdt_pp);
  C.dqout = dc(s->dqhdt_pp);
  C.mixUQ = mU; C.mixVQ = mV;
  C.mixU = mU; C.mixV = mV; C.mixQ = mQ;
  if (aux) { C.ph = dc(aux->ph); C.uh = dc(aux->uh); C.vh = dc(aux->vh); C.uqh = dc(aux->uqh); C.vqh = dc(aux->vqh); }
  ab_coeffs(s->ablevel, s->dt, C.c1, C.c2, C.c3);
  rc = launch_col_fused(p, C, st);
  if (rc) return rc;
  if (ev) PQG_CUDA(cudaEventRecord(ev[2], st));
  // history rotation by pointers (values as pyqg/kernel.pyx:509-510)
  double* newest = s->dqhdt_pp;
  s->dqhdt_pp = s->dqhdt_p;
  s->dqhdt_p = newest;
  s->dqhdt = newest;
  s->ablevel = s->ablevel >= 2 ? 2 : s->ablevel + 1;
  s->tc += 1;
  s->t += s->dt;
  return PQG_OK;
}

PQG_API int pqg_step(pqg_plan* p, pqg_state* s, int nsteps, const pqg_aux* aux, void* stream) {
  if (!p || !s || !s->q || !s->qh || !s->dqhdt_p || !s->dqhdt_pp)
    return fail(PQG_ERR_INVALID, "NULL argument to pqg_step");
  if (s->dqhdt_p == s->dqhdt_pp) return fail(PQG_ERR_INVALID, "dqhdt_p and dqhdt_pp must be distinct buffers");
  if (nsteps <= 0) return nsteps == 0 ? PQG_OK : fail(PQG_ERR_INVALID, "nsteps < 0");
  cudaStream_t st = (cudaStream_t)stream;
  const size_t pc = (size_t)p->ny * p->nk;
  // prologue: mixed U, V of the current qh
  dim3 grid(p->nz, p->nk);
  col_invert_kernel(p->engine, p->ny)<<<grid, p->T_col, col_smem(p, 2), st>>>(
      geo(p), consts(p), dc(s->qh), nullptr, nullptr, nullptr, p->scratch, p->scratch + p->nz * pc, p->twy_q);
  CHECK_LAUNCH();
  int done = 0;
  int rc = fused_step(p, s, true, nsteps == 1 ? aux : nullptr, st);
  if (rc) return rc;
  done = 1;
  // warm-up steps until AB3 (coefficients constant afterwards)
  while (done < nsteps - 1 && s->ablevel < 2) {
    rc = fused_step(p, s, false, nullptr, st);
    if (rc) return rc;
    done++;
  }
  // steady state: replay cached graphs of an even number of steps (the
  // history buffers return to the same roles every two steps)
  const int chunk = 16;
  while (p->use_graphs && nsteps - 1 - done >= chunk) {
    std::vector<const void*> key = {s->q, s->qh, s->dqhdt_p, s->dqhdt_pp, p->scratch, stream};
    double c[3];
    ab_coeffs(2, s->dt, c[0], c[1], c[2]);
    GraphEntry* hit = nullptr;
    for (auto& e : p->graphs)
      if (e.key == key && e.nsteps == chunk && e.c[0] == c[0] && e.c[1] == c[1] && e.c[2] == c[2]) hit = &e;
    pqg_state s2 = *s;
    if (!hit) {
      cudaGraph_t graph;
      PQG_CUDA(cudaStreamBeginCapture(p->cap_stream, cudaStreamCaptureModeThreadLocal));
      for (int i = 0; i < chunk; i++) {
        rc = fused_step(p, &s2, false, nullptr, p->cap_stream);
        if (rc) {
          cudaStreamEndCapture(p->cap_stream, &graph);
          if (graph) cudaGraphDestroy(graph);
          return rc;
        }
      }
      PQG_CUDA(cudaStreamEndCapture(p->cap_stream, &graph));
      GraphEntry e;
      e.key = key;
      e.nsteps = chunk;
      e.c[0] = c[0]; e.c[1] = c[1]; e.c[2] = c[2];
      cudaError_t ie = cudaGraphInstantiate(&e.exec, graph, 0);
      cudaGraphDestroy(graph);
      if (ie != cudaSuccess) return fail(PQG_ERR_CUDA, std::string("cudaGraphInstantiate: ") + cudaGetErrorString(ie));
      if (p->graphs.size() >= 8) {
        cudaGraphExecDestroy(p->graphs.front().exec);
        p->graphs.erase(p->graphs.begin());
      }
      p->graphs.push_back(e);
      hit = &p->graphs.back();
    } else {
      for (int i = 0; i < chunk; i++) {
        double* newest = s2.dqhdt_pp;
        s2.dqhdt_pp = s2.dqhdt_p;
        s2.dqhdt_p = newest;
        s2.dqhdt = newest;
        s2.tc += 1;
        s2.t += s2.dt;
      }
    }
    PQG_CUDA(cudaGraphLaunch(hit->exec, st));
    *s = s2;
    done += chunk;
  }
  while (done < nsteps) {
    rc = fused_step(p, s, false, done == nsteps - 1 ? aux : nullptr, st);
    if (rc) return rc;
    done++;
  }
  // epilogue: physical q of the final state
  return launch_row_c2r(p, p->scratch + 2 * p->nz * pc, s->q, p->nz, st, p->engine);
}

PQG_API int pqg_step_profile(pqg_plan* p, pqg_state* s, int nsteps, double* ms, int* counts,
                             void* stream) {
  if (!p || !s || !ms || !counts || nsteps < 1) return fail(PQG_ERR_INVALID, "bad argument to pqg_step_profile");
  if (s->dqhdt_p == s->dqhdt_pp) return fail(PQG_ERR_INVALID, "dqhdt_p and dqhdt_pp must be distinct buffers");
  cudaStream_t st = (cudaStream_t)stream;
  const size_t pc = (size_t)p->ny * p->nk;
  dim3 grid(p->nz, p->nk);
  col_invert_kernel(p->engine, p->ny)<<<grid, p->T_col, col_smem(p, 2), st>>>(
      geo(p), consts(p), dc(s->qh), nullptr, nullptr, nullptr, p->scratch, p->scratch + p->nz * pc, p->twy_q);
  CHECK_LAUNCH();
  std::vector<cudaEvent_t> ev(3 * nsteps);
  for (auto& e : ev) PQG_CUDA(cudaEventCreate(&e));
  int rc = PQG_OK;
  for (int i = 0; i < nsteps && !rc; i++) rc = fused_step(p, s, i == 0, nullptr, st, &ev[3 * i]);
  if (!rc) rc = launch_row_c2r(p, p->scratch + 2 * p->nz * pc, s->q, p->nz, st, p->engine);
  if (!rc) {
    PQG_CUDA(cudaStreamSynchronize(st));
    ms[0] = ms[1] = 0.0;
    for (int i = 0; i < nsteps; i++) {
      float a = 0.f, b = 0.f;
      cudaEventElapsedTime(&a, ev[3 * i], ev[3 * i + 1]);
      cudaEventElapsedTime(&b, ev[3 * i + 1], ev[3 * i + 2]);
      ms[0] += a;
      ms[1] += b;
    }
    counts[0] = counts[1] = nsteps;
  }
  for (auto& e : ev) cudaEventDestroy(e);
  return rc;
}

// ---------------------------------------------------------------------------
// Inversion matrices in FP64 on the device (the precision form builds its
// matrices here before rounding them once): a = (S - kappa^2 I)^-1 per
// wavenumber, kappa^2 = kk[k]^2 + ll[l]^2, the singular kappa = 0 entry 0.
//   form 0: two-layer QG closed form (pyqg/qg_model.py:146-161) from
//           F1 = S[0][1], F2 = S[1][0]: det = kappa^2 (kappa^2 + F1 + F2)
//   form 1: layered (pyqg/layered_model.py:211-229): the nz = 2 closed form
//           det = (S00 - kappa^2)(S11 - kappa^2) - S01 S10, Gauss-Jordan
//           elimination with partial pivoting for nz > 2
// The closed forms follow numpy's operation order without contraction, so
// they equal the host build bit for bit; nz > 2 differs from LAPACK's LU in
// the last bits.
// ---------------------------------------------------------------------------
struct InvArgs {
  int nz, nl, nk, form;
  double S[PQG_DIAG_MAXZ * PQG_DIAG_MAXZ];
};

__global__ void k_inversion(InvArgs A, const double* __restrict__ kk, const double* __restrict__ ll, double* a) {
  const int n = A.nl * A.nk;
  const int nz = A.nz;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int l = i / A.nk, k = i - l * A.nk;
    const double w = __dadd_rn(__dmul_rn(kk[k], kk[k]), __dmul_rn(ll[l], ll[l]));
    auto put = [&](int r, int c, double v) { a[((size_t)(r * nz + c) * A.nl + l) * A.nk + k] = v; };
    if (nz == 2) {
      double det;
      if (A.form == 0) {
        const double F1 = A.S[1], F2 = A.S[2];
        det = __dmul_rn(w, __dadd_rn(__dadd_rn(w, F1), F2));
      } else {
        det = __dsub_rn(__dmul_rn(__dsub_rn(A.S[0], w), __dsub_rn(A.S[3], w)), __dmul_rn(A.S[1], A.S[2]));
      }
      if (det == 0.0 || !isfinite(det)) {
        put(0, 0, 0.0); put(0, 1, 0.0); put(1, 0, 0.0); put(1, 1, 0.0);
        continue;
      }
      const double di = __drcp_rn(det);
      if (A.form == 0) {
        const double F1 = A.S[1], F2 = A.S[2];
        put(0, 0, __dmul_rn(-__dadd_rn(w, F2), di));
        put(0, 1, __dmul_rn(-F1, di));
        put(1, 0, __dmul_rn(-F2, di));
        put(1, 1, __dmul_rn(-__dadd_rn(w, F1), di));
      } else {
        put(0, 0, __dmul_rn(__dsub_rn(A.S[3], w), di));
        put(0, 1, __dmul_rn(-A.S[1], di));
        put(1, 0, __dmul_rn(-A.S[2], di));
        put(1, 1, __dmul_rn(__dsub_rn(A.S[0], w), di));
      }
      continue;
    }
    double m[PQG_DIAG_MAXZ][2 * PQG_DIAG_MAXZ];
    bool singular = (l == 0 && k == 0);
    for (int r = 0; r < nz; r++)
      for (int c = 0; c < 2 * nz; c++)
        m[r][c] = c < nz ? (r == c ? __dsub_rn(A.S[r * nz + c], w) : A.S[r * nz + c]) : (c - nz == r ? 1.0 : 0.0);
    for (int c = 0; c < nz && !singular; c++) {
      int piv = c;
      for (int r = c + 1; r < nz; r++)
        if (fabs(m[r][c]) > fabs(m[piv][c])) piv = r;
      if (m[piv][c] == 0.0) { singular = true; break; }
      if (piv != c)
        for (int q = 0; q < 2 * nz; q++) { const double t = m[c][q]; m[c][q] = m[piv][q]; m[piv][q] = t; }
      const double inv = 1.0 / m[c][c];
      for (int q = 0; q < 2 * nz; q++) m[c][q] *= inv;
      for (int r = 0; r < nz; r++) {
        if (r == c) continue;
        const double f = m[r][c];
        if (f != 0.0)
          for (int q = 0; q < 2 * nz; q++) m[r][q] = __fma_rn(-f, m[c][q], m[r][q]);
      }
    }
    for (int r = 0; r < nz; r++)
      for (int c = 0; c < nz; c++) {
        const double v = m[r][nz + c];
        put(r, c, (singular || !isfinite(v)) ? 0.0 : v);
      }
  }
}

PQG_API int pqg_inversion_matrix(int form, int nz, int nl, int nk, const double* S, const double* kk,
                                 const double* ll, double* a, void* stream) {
  if (!S || !kk || !ll || !a || nl < 1 || nk < 1) return fail(PQG_ERR_INVALID, "bad argument to pqg_inversion_matrix");
  if (nz < 2 || nz > PQG_DIAG_MAXZ) return fail(PQG_ERR_UNSUPPORTED, "nz must be 2..8");
  if (form != 0 && form != 1) return fail(PQG_ERR_INVALID, "form must be 0 (two-layer QG) or 1 (layered)");
  if (form == 0 && nz != 2) return fail(PQG_ERR_INVALID, "the two-layer QG form needs nz = 2");
  InvArgs A{};
  A.nz = nz; A.nl = nl; A.nk = nk; A.form = form;
  for (int i = 0; i < nz * nz; i++) A.S[i] = S[i];
  const size_t n = (size_t)nl * nk;
  const unsigned grid = (unsigned)std::min<size_t>((n + 127) / 128, 152 * 16);
  k_inversion<<<grid, 128, 0, (cudaStream_t)stream>>>(A, kk, ll, a);
  PQG_CUDA(cudaGetLastError());
  return PQG_OK;
}

// ---------------------------------------------------------------------------
// Forward 2-D real transform that allocates no device memory.
//
// For callers that cannot call cudaMalloc: processes whose device memory is
// owned by another allocator (a framework's caching allocator, or a fixed
// arena reserved at start-up), and callers that must not stall the device,
// since cudaMalloc / cudaFree may wait for outstanding GPU work.  The
// transposition scratch and the twiddle tables live in file-scope
// `static __device__` arrays that every GPU loading this library keeps until
// the process exits (about 8.1 MiB per device).  Their device addresses are
// looked up once per device with cudaGetSymbolAddress (the first call on a
// device, which should therefore come before any stream capture).  The
// twiddle tables are uploaded when the (ny, nx) of a call differs from the
// previous call's on that device; such a call is not capturable either.
// All calls on a device share these arrays and overwrite them, so calls
// that may overlap on the GPU (different streams, no ordering) race; calls
// on one stream are ordered.  Every scratch element a call reads is first
// written by that call, so nothing has to be cleared between calls.
// ---------------------------------------------------------------------------
static __device__ __align__(256) double2 g_noalloc_scratch[PQG_NOALLOC_MAX_COMPLEX];
static __device__ __align__(256) double2 g_noalloc_twx[2 * 2048];
static __device__ __align__(256) double2 g_noalloc_twy[2048];

namespace {
constexpr int kMaxDevices = 64;
struct NoAllocDevice {
  bool ready = false;
  double2* scratch = nullptr;
  double2* twx = nullptr;
  double2* twy = nullptr;
  int tw_nx = 0, tw_ny = 0;
};
NoAllocDevice g_noalloc_dev[kMaxDevices];
std::mutex g_noalloc_mutex;
double2 g_noalloc_host_tw[2 * 2048];  // host staging for table uploads

void twiddles_into(int n, double2* w) {
  std::vector<double2> tmp;  // host memory only
  twiddles(n, tmp);
  std::memcpy(w, tmp.data(), sizeof(double2) * n);
}
}  // namespace

PQG_API int pqg_rfft2_noalloc(const double* x, double* xh, int nplanes, int ny, int nx, void* stream) {
  if (!x || !xh || nplanes < 1 || ny < 2 || nx < 2) return fail(PQG_ERR_INVALID, "bad argument to pqg_rfft2_noalloc");
  if (nx % 2 || ny % 2) return fail(PQG_ERR_UNSUPPORTED, "nx and ny must be even");
  if (nx / 2 > 2048 || ny > 2048) return fail(PQG_ERR_UNSUPPORTED, "nx/2 and ny must be <= 2048");
  const long long need = (long long)nplanes * ny * (nx / 2 + 1);
  if (need > PQG_NOALLOC_MAX_COMPLEX)
    return fail(PQG_ERR_UNSUPPORTED, "pqg_rfft2_noalloc: nplanes*ny*(nx/2+1) = " + std::to_string(need) +
                                         " exceeds the static scratch of " +
                                         std::to_string(PQG_NOALLOC_MAX_COMPLEX) + " complex values");
  pqg_plan p;  // shapes and block sizes only; no device memory
  p.nz = 1; p.ny = ny; p.nx = nx; p.nk = nx / 2 + 1; p.M = nx / 2;
  if (!factor(p.M, p.fx) || !factor(ny, p.fy)) return fail(PQG_ERR_UNSUPPORTED, "nx/2 and ny must factor into 2, 3 and 5");
  p.T_col = std::max(64, std::min(256, ny / 2));
  p.T_row = std::max(64, std::min(256, p.M));
  if (p.T_col < min_threads(p.fy)) p.T_col = std::min(1024, (min_threads(p.fy) + 31) / 32 * 32);
  if (p.T_row < min_threads(p.fx)) p.T_row = std::min(1024, (min_threads(p.fx) + 31) / 32 * 32);
  p.T_row_batch = p.T_row;
  p.rb_batch = std::max(1, std::min(8, 256 / p.M));
  if (p.T_col < min_threads(p.fy) || p.T_row < min_threads(p.fx))
    return fail(PQG_ERR_UNSUPPORTED, "transform too long for the block size");
  int rc = set_smem_limits();
  if (rc) return rc;
  int dev = 0;
  PQG_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) return fail(PQG_ERR_UNSUPPORTED, "device ordinal out of range");
  cudaStream_t st = (cudaStream_t)stream;
  // The lock is held until both kernels are queued: a call from another
  // host thread on the same stream that uploads other twiddle tables is
  // then ordered behind this call's kernels.
  std::lock_guard<std::mutex> lock(g_noalloc_mutex);
  {
    NoAllocDevice& d = g_noalloc_dev[dev];
    if (!d.ready) {
      // once per device, with that device current: host-side names of the
      // arrays are not device addresses; ask the runtime for those
      PQG_CUDA(cudaGetSymbolAddress((void**)&d.scratch, g_noalloc_scratch));
      PQG_CUDA(cudaGetSymbolAddress((void**)&d.twx, g_noalloc_twx));
      PQG_CUDA(cudaGetSymbolAddress((void**)&d.twy, g_noalloc_twy));
      d.ready = true;
    }
    if (d.tw_nx != nx) {
      twiddles_into(nx, g_noalloc_host_tw);
      PQG_CUDA(cudaMemcpyAsync(d.twx, g_noalloc_host_tw, sizeof(double2) * nx, cudaMemcpyHostToDevice, st));
      PQG_CUDA(cudaStreamSynchronize(st));
      d.tw_nx = nx;
    }
    if (d.tw_ny != ny) {
      twiddles_into(ny, g_noalloc_host_tw);
      PQG_CUDA(cudaMemcpyAsync(d.twy, g_noalloc_host_tw, sizeof(double2) * ny, cudaMemcpyHostToDevice, st));
      PQG_CUDA(cudaStreamSynchronize(st));
      d.tw_ny = ny;
    }
    p.twx = d.twx;
    p.twy = d.twy;
    p.scratch = d.scratch;
  }
  rc = launch_row_r2c(&p, x, p.scratch, nplanes, st, 0);
  if (!rc) rc = launch_col_batch<false>(&p, p.scratch, reinterpret_cast<double2*>(xh), nplanes, st, 0);
  p.twx = p.twy = nullptr;  // not owned: keep the plan destructor-free path
  p.scratch = nullptr;
  return rc;
}

// ---------------------------------------------------------------------------
// advection of arbitrary fields and spectral coarse-graining (FP64 transforms)
// ---------------------------------------------------------------------------
static unsigned grid_of(size_t n) { return (unsigned)std::min<size_t>((n + 255) / 256, 152 * 32); }

// out = ik fft(u f) + il fft(v f); tmp holds 4 * nplanes planes
static int advect_into(pqg_plan* p, const double* f, const double* u, const double* v, int nplanes,
                       double2* out, double2* tmp, cudaStream_t st) {
  const size_t pc = (size_t)p->ny * p->nk, pr = (size_t)p->ny * p->nx;
  double* uf = reinterpret_cast<double*>(tmp);
  double* vf = reinterpret_cast<double*>(tmp + nplanes * pc);
  double2* A = tmp + 2 * nplanes * pc;
  double2* B = tmp + 3 * nplanes * pc;
  // the physical products are packed plane after plane (stride ny * nx)
  const size_t n = (size_t)nplanes * pr;
  k_products<<<grid_of(n), 256, 0, st>>>(n, f, u, v, uf, vf);
  CHECK_LAUNCH();
  int rc = pqg_rfft2(p, uf, reinterpret_cast<double*>(A), nplanes, st);
  if (!rc) rc = pqg_rfft2(p, vf, reinterpret_cast<double*>(B), nplanes, st);
  if (rc) return rc;
  k_adv_combine<<<grid_of(nplanes * pc), 256, 0, st>>>(nplanes, p->ny, p->nk, p->kk, p->ll, A, B, out);
  CHECK_LAUNCH();
  return PQG_OK;
}

// u, v (physical) of spectral PV qh with FP64 transforms
static int velocities(pqg_plan* p, const double2* qh, double* u, double* v, cudaStream_t st) {
  const size_t pc = (size_t)p->ny * p->nk;
  double2* mU = p->scratch;
  double2* mV = p->scratch + p->nz * pc;
  dim3 grid(p->nz, p->nk);
  col_invert_kernel(0, p->ny)<<<grid, p->T_col, col_smem(p, 2), st>>>(geo(p), consts(p), qh, nullptr, nullptr,
                                                                      nullptr, mU, mV, p->twy_q);
  CHECK_LAUNCH();
  int rc = launch_row_c2r(p, mU, u, p->nz, st, 0);
  if (!rc) rc = launch_row_c2r(p, mV, v, p->nz, st, 0);
  return rc;
}

PQG_API int pqg_advect(pqg_plan* p, const double* f, const double* u, const double* v, int nplanes,
                       double* out_h, void* stream) {
  if (!p || !f || !u || !v || !out_h || nplanes < 1) return fail(PQG_ERR_INVALID, "bad argument to pqg_advect");
  if (!p->have_kk || !p->have_ll) return fail(PQG_ERR_STATE, "wavenumbers not set");
  int rc = ensure_work(p, 4 * nplanes);
  if (rc) return rc;
  return advect_into(p, f, u, v, nplanes, dc(out_h), p->work, (cudaStream_t)stream);
}

PQG_API int pqg_coarse_forcing(pqg_plan* pf, pqg_plan* pc, const double* qh_f, double* q_c, double* S,
                               void* stream) {
  if (!pf || !pc || !qh_f || !q_c || !S) return fail(PQG_ERR_INVALID, "NULL argument to pqg_coarse_forcing");
  if (pf->nz != pc->nz) return fail(PQG_ERR_INVALID, "layer counts differ");
  if (pc->nx > pf->nx || pc->ny > pf->ny || (pc->nx & 1) || (pc->ny & 1))
    return fail(PQG_ERR_INVALID, "coarse grid must be even and not finer than the fine grid");
  if (!pf->have_kk || !pf->have_ll || !pc->have_kk || !pc->have_ll) return fail(PQG_ERR_STATE, "wavenumbers not set");
  cudaStream_t st = (cudaStream_t)stream;
  const int nz = pf->nz;
  int rc = ensure_work(pf, 8 * nz);
  if (!rc) rc = ensure_work(pc, 9 * nz);
  if (rc) return rc;
  const size_t sf = (size_t)nz * pf->ny * pf->nk, sc = (size_t)nz * pc->ny * pc->nk;
  // fine: u, v, q, J = ik fft(u q) + il fft(v q)
  double* uf = reinterpret_cast<double*>(pf->work);
  double* vf = reinterpret_cast<double*>(pf->work + sf);
  double* qf = reinterpret_cast<double*>(pf->work + 2 * sf);
  double2* Jf = pf->work + 3 * sf;
  rc = velocities(pf, dc(qh_f), uf, vf, st);
  if (!rc) rc = pqg_irfft2(pf, qh_f, qf, nz, st);
  if (!rc) rc = advect_into(pf, qf, uf, vf, nz, Jf, pf->work + 4 * sf, st);
  if (rc) return rc;
  // truncate J and qh
  const double scale = ((double)pc->nx * pc->ny) / ((double)pf->nx * pf->ny);
  double2* Jbar = pc->work;
  double2* qbar = pc->work + sc;
  k_truncate<<<grid_of(sc), 256, 0, st>>>(nz, pf->ny, pf->nk, Jf, pc->ny, pc->nk, Jbar, scale);
  k_truncate<<<grid_of(sc), 256, 0, st>>>(nz, pf->ny, pf->nk, dc(qh_f), pc->ny, pc->nk, qbar, scale);
  CHECK_LAUNCH();
  // coarse: q, u, v of the truncated PV and their advection
  double* ubar = reinterpret_cast<double*>(pc->work + 2 * sc);
  double* vbar = reinterpret_cast<double*>(pc->work + 3 * sc);
  double2* Jc = pc->work + 4 * sc;
  rc = pqg_irfft2(pc, reinterpret_cast<const double*>(qbar), q_c, nz, st);
  if (!rc) rc = velocities(pc, qbar, ubar, vbar, st);
  if (!rc) rc = advect_into(pc, q_c, ubar, vbar, nz, Jc, pc->work + 5 * sc, st);
  if (rc) return rc;
  // S = filtered(J(psi, q)) - J(filtered psi, filtered q)
  k_csub<<<grid_of(sc), 256, 0, st>>>(sc, Jbar, Jc, qbar);   // qbar no longer needed
  CHECK_LAUNCH();
  return pqg_irfft2(pc, reinterpret_cast<const double*>(qbar), S, nz, st);
}

// ---------------------------------------------------------------------------
// diagnostics: FP64 accumulation on the device of the models' built-in
// diagnostics (pyqg/model.py:640-760, pyqg/qg_diagnostics.py:1-75,
// pyqg/qg_model.py:213-263, pyqg/layered_model.py:242-300), replacing the
// host loop of pyqg/model.py:802-814.  One thread per (l, k) for the
// spectral diagnostics (deterministic), block reductions with FP64 atomics
// for the domain totals.
// ---------------------------------------------------------------------------
struct DiagParams {
  int kind, nz, ny, nk, nx;
  double M2, H, rek, dt, c1, c2, c3, rd, del1, del2, U;
  double Hi[PQG_DIAG_MAXZ], Qx[PQG_DIAG_MAXZ], Qy[PQG_DIAG_MAXZ], Ubg[PQG_DIAG_MAXZ], Vbg[PQG_DIAG_MAXZ];
  double f2gpi[PQG_DIAG_MAXZ], kdi2[PQG_DIAG_MAXZ], S[PQG_DIAG_MAXZ * PQG_DIAG_MAXZ];
};

__device__ __forceinline__ double2 cget(const double* p, size_t i) {
  return reinterpret_cast<const double2*>(p)[i];
}
__device__ __forceinline__ double re_conj_mul(double2 a, double2 b) {   // Re(conj(a) b)
  return a.x * b.x + a.y * b.y;
}
__device__ __forceinline__ double abs2(double2 a) { return a.x * a.x + a.y * a.y; }

// parameterization contribution dqh + (-il duh + ik dvh) of layer z at i
__device__ __forceinline__ double2 param_contrib(const pqg_diag_fields& f, size_t o, double kx, double ly) {
  double2 r = make_double2(0.0, 0.0);
  if (f.duh && f.dvh) {
    const double2 du = cget(f.duh, o), dv = cget(f.dvh, o);
    // -il duh + ik dvh = (ly du.y - kx dv.y) + i(-ly du.x + kx dv.x)
    r.x += ly * du.y - kx * dv.y;
    r.y += -ly * du.x + kx * dv.x;
  }
  if (f.dqh) {
    const double2 d = cget(f.dqh, o);
    r.x += d.x;
    r.y += d.y;
  }
  return r;
}

__global__ void k_diag_spec(DiagParams P, pqg_diag_fields f, const double* __restrict__ a,
                            const double* __restrict__ kk, const double* __restrict__ ll,
                            const double* __restrict__ k2l2, const double* __restrict__ filtr, double* acc) {
  const int nz = P.nz, n = P.ny * P.nk;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int k = i % P.nk, l = i / P.nk;
    const double kx = kk[k], ly = ll[l], wv2 = k2l2[i];
    auto at = [&](int z) { return (size_t)z * n + i; };
    switch (P.kind) {
      case PQG_DIAG_ENSSPEC:
        for (int z = 0; z < nz; z++) acc[at(z)] += abs2(cget(f.qh, at(z))) / P.M2;
        break;
      case PQG_DIAG_KESPEC:
        for (int z = 0; z < nz; z++) acc[at(z)] += wv2 * abs2(cget(f.ph, at(z))) / P.M2;
        break;
      case PQG_DIAG_KEFRICTIONSPEC:
        acc[i] += -P.rek * P.Hi[nz - 1] / P.H * wv2 * abs2(cget(f.ph, at(nz - 1))) / P.M2;
        break;
      case PQG_DIAG_DISSSPEC:
      case PQG_DIAG_ENSDISSSPEC: {
        double s = 0.0;
        const double fm1 = filtr[i] - 1.0;
        for (int z = 0; z < nz; z++) {
          const double2 q = cget(f.qh, at(z)), d = cget(f.dqhdt, at(z)), dp = cget(f.dqhdt_p, at(z)),
                        dpp = cget(f.dqhdt_pp, at(z));
          double2 fd;
          fd.x = fm1 * (((q.x + P.c1 * d.x) + P.c2 * dp.x) + P.c3 * dpp.x);
          fd.y = fm1 * (((q.y + P.c1 * d.y) + P.c2 * dp.y) + P.c3 * dpp.y);
          const double2 w = P.kind == PQG_DIAG_DISSSPEC ? cget(f.ph, at(z)) : q;
          s += P.Hi[z] * re_conj_mul(w, fd);
        }
        acc[i] += (P.kind == PQG_DIAG_DISSSPEC ? -s : s) / P.H / P.dt / P.M2;
        break;
      }
      case PQG_DIAG_ENTSPEC: {
        double2 t = make_double2(0.0, 0.0);
        for (int z = 0; z < nz; z++) {
          const double2 q = cget(f.qh, at(z));
          t.x += P.Hi[z] * q.x;
          t.y += P.Hi[z] * q.y;
        }
        t.x /= P.H;
        t.y /= P.H;
        acc[i] += abs2(t) / P.M2;
        break;
      }
      case PQG_DIAG_ENSFLUX:
      case PQG_DIAG_KEFLUX_DIV:
      case PQG_DIAG_APEFLUX_DIV: {
        const double* J = P.kind == PQG_DIAG_ENSFLUX ? f.Jq : (P.kind == PQG_DIAG_KEFLUX_DIV ? f.Jpxi : f.JSp);
        const double* X = P.kind == PQG_DIAG_ENSFLUX ? f.qh : f.ph;
        double s = 0.0;
        for (int z = 0; z < nz; z++) s += P.Hi[z] * re_conj_mul(cget(X, at(z)), cget(J, at(z)));
        s = s / P.H / P.M2;
        acc[i] += P.kind == PQG_DIAG_ENSFLUX ? -s : s;
        break;
      }
      case PQG_DIAG_ENSFRICTIONSPEC:
        acc[i] += P.rek * P.Hi[nz - 1] / P.H * wv2 * re_conj_mul(cget(f.qh, at(nz - 1)), cget(f.ph, at(nz - 1))) / P.M2;
        break;
      case PQG_DIAG_ENSGENSPEC: {
        double s = 0.0;
        for (int z = 0; z < nz; z++) {
          // Re(i c conj(Sph) ph), c = l Qx - k Qy
          const double c = ly * P.Qx[z] - kx * P.Qy[z];
          const double2 sp = cget(f.Sph, at(z)), p = cget(f.ph, at(z));
          const double im = sp.x * p.y - sp.y * p.x;   // Im(conj(Sph) ph)
          s += P.Hi[z] * (-c * im);
        }
        acc[i] += s / P.H / P.M2;
        break;
      }
      case PQG_DIAG_APEGENSPEC: {
        double s = 0.0;
        for (int z = 0; z < nz; z++) {
          // Re((U k + V l) i conj(ph) Sph)
          const double c = P.Ubg[z] * kx + P.Vbg[z] * ly;
          const double2 p = cget(f.ph, at(z)), sp = cget(f.Sph, at(z));
          const double im = p.x * sp.y - p.y * sp.x;   // Im(conj(ph) Sph)
          s += P.Hi[z] * (-c * im);
        }
        acc[i] += s / P.H / P.M2;
        break;
      }
      case PQG_DIAG_KEFLUX: {
        const double2 p0 = cget(f.ph, at(0)), p1 = cget(f.ph, at(1));
        const double2 j0 = cget(f.Jpxi, at(0)), j1 = cget(f.Jpxi, at(1));
        acc[i] += (P.del1 * re_conj_mul(j0, p0) + P.del2 * re_conj_mul(j1, p1)) / P.M2;
        break;
      }
      case PQG_DIAG_APEFLUX: {
        const double2 p0 = cget(f.ph, at(0)), p1 = cget(f.ph, at(1));
        const double2 d = make_double2(p0.x - p1.x, p0.y - p1.y);
        acc[i] += 1.0 / (P.rd * P.rd) * P.del1 * P.del2 * re_conj_mul(cget(f.Jptpc, i), d) / P.M2;
        break;
      }
      case PQG_DIAG_APESPEC: {
        double s = 0.0;
        for (int z = 0; z + 1 < nz; z++) {
          const double2 p0 = cget(f.ph, at(z)), p1 = cget(f.ph, at(z + 1));
          s += P.f2gpi[z] * abs2(make_double2(p0.x - p1.x, p0.y - p1.y));
        }
        acc[i] += s / P.H / P.M2;
        break;
      }
      case PQG_DIAG_KESPEC_MODAL:
        for (int z = 0; z < nz; z++) acc[at(z)] += wv2 * abs2(cget(f.phn, at(z))) / P.M2;
        break;
      case PQG_DIAG_PESPEC_MODAL:
        for (int z = 1; z < nz; z++) acc[at(z - 1)] += P.kdi2[z] * abs2(cget(f.phn, at(z))) / P.M2;
        break;
      case PQG_DIAG_PARAMSPEC:
      case PQG_DIAG_ENSPARAMSPEC: {
        double s = 0.0;
        for (int z = 0; z < nz; z++) {
          const double2 dq = param_contrib(f, at(z), kx, ly);
          const double2 w = P.kind == PQG_DIAG_PARAMSPEC ? cget(f.ph, at(z)) : cget(f.qh, at(z));
          s += P.Hi[z] / P.H * re_conj_mul(w, dq);
        }
        acc[i] += (P.kind == PQG_DIAG_PARAMSPEC ? -s : s) / P.M2;
        break;
      }
      case PQG_DIAG_PARAMSPEC_KEFLUX:
      case PQG_DIAG_PARAMSPEC_APEFLUX: {
        double2 dq[PQG_DIAG_MAXZ], adq[PQG_DIAG_MAXZ];
        for (int z = 0; z < nz; z++) dq[z] = param_contrib(f, at(z), kx, ly);
        for (int z = 0; z < nz; z++) {
          double2 t = make_double2(0.0, 0.0);
          for (int z1 = 0; z1 < nz; z1++) {
            const double c = a[(size_t)(z * nz + z1) * n + i];
            t.x += c * dq[z1].x;
            t.y += c * dq[z1].y;
          }
          adq[z] = t;
        }
        double s = 0.0;
        for (int z = 0; z < nz; z++) {
          double2 term = adq[z];
          if (P.kind == PQG_DIAG_PARAMSPEC_APEFLUX) {
            term = make_double2(0.0, 0.0);
            for (int z1 = 0; z1 < nz; z1++) {
              term.x += P.S[z * nz + z1] * adq[z1].x;
              term.y += P.S[z * nz + z1] * adq[z1].y;
            }
          }
          s += P.Hi[z] / P.H * re_conj_mul(cget(f.ph, at(z)), term);
        }
        s /= P.M2;
        acc[i] += P.kind == PQG_DIAG_PARAMSPEC_KEFLUX ? wv2 * s : -s;
        break;
      }
      default:
        break;
    }
  }
}

// domain totals: EKE (per layer), EKEdiss, APEgen
__global__ void k_diag_sum(DiagParams P, pqg_diag_fields f, const double* __restrict__ kk, double* acc) {
  const int nz = P.nz;
  const size_t plane = (size_t)P.ny * P.nx;
  __shared__ double red[32];
  const int nout = P.kind == PQG_DIAG_EKE ? nz : 1;
  for (int o = 0; o < nout; o++) {
    double s = 0.0;
    if (P.kind == PQG_DIAG_EKE || P.kind == PQG_DIAG_EKEDISS) {
      const int z = P.kind == PQG_DIAG_EKE ? o : nz - 1;
      for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < plane; i += (size_t)gridDim.x * blockDim.x) {
        const double u = f.u[(size_t)z * plane + i], v = f.v[(size_t)z * plane + i];
        s += v * v + u * u;
      }
    } else {   // APEgen: -k Im(bt conj(bc)), interior columns 1..nk-3 counted twice
      const size_t n = (size_t)P.ny * P.nk;
      for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const int k = (int)(i % P.nk);
        const double2 p0 = cget(f.ph, i), p1 = cget(f.ph, n + i);
        const double2 bt = make_double2(P.del1 * p0.x + P.del2 * p1.x, P.del1 * p0.y + P.del2 * p1.y);
        const double2 bc = make_double2(p0.x - p1.x, p0.y - p1.y);
        const double im = bt.y * bc.x - bt.x * bc.y;   // Im(bt conj(bc))
        const double v = -kk[k] * im;
        s += (k >= 1 && k <= P.nk - 3) ? 2.0 * v : v;
      }
    }
    for (int off = 16; off > 0; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0) red[w] = s;
    __syncthreads();
    if (w == 0) {
      s = lane < (int)(blockDim.x >> 5) ? red[lane] : 0.0;
      for (int off = 16; off > 0; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
      if (lane == 0) {
        double scale;
        if (P.kind == PQG_DIAG_EKE) scale = 0.5 / (double)plane;
        else if (P.kind == PQG_DIAG_EKEDISS) scale = P.Hi[nz - 1] / P.H * P.rek / (double)plane;
        else scale = P.U / (P.rd * P.rd) * P.del1 * P.del2 / P.M2;
        atomicAdd(acc + o, s * scale);
      }
    }
    __syncthreads();
  }
}

PQG_API int pqg_diag_accumulate(pqg_plan* p, int kind, const pqg_diag_fields* f, double* acc, void* stream) {
  if (!p || !f || !acc) return fail(PQG_ERR_INVALID, "NULL argument to pqg_diag_accumulate");
  if (p->nz > PQG_DIAG_MAXZ) return fail(PQG_ERR_UNSUPPORTED, "too many layers for the device diagnostics");
  if (!p->have_kk || !p->have_ll) return fail(PQG_ERR_STATE, "wavenumbers not set");
  if (kind < 0 || kind >= PQG_DIAG_COUNT) return fail(PQG_ERR_INVALID, "unknown diagnostic");
  DiagParams P{};
  P.kind = kind;
  P.nz = p->nz;
  P.ny = p->ny;
  P.nk = p->nk;
  P.nx = p->nx;
  P.M2 = (double)p->nx * p->ny * (double)p->nx * p->ny;
  P.H = f->H;
  P.rek = p->rek;
  P.dt = f->dt;
  P.c1 = f->c1;
  P.c2 = f->c2;
  P.c3 = f->c3;
  P.rd = f->rd;
  P.del1 = f->del1;
  P.del2 = f->del2;
  P.U = f->U;
  for (int z = 0; z < p->nz; z++) {
    P.Hi[z] = f->Hi ? f->Hi[z] : 0.0;
    P.Qx[z] = f->Qx ? f->Qx[z] : 0.0;
    P.Qy[z] = f->Qy ? f->Qy[z] : 0.0;
    P.Ubg[z] = f->Ubg ? f->Ubg[z] : 0.0;
    P.Vbg[z] = f->Vbg ? f->Vbg[z] : 0.0;
    P.f2gpi[z] = f->f2gpi ? f->f2gpi[z] : 0.0;
    P.kdi2[z] = f->kdi2 ? f->kdi2[z] : 0.0;
    for (int z1 = 0; z1 < p->nz; z1++) P.S[z * p->nz + z1] = f->S ? f->S[z * p->nz + z1] : 0.0;
  }
  auto need = [&](const double* q, const char* what) -> bool {
    if (q) return true;
    fail(PQG_ERR_INVALID, std::string("diagnostic needs the field ") + what);
    return false;
  };
  bool ok = true;
  switch (kind) {
    case PQG_DIAG_ENSSPEC: case PQG_DIAG_ENTSPEC: ok = need(f->qh, "qh"); break;
    case PQG_DIAG_KESPEC: case PQG_DIAG_KEFRICTIONSPEC: case PQG_DIAG_APESPEC: case PQG_DIAG_APEGEN:
      ok = need(f->ph, "ph"); break;
    case PQG_DIAG_DISSSPEC: case PQG_DIAG_ENSDISSSPEC:
      ok = need(f->qh, "qh") && need(f->ph, "ph") && need(f->dqhdt, "dqhdt") && need(f->dqhdt_p, "dqhdt_p") &&
           need(f->dqhdt_pp, "dqhdt_pp");
      break;
    case PQG_DIAG_ENSFLUX: ok = need(f->qh, "qh") && need(f->Jq, "Jq"); break;
    case PQG_DIAG_ENSFRICTIONSPEC: ok = need(f->qh, "qh") && need(f->ph, "ph"); break;
    case PQG_DIAG_ENSGENSPEC: case PQG_DIAG_APEGENSPEC: ok = need(f->ph, "ph") && need(f->Sph, "Sph"); break;
    case PQG_DIAG_KEFLUX: case PQG_DIAG_KEFLUX_DIV: ok = need(f->ph, "ph") && need(f->Jpxi, "Jpxi"); break;
    case PQG_DIAG_APEFLUX: ok = need(f->ph, "ph") && need(f->Jptpc, "Jptpc"); break;
    case PQG_DIAG_APEFLUX_DIV: ok = need(f->ph, "ph") && need(f->JSp, "JSp"); break;
    case PQG_DIAG_KESPEC_MODAL: case PQG_DIAG_PESPEC_MODAL: ok = need(f->phn, "phn"); break;
    case PQG_DIAG_EKE: case PQG_DIAG_EKEDISS: ok = need(f->u, "u") && need(f->v, "v"); break;
    default: ok = need(f->ph, "ph") && need(f->qh, "qh"); break;
  }
  if (!ok) return PQG_ERR_INVALID;
  if ((kind == PQG_DIAG_KEFLUX || kind == PQG_DIAG_APEFLUX || kind == PQG_DIAG_APEGEN) && p->nz != 2)
    return fail(PQG_ERR_INVALID, "two-layer diagnostic on a model with nz != 2");
  cudaStream_t st = (cudaStream_t)stream;
  if (kind == PQG_DIAG_EKE || kind == PQG_DIAG_EKEDISS || kind == PQG_DIAG_APEGEN) {
    k_diag_sum<<<152, 256, 0, st>>>(P, *f, p->kk, acc);
  } else {
    const int n = p->ny * p->nk;
    k_diag_spec<<<(n + 255) / 256, 256, 0, st>>>(P, *f, p->a, p->kk, p->ll, p->k2l2, p->filtr, acc);
  }
  CHECK_LAUNCH();
  return PQG_OK;
}

}  // extern "C"
