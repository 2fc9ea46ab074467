// Batched ensembles of independent models on sm_103a, in FP32 or FP64.
//
// A group holds B members of one shape (nz, ny, nx) and one physics
// (inversion matrix, filter, background flow), differing in beta (through
// ikQy), bottom drag and initial state.  All members advance together: each
// model step is two kernels over the whole group (rows of all members, then
// columns of all members), so a group of small models fills the GPU.
// Several groups (uneven sizes) advance in one CUDA graph per chunk of steps,
// one graph branch per group.
//
// Precision forms: FP32 state, transforms, products and Adams-Bashforth
// update (`float2`), with the inversion matrix built in FP64 (on the GPU,
// pqg_inversion_matrix) and the constants rounded once, and the energy /
// enstrophy sums accumulated in FP64; or FP64 throughout (`double2`), which
// reproduces the single-model FP64 step bit for bit.  FP32 groups with
// 16 <= nx, ny <= 256 and at most three layers run the warp-owned row and
// column kernels of pqg_ens_warp.cuh; the others the block-wide kernels
// below (or, where the autotuner picks it, one CTA per member).
//
// Layout (member-major, spectral planes k-major so that a column is
// contiguous): q (B, nz, ny, nx); qh and the tendencies (B, nz, nk, ny);
// transposition scratch (B, nfield nz, nk, ny) (planes U, V, Q, and F, the
// closure's forcing, when a network is attached).
#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/pyqg_gb300.h"
#include "pqg_fft.cuh"

namespace cg = cooperative_groups;
using namespace pqg;

#define PQG_API __attribute__((visibility("default")))

namespace {

thread_local std::string e_last_error;
int efail(int code, const std::string& msg) {
  e_last_error = msg;
  return code;
}
#define ECUDA(call)                                                                  \
  do {                                                                               \
    cudaError_t e_ = (call);                                                         \
    if (e_ != cudaSuccess) return efail(PQG_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

// ---------------------------------------------------------------------------
// pointwise physics, generic over the precision (the double2 versions are
// the same operations as the single-model kernels)
// ---------------------------------------------------------------------------
template <class V, class S>
__device__ __forceinline__ V g_ph_acc(V acc, S a, V q) { return mk(sfma(a, q.x, acc.x), sfma(a, q.y, acc.y)); }
template <class V, class S>
__device__ __forceinline__ V g_uh(S l, V ph) { return mk(smul(l, ph.y), -smul(l, ph.x)); }
template <class V, class S>
__device__ __forceinline__ V g_vh(S k, V ph) { return mk(-smul(k, ph.y), smul(k, ph.x)); }
template <class V, class S>
__device__ __forceinline__ V g_tendency(S k, S l, S kQy, V uqh, V vqh, V ph) {
  const S re = sfma(kQy, ph.y, sfma(l, vqh.y, smul(k, uqh.y)));
  const S im = sfma(kQy, ph.x, sfma(l, vqh.x, smul(k, uqh.x)));
  return mk(re, -im);
}
template <class V, class S>
__device__ __forceinline__ V g_friction(V dq, S rk2, V ph) { return mk(sfma(rk2, ph.x, dq.x), sfma(rk2, ph.y, dq.y)); }
template <class V, class S>
__device__ __forceinline__ V g_ab(S f, V qh, V dq, V dqp, V dqpp, S c1, S c2, S c3) {
  const S re = sfma(c3, dqpp.x, sfma(c2, dqp.x, sfma(c1, dq.x, qh.x)));
  const S im = sfma(c3, dqpp.y, sfma(c2, dqp.y, sfma(c1, dq.y, qh.y)));
  return mk(smul(f, re), smul(f, im));
}

template <class V> struct Sc;
template <> struct Sc<double2> { typedef double T; };
template <> struct Sc<float2> { typedef float T; };

struct EGeo {
  int B, nz, ny, nx, nk, M;
  size_t mstride;   // scratch complex values per member (3 nz ny nk)
};

template <class S>
struct EConsts {
  const S* a;      // (nz, nz, nk, ny)  column-major in (l, k)
  const S* kk;     // (nk)
  const S* ll;     // (ny)
  const S* k2l2;   // (nk, ny)
  const S* filtr;  // (nk, ny)
  const S* kQy;    // (B, nz, nk)
  const S* Ubg;    // (B, nz)
  const S* rek;    // (B)
};

// Ensemble layout, k-major so that a spectral column is contiguous:
// spectral (B, nz, nk, ny); scratch plane (f, z) of member b holds the mixed
// values (k, y) at b*mstride + (f*nz + z)*ny*nk + k*ny + y.
__device__ __forceinline__ size_t sidx(int b, int z, int l, int k, int nz, int ny, int nk) {
  return (((size_t)b * nz + z) * nk + k) * ny + l;
}

// ---------------------------------------------------------------------------
// row kernel: rows of all members (rb consecutive rows of one plane per CTA);
// C2R of mixed U, V and Q (or physical q), products, R2C of uq, vq back into
// the U, V planes.  Spectral values of a row are at stride ny.
// ---------------------------------------------------------------------------
template <class V, int LOGM>
__global__ void e_row_adv(EGeo g, EConsts<typename Sc<V>::T> c, V* scratch, const typename Sc<V>::T* qphys,
                          const V* __restrict__ twx, typename Sc<V>::T scale, int rb,
                          typename Sc<V>::T* qout) {
  typedef typename Sc<V>::T S;
  constexpr int M = 1 << LOGM;
  extern __shared__ __align__(16) unsigned char esm[];
  V* tw = reinterpret_cast<V*>(esm);
  const int nx = 2 * M, ny = g.ny;
  const int rows_m = g.nz * ny;
  const int r0 = blockIdx.x * rb;            // rb divides ny: one plane per CTA
  const int b = r0 / rows_m, rm = r0 - b * rows_m;
  const int z = rm / ny, y0 = rm - z * ny;
  const size_t plane = (size_t)ny * g.nk;
  V* base = scratch + b * g.mstride + (size_t)z * plane + y0;   // field 0 (U)
  V* bU = tw + nx;
  V* bV = bU + rb * M;
  V* bQ = bV + rb * M;
  for (int i = threadIdx.x; i < nx; i += blockDim.x) tw[i] = twx[i];
  __syncthreads();
  const int half = M / 2 + 1;
  for (int t = threadIdx.x; t < 3 * rb * half; t += blockDim.x) {
    const int rr = t % rb, rest = t / rb;
    const int k = rest % half, f = rest / half;
    V* buf = (f == 0 ? bU : (f == 1 ? bV : bQ)) + rr * M;
    if (f < 2 || !qphys) {
      c2r_pre_s(base + (size_t)f * g.nz * plane + rr, ny, buf, M, k, tw);
    } else {
      const V* row = reinterpret_cast<const V*>(qphys + (size_t)(r0 + rr) * nx);
      if (k < M - k) buf[k] = row[k];
      if (k < M - k && M - 1 - k != k) buf[M - 1 - k] = row[M - 1 - k];
    }
  }
  __syncthreads();
  Pow2Fft<M, 1, true, V>::run(bU, M, (qphys ? 2 : 3) * rb, tw, 2);
  const S ub = c.Ubg[b * g.nz + z];
  for (int t = threadIdx.x; t < rb * M; t += blockDim.x) {
    V u = cscale(bU[t], scale), v = cscale(bV[t], scale);
    V q = bQ[t];
    if (!qphys) q = cscale(q, scale);
    if (qout) {
      const int rr = t / M, m = t - rr * M;
      *reinterpret_cast<V*>(qout + (size_t)(r0 + rr) * nx + 2 * m) = q;
    }
    bU[t] = mk(smul(sadd(u.x, ub), q.x), smul(sadd(u.y, ub), q.y));
    bV[t] = mk(smul(v.x, q.x), smul(v.y, q.y));
  }
  __syncthreads();
  Pow2Fft<M, 1, false, V>::run(bU, M, 2 * rb, tw, 2);
  for (int t = threadIdx.x; t < 2 * rb * half; t += blockDim.x) {
    const int rr = t % rb, rest = t / rb;
    const int k = rest % half, f = rest / half;
    r2c_post_s((f == 0 ? bU : bV) + rr * M, base + (size_t)f * g.nz * plane + rr, ny, M, k, tw);
  }
}

// ---------------------------------------------------------------------------
// fused column kernel: grid (nz, ceil(nk / C), B), cluster (nz, 1, 1); each
// CTA handles C consecutive columns of one layer of one member.  Shared:
// [tw (ny)] [U: C][V: C][X: C][QO: C] sequences of ny, where X first holds
// the mixed subgrid forcing F (when `forcing`), transformed with U and V and
// added to the tendency after the drag (the q_parameterization order,
// pyqg/model.py:406-436), then the new qh.
// ---------------------------------------------------------------------------
template <class V, int LOGN>
__global__ void e_col_fused(EGeo g, EConsts<typename Sc<V>::T> c, V* scratch, V* qh, const V* dqp,
                            V* dqpp, const V* __restrict__ twy, typename Sc<V>::T c1,
                            typename Sc<V>::T c2, typename Sc<V>::T c3, int C, int forcing) {
  typedef typename Sc<V>::T S;
  constexpr int N = 1 << LOGN;
  extern __shared__ __align__(16) unsigned char esm[];
  cg::cluster_group cluster = cg::this_cluster();
  const int ny = N, nk = g.nk, nz = g.nz;
  const int z = blockIdx.x, k0 = blockIdx.y * C, b = blockIdx.z;
  V* tw = reinterpret_cast<V*>(esm);
  V* bU = tw + ny;
  V* bV = bU + C * ny;
  V* bQN = bV + C * ny;   // X
  V* bQO = bQN + C * ny;
  const size_t plane = (size_t)ny * nk;
  V* mU = scratch + b * g.mstride + (size_t)z * plane;
  V* mV = mU + (size_t)nz * plane;
  V* mQ = mV + (size_t)nz * plane;
  const V* mF = mQ + (size_t)nz * plane;
  for (int i = threadIdx.x; i < ny; i += blockDim.x) tw[i] = twy[i];
  for (int t = threadIdx.x; t < C * ny; t += blockDim.x) {
    const int cc = t / ny, l = t - cc * ny, k = k0 + cc;
    const bool ok = k < nk;
    const size_t mo = (size_t)k * ny + l;
    bU[t] = ok ? mU[mo] : mk((S)0, (S)0);
    bV[t] = ok ? mV[mo] : mk((S)0, (S)0);
    if (forcing) bQN[t] = ok ? mF[mo] : mk((S)0, (S)0);
    bQO[t] = ok ? qh[sidx(b, z, l, k, nz, ny, nk)] : mk((S)0, (S)0);
  }
  __syncthreads();
  Pow2Fft<N, 1, false, V>::run(bU, ny, (forcing ? 3 : 2) * C, tw, 1);
  cluster.sync();
  const S rek = c.rek[b];
  const bool drag = (rek != (S)0) && (z == nz - 1);
  for (int t = threadIdx.x; t < C * ny; t += blockDim.x) {
    const int cc = t / ny, l = t - cc * ny, k = k0 + cc;
    if (k >= nk) continue;
    const size_t o = sidx(b, z, l, k, nz, ny, nk);
    const size_t ck = (size_t)k * ny + l;
    V p = mk((S)0, (S)0);
    for (int z1 = 0; z1 < nz; z1++) {
      const V* rq = cluster.map_shared_rank(bQO, z1);
      p = g_ph_acc(p, c.a[((size_t)z * nz + z1) * plane + ck], rq[t]);
    }
    const S kk = c.kk[k], kQy = c.kQy[((size_t)b * nz + z) * nk + k];
    V d = g_tendency(kk, c.ll[l], kQy, bU[t], bV[t], p);
    if (drag) d = g_friction(d, smul(rek, c.k2l2[ck]), p);
    if (forcing) {
      const V f = bQN[t];
      d = mk(sadd(d.x, f.x), sadd(d.y, f.y));
    }
    const V pv = dqp[o], ppv = dqpp[o];
    const V qn = g_ab(c.filtr[ck], bQO[t], d, pv, ppv, c1, c2, c3);
    qh[o] = qn;
    dqpp[o] = d;   // the newest tendency takes the oldest one's buffer
    bQN[t] = qn;
  }
  cluster.sync();
  for (int t = threadIdx.x; t < C * ny; t += blockDim.x) {
    const int cc = t / ny, l = t - cc * ny, k = k0 + cc;
    if (k >= nk) { bU[t] = mk((S)0, (S)0); bV[t] = mk((S)0, (S)0); bQN[t] = mk((S)0, (S)0); continue; }
    const size_t ck = (size_t)k * ny + l;
    V p = mk((S)0, (S)0);
    for (int z1 = 0; z1 < nz; z1++) {
      const V* rq = cluster.map_shared_rank(bQN, z1);
      p = g_ph_acc(p, c.a[((size_t)z * nz + z1) * plane + ck], rq[t]);
    }
    bU[t] = g_uh(c.ll[l], p);
    bV[t] = g_vh(c.kk[k], p);
  }
  cluster.sync();
  Pow2Fft<N, 1, true, V>::run(bU, ny, 3 * C, tw, 1);
  for (int t = threadIdx.x; t < C * ny; t += blockDim.x) {
    const int cc = t / ny, l = t - cc * ny, k = k0 + cc;
    if (k >= nk) continue;
    const size_t mo = (size_t)k * ny + l;
    mU[mo] = bU[t];
    mV[mo] = bV[t];
    mQ[mo] = bQN[t];
  }
}

// prologue: mixed U, V of the current qh (grid (nz, ceil(nk / C), B))
template <class V, int LOGN>
__global__ void e_col_invert(EGeo g, EConsts<typename Sc<V>::T> c, V* scratch, const V* qh,
                             const V* __restrict__ twy, int C) {
  typedef typename Sc<V>::T S;
  constexpr int N = 1 << LOGN;
  extern __shared__ __align__(16) unsigned char esm[];
  const int ny = N, nk = g.nk, nz = g.nz;
  const int z = blockIdx.x, k0 = blockIdx.y * C, b = blockIdx.z;
  V* tw = reinterpret_cast<V*>(esm);
  V* bU = tw + ny;
  V* bV = bU + C * ny;
  const size_t plane = (size_t)ny * nk;
  V* mU = scratch + b * g.mstride + (size_t)z * plane;
  V* mV = mU + (size_t)nz * plane;
  for (int i = threadIdx.x; i < ny; i += blockDim.x) tw[i] = twy[i];
  for (int t = threadIdx.x; t < C * ny; t += blockDim.x) {
    const int cc = t / ny, l = t - cc * ny, k = k0 + cc;
    if (k >= nk) { bU[t] = mk((S)0, (S)0); bV[t] = mk((S)0, (S)0); continue; }
    const size_t ck = (size_t)k * ny + l;
    V p = mk((S)0, (S)0);
    for (int z1 = 0; z1 < nz; z1++)
      p = g_ph_acc(p, c.a[((size_t)z * nz + z1) * plane + ck], qh[sidx(b, z1, l, k, nz, ny, nk)]);
    bU[t] = g_uh(c.ll[l], p);
    bV[t] = g_vh(c.kk[k], p);
  }
  __syncthreads();
  Pow2Fft<N, 1, true, V>::run(bU, ny, 2 * C, tw, 1);
  for (int t = threadIdx.x; t < C * ny; t += blockDim.x) {
    const int cc = t / ny, l = t - cc * ny, k = k0 + cc;
    if (k >= nk) continue;
    mU[(size_t)k * ny + l] = bU[t];
    mV[(size_t)k * ny + l] = bV[t];
  }
}

// mixed plane `field` of every member -> physical (B, nz, ny, nx)
template <class V, int LOGM>
__global__ void e_row_c2r(EGeo g, const V* scratch, int field, typename Sc<V>::T* phys,
                          const V* __restrict__ twx, typename Sc<V>::T scale, int rb) {
  constexpr int M = 1 << LOGM;
  extern __shared__ __align__(16) unsigned char esm[];
  V* tw = reinterpret_cast<V*>(esm);
  V* bq = tw + 2 * M;
  const int nx = 2 * M, ny = g.ny, rows_m = g.nz * ny;
  const int r0 = blockIdx.x * rb;
  const int b = r0 / rows_m, rm = r0 - b * rows_m, z = rm / ny, y0 = rm - z * ny;
  const size_t plane = (size_t)ny * g.nk;
  const V* base = scratch + b * g.mstride + ((size_t)field * g.nz + z) * plane + y0;
  for (int i = threadIdx.x; i < nx; i += blockDim.x) tw[i] = twx[i];
  __syncthreads();
  const int half = M / 2 + 1;
  for (int t = threadIdx.x; t < rb * half; t += blockDim.x) {
    const int rr = t % rb, k = t / rb;
    c2r_pre_s(base + rr, ny, bq + rr * M, M, k, tw);
  }
  __syncthreads();
  Pow2Fft<M, 1, true, V>::run(bq, M, rb, tw, 2);
  for (int t = threadIdx.x; t < rb * M; t += blockDim.x) {
    const int rr = t / M, m = t - rr * M;
    *reinterpret_cast<V*>(phys + (size_t)(r0 + rr) * nx + 2 * m) = cscale(bq[t], scale);
  }
}

// physical (B, nz, ny, nx) -> mixed plane 0 of every member
template <class V, int LOGM>
__global__ void e_row_r2c(EGeo g, V* scratch, const typename Sc<V>::T* phys, const V* __restrict__ twx, int rb,
                          int field) {
  constexpr int M = 1 << LOGM;
  extern __shared__ __align__(16) unsigned char esm[];
  V* tw = reinterpret_cast<V*>(esm);
  V* bq = tw + 2 * M;
  const int nx = 2 * M, ny = g.ny, rows_m = g.nz * ny;
  const int r0 = blockIdx.x * rb;
  const int b = r0 / rows_m, rm = r0 - b * rows_m, z = rm / ny, y0 = rm - z * ny;
  const size_t plane = (size_t)ny * g.nk;
  V* base = scratch + b * g.mstride + ((size_t)field * g.nz + z) * plane + y0;
  for (int i = threadIdx.x; i < nx; i += blockDim.x) tw[i] = twx[i];
  for (int t = threadIdx.x; t < rb * M; t += blockDim.x) {
    const int rr = t / M, m = t - rr * M;
    bq[t] = reinterpret_cast<const V*>(phys + (size_t)(r0 + rr) * nx)[m];
  }
  __syncthreads();
  Pow2Fft<M, 1, false, V>::run(bq, M, rb, tw, 2);
  const int half = M / 2 + 1;
  for (int t = threadIdx.x; t < rb * half; t += blockDim.x) {
    const int rr = t % rb, k = t / rb;
    r2c_post_s(bq + rr * M, base + rr, ny, M, k, tw);
  }
}

// mixed plane 0 -> spectral qh (grid (nz, ceil(nk / C), B))
template <class V, int LOGN>
__global__ void e_col_fwd(EGeo g, const V* scratch, V* qh, const V* __restrict__ twy, int C) {
  typedef typename Sc<V>::T S;
  constexpr int N = 1 << LOGN;
  extern __shared__ __align__(16) unsigned char esm[];
  const int ny = N, nk = g.nk, nz = g.nz;
  const int z = blockIdx.x, k0 = blockIdx.y * C, b = blockIdx.z;
  V* tw = reinterpret_cast<V*>(esm);
  V* bq = tw + ny;
  const V* m0 = scratch + b * g.mstride + (size_t)z * ny * nk;
  for (int i = threadIdx.x; i < ny; i += blockDim.x) tw[i] = twy[i];
  for (int t = threadIdx.x; t < C * ny; t += blockDim.x) {
    const int cc = t / ny, l = t - cc * ny, k = k0 + cc;
    bq[t] = k < nk ? m0[(size_t)k * ny + l] : mk((S)0, (S)0);
  }
  __syncthreads();
  Pow2Fft<N, 1, false, V>::run(bq, ny, C, tw, 1);
  for (int t = threadIdx.x; t < C * ny; t += blockDim.x) {
    const int cc = t / ny, l = t - cc * ny, k = k0 + cc;
    if (k < nk) qh[sidx(b, z, l, k, nz, ny, nk)] = bq[t];
  }
}

// ---------------------------------------------------------------------------
// whole model steps of one member per CTA, for square grids small enough
// that the member's mixed planes U, V, Q (3 nz x nk x N values) fit in
// shared memory: the prologue, n steps and the epilogue of the two-kernel
// path (e_col_invert; e_row_adv + e_col_fused per step; e_row_c2r) in one
// launch, with the same transforms and pointwise operations in the same
// order, so the results are identical.  The mixed planes never leave shared
// memory; qh and the AB3 history stay in global memory (each value is read
// and written by the same thread every step).
// Shared: [tw (N)] [planes (f, z) at (f nz + z) nk N, k-major] [row buffers
// U, V, Q: rb x M each].
// ---------------------------------------------------------------------------
constexpr int kMemberMaxZ = 4;

template <class S>
struct AbCoef { S c1[3], c2[3], c3[3]; };   // per start-up level 0, 1, 2

// The phases are separate (not inlined) functions.  At most 512 threads
// (FP32: 128 registers a thread) or 256 (FP64).
template <class V, int LOGN>
__device__ __noinline__ void member_prologue(const EGeo& g, const EConsts<typename Sc<V>::T>& c, const V* qh, V* P,
                                             const V* tw, int b) {
  typedef typename Sc<V>::T S;
  constexpr int N = 1 << LOGN, nk = N / 2 + 1;
  const int nz = g.nz;
  const size_t plane = (size_t)N * nk;
  for (int t = threadIdx.x; t < nz * nk * N; t += blockDim.x) {
    const int z = t / (nk * N), ck = t - z * nk * N;
    const int k = ck / N, l = ck - k * N;
    V p = mk((S)0, (S)0);
    for (int z1 = 0; z1 < nz; z1++)
      p = g_ph_acc(p, c.a[((size_t)z * nz + z1) * plane + ck], qh[sidx(b, z1, l, k, nz, N, nk)]);
    P[(size_t)z * plane + ck] = g_uh(c.ll[l], p);
    P[(size_t)(nz + z) * plane + ck] = g_vh(c.kk[k], p);
  }
  __syncthreads();
  Pow2Fft<N, 1, true, V>::run(P, N, 2 * nz * nk, tw, 1);
}

// rows of one model step (e_row_adv); `first`: q from its physical field
template <class V, int LOGN>
__device__ __noinline__ void member_rows(const EGeo& g, const EConsts<typename Sc<V>::T>& c,
                                         const typename Sc<V>::T* q, V* P, V* bU, const V* tw,
                                         typename Sc<V>::T scale, int b, bool first, int rb) {
  typedef typename Sc<V>::T S;
  constexpr int N = 1 << LOGN, M = N / 2, nk = M + 1, half = M / 2 + 1;
  const int nz = g.nz;
  const size_t plane = (size_t)N * nk;
  V* bV = bU + rb * M;
  V* bQ = bV + rb * M;
  for (int r0 = 0; r0 < nz * N; r0 += rb) {
    const int z = r0 / N, y0 = r0 - z * N;
    for (int t = threadIdx.x; t < 3 * rb * half; t += blockDim.x) {
      const int rr = t % rb, rest = t / rb;
      const int k = rest % half, f = rest / half;
      V* buf = (f == 0 ? bU : (f == 1 ? bV : bQ)) + rr * M;
      if (f < 2 || !first) {
        c2r_pre_s(P + (size_t)(f * nz + z) * plane + y0 + rr, N, buf, M, k, tw);
      } else {
        const V* row = reinterpret_cast<const V*>(q + (((size_t)b * nz + z) * N + y0 + rr) * N);
        if (k < M - k) buf[k] = row[k];
        if (k < M - k && M - 1 - k != k) buf[M - 1 - k] = row[M - 1 - k];
      }
    }
    __syncthreads();
    Pow2Fft<M, 1, true, V>::run(bU, M, (first ? 2 : 3) * rb, tw, 2);
    const S ub = c.Ubg[b * nz + z];
    for (int t = threadIdx.x; t < rb * M; t += blockDim.x) {
      const V u = cscale(bU[t], scale), v = cscale(bV[t], scale);
      V qq = bQ[t];
      if (!first) qq = cscale(qq, scale);
      bU[t] = mk(smul(sadd(u.x, ub), qq.x), smul(sadd(u.y, ub), qq.y));
      bV[t] = mk(smul(v.x, qq.x), smul(v.y, qq.y));
    }
    __syncthreads();
    Pow2Fft<M, 1, false, V>::run(bU, M, 2 * rb, tw, 2);
    for (int t = threadIdx.x; t < 2 * rb * half; t += blockDim.x) {
      const int rr = t % rb, rest = t / rb;
      const int k = rest % half, f = rest / half;
      r2c_post_s((f == 0 ? bU : bV) + rr * M, P + (size_t)(f * nz + z) * plane + y0 + rr, N, M, k, tw);
    }
    __syncthreads();
  }
}

// columns of one model step (e_col_fused without forcing): the new qh of
// every layer goes to plane Q first (global qh still holds the old values
// the other layers' inversions read), then to qh and through the inversion
// to U and V
template <class V, int LOGN>
__device__ __noinline__ void member_cols(const EGeo& g, const EConsts<typename Sc<V>::T>& c, V* qh, const V* dqp,
                                         V* dqpp, V* P, const V* tw, int b, typename Sc<V>::T c1,
                                         typename Sc<V>::T c2, typename Sc<V>::T c3) {
  typedef typename Sc<V>::T S;
  constexpr int N = 1 << LOGN, nk = N / 2 + 1;
  const int nz = g.nz;
  const size_t plane = (size_t)N * nk;
  const S rek = c.rek[b];
  Pow2Fft<N, 1, false, V>::run(P, N, 2 * nz * nk, tw, 1);
  for (int t = threadIdx.x; t < nz * nk * N; t += blockDim.x) {
    const int z = t / (nk * N), ck = t - z * nk * N;
    const int k = ck / N, l = ck - k * N;
    V p = mk((S)0, (S)0);
    for (int z1 = 0; z1 < nz; z1++)
      p = g_ph_acc(p, c.a[((size_t)z * nz + z1) * plane + ck], qh[sidx(b, z1, l, k, nz, N, nk)]);
    const S kQy = c.kQy[((size_t)b * nz + z) * nk + k];
    V d = g_tendency(c.kk[k], c.ll[l], kQy, P[(size_t)z * plane + ck], P[(size_t)(nz + z) * plane + ck], p);
    if (rek != (S)0 && z == nz - 1) d = g_friction(d, smul(rek, c.k2l2[ck]), p);
    const size_t o = sidx(b, z, l, k, nz, N, nk);
    P[(size_t)(2 * nz + z) * plane + ck] = g_ab(c.filtr[ck], qh[o], d, dqp[o], dqpp[o], c1, c2, c3);
    dqpp[o] = d;   // the newest tendency takes the oldest one's buffer
  }
  __syncthreads();
  for (int t = threadIdx.x; t < nz * nk * N; t += blockDim.x) {
    const int z = t / (nk * N), ck = t - z * nk * N;
    const int k = ck / N, l = ck - k * N;
    qh[sidx(b, z, l, k, nz, N, nk)] = P[(size_t)(2 * nz + z) * plane + ck];
    V p = mk((S)0, (S)0);
    for (int z1 = 0; z1 < nz; z1++)
      p = g_ph_acc(p, c.a[((size_t)z * nz + z1) * plane + ck], P[(size_t)(2 * nz + z1) * plane + ck]);
    P[(size_t)z * plane + ck] = g_uh(c.ll[l], p);
    P[(size_t)(nz + z) * plane + ck] = g_vh(c.kk[k], p);
  }
  __syncthreads();
  Pow2Fft<N, 1, true, V>::run(P, N, 3 * nz * nk, tw, 1);
}

// physical q from mixed plane Q (e_row_c2r)
template <class V, int LOGN>
__device__ __noinline__ void member_epilogue(const EGeo& g, typename Sc<V>::T* q, const V* P, V* bQ, const V* tw,
                                             typename Sc<V>::T scale, int b, int rb) {
  constexpr int N = 1 << LOGN, M = N / 2, nk = M + 1, half = M / 2 + 1;
  const int nz = g.nz;
  const size_t plane = (size_t)N * nk;
  for (int r0 = 0; r0 < nz * N; r0 += rb) {
    const int z = r0 / N, y0 = r0 - z * N;
    for (int t = threadIdx.x; t < rb * half; t += blockDim.x) {
      const int rr = t % rb, k = t / rb;
      c2r_pre_s(P + (size_t)(2 * nz + z) * plane + y0 + rr, N, bQ + rr * M, M, k, tw);
    }
    __syncthreads();
    Pow2Fft<M, 1, true, V>::run(bQ, M, rb, tw, 2);
    for (int t = threadIdx.x; t < rb * M; t += blockDim.x) {
      const int rr = t / M, m = t - rr * M;
      *reinterpret_cast<V*>(q + (((size_t)b * nz + z) * N + y0 + rr) * N + 2 * m) = cscale(bQ[t], scale);
    }
    __syncthreads();
  }
}

template <class V, int LOGN>
__global__ void __launch_bounds__(sizeof(V) == 8 ? 512 : 256) e_member_steps(EGeo g, EConsts<typename Sc<V>::T> c, V* qh, V* dqp,
                                                      V* dqpp, typename Sc<V>::T* q, const V* __restrict__ tw_g,
                                                      typename Sc<V>::T scale, AbCoef<typename Sc<V>::T> ab,
                                                      int ablevel, int nsteps, int rb) {
  constexpr int N = 1 << LOGN, nk = N / 2 + 1;
  extern __shared__ __align__(16) unsigned char esm[];
  const int b = blockIdx.x;
  V* tw = reinterpret_cast<V*>(esm);
  V* P = tw + N;
  V* bU = P + 3 * (size_t)g.nz * N * nk;
  for (int i = threadIdx.x; i < N; i += blockDim.x) tw[i] = tw_g[i];
  __syncthreads();
  member_prologue<V, LOGN>(g, c, qh, P, tw, b);
  for (int s = 0; s < nsteps; s++) {
    const int lvl = min(ablevel + s, 2);
    member_rows<V, LOGN>(g, c, q, P, bU, tw, scale, b, s == 0, rb);
    member_cols<V, LOGN>(g, c, qh, dqp, dqpp, P, tw, b, ab.c1[lvl], ab.c2[lvl], ab.c3[lvl]);
    V* tmp = dqp;
    dqp = dqpp;
    dqpp = tmp;
  }
  member_epilogue<V, LOGN>(g, q, P, bU + 2 * rb * (N / 2), tw, scale, b, rb);
}

// precision conversions between an FP64 staging buffer and the state
template <class S>
__global__ void e_from_f64(const double* src, S* dst, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    dst[i] = (S)src[i];
}
template <class S>
__global__ void e_to_f64(const S* src, double* dst, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    dst[i] = (double)src[i];
}

// FP64 sums per (member, layer): kinetic energy 0.5 sum w |kappa ph|^2 / M^2
// and enstrophy 0.5 sum w |qh|^2 / M^2, w = 2 for interior k columns and 1 at
// k = 0 and k = nx/2 (half-plane spectrum).  Grid (nz, B), 256 threads.
template <class V>
__global__ void e_energy(EGeo g, EConsts<typename Sc<V>::T> c, const V* qh, double* ke, double* en,
                         double inv_m2) {
  const int z = blockIdx.x, b = blockIdx.y;
  const int nz = g.nz, ny = g.ny, nk = g.nk;
  double ske = 0.0, sen = 0.0;
  for (int i = threadIdx.x; i < ny * nk; i += blockDim.x) {
    const int k = i / ny, l = i - k * ny;
    double pr = 0.0, pi = 0.0;
    for (int z1 = 0; z1 < nz; z1++) {
      const double a = (double)c.a[((size_t)z * nz + z1) * ny * nk + (size_t)k * ny + l];
      const V q = qh[sidx(b, z1, l, k, nz, ny, nk)];
      pr = fma(a, (double)q.x, pr);
      pi = fma(a, (double)q.y, pi);
    }
    const V q = qh[sidx(b, z, l, k, nz, ny, nk)];
    const double w = (k == 0 || k == nk - 1) ? 1.0 : 2.0;
    const double k2 = (double)c.k2l2[(size_t)k * ny + l];
    ske += w * k2 * (pr * pr + pi * pi);
    sen += w * ((double)q.x * (double)q.x + (double)q.y * (double)q.y);
  }
  __shared__ double red[2][32];
  for (int off = 16; off > 0; off >>= 1) {
    ske += __shfl_xor_sync(0xffffffffu, ske, off);
    sen += __shfl_xor_sync(0xffffffffu, sen, off);
  }
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (lane == 0) { red[0][w] = ske; red[1][w] = sen; }
  __syncthreads();
  if (w == 0) {
    ske = lane < (int)(blockDim.x >> 5) ? red[0][lane] : 0.0;
    sen = lane < (int)(blockDim.x >> 5) ? red[1][lane] : 0.0;
    for (int off = 16; off > 0; off >>= 1) {
      ske += __shfl_xor_sync(0xffffffffu, ske, off);
      sen += __shfl_xor_sync(0xffffffffu, sen, off);
    }
    if (lane == 0) {
      ke[(size_t)b * nz + z] = 0.5 * ske * inv_m2;
      en[(size_t)b * nz + z] = 0.5 * sen * inv_m2;
    }
  }
}

#include "pqg_ens_warp.cuh"

}  // namespace

// ===========================================================================
// host side
// ===========================================================================
struct pqg_ens {
  int B, nz, ny, nx, nk, M, prec;
  size_t esz;  // scalar bytes
  void* twx = nullptr; void* twy = nullptr;
  void* a = nullptr; void* kk = nullptr; void* ll = nullptr; void* k2l2 = nullptr; void* filtr = nullptr;
  void* kQy = nullptr; void* Ubg = nullptr; void* rek = nullptr;
  void* q = nullptr; void* qh = nullptr; void* dq[3] = {nullptr, nullptr, nullptr};
  void* scratch = nullptr;
  double* d_red = nullptr;   // 2 B nz FP64 sums
  int role_p = 1, role_pp = 2;
  int ablevel = 0;
  long long tc = 0;
  double t = 0.0, dt = 0.0;
  int T_row = 128, rb = 1, T_col = 128, C = 1;
  bool fused = false;           // whole steps per CTA (e_member_steps; the autotuner's choice)
  int T_mem = 256;              // threads of the per-member kernel
  int w_row = 8, w_col = 4;     // warps per CTA of the warp-owned FP32 row / column kernels
  bool w_stage = true;          // the row kernel stages its planes' tiles (when its rows divide ny)
  int rb_mem = 16;              // its rows per chunk of the row transforms
  int nfield = 3;               // mixed planes per member: U, V, Q (+ forcing F)
  long long version = 0;        // bumped when launch parameters change (graph cache key)
  pqg_cnn* net = nullptr;       // closure: forcing = net(q) every step
  void* qcur = nullptr;         // physical q of the current step (closure input)
  void* dqf = nullptr;          // closure output, physical
  std::vector<double> h_kk, h_Qy;  // for kQy
  bool have_consts = false, have_members = false;
};

namespace {

void drop_graphs_of(pqg_ens* e);   // graph cache (defined with the step entry points)

void cos_sin(int n, int m, long double& cr, long double& sr) {
  const long double pi = 3.141592653589793238462643383279502884L;
  long long num = 8LL * m, oct = num / n, rem = num - oct * n;
  long double x = pi / 4 * (long double)rem / (long double)n;
  long double c = cosl(x), s = sinl(x), y = pi / 4 - x;
  switch (oct) {
    case 0: cr = c; sr = s; break;
    case 1: cr = sinl(y); sr = cosl(y); break;
    case 2: cr = -s; sr = c; break;
    case 3: cr = -cosl(y); sr = sinl(y); break;
    case 4: cr = -c; sr = -s; break;
    case 5: cr = -sinl(y); sr = -cosl(y); break;
    case 6: cr = s; sr = -c; break;
    default: cr = cosl(y); sr = -sinl(y); break;
  }
}

int upload_scalars(pqg_ens* e, void* dst, const double* src, size_t n) {
  if (e->prec == 8) {
    ECUDA(cudaMemcpy(dst, src, n * sizeof(double), cudaMemcpyHostToDevice));
  } else {
    std::vector<float> f(n);
    for (size_t i = 0; i < n; i++) f[i] = (float)src[i];
    ECUDA(cudaMemcpy(dst, f.data(), n * sizeof(float), cudaMemcpyHostToDevice));
  }
  return PQG_OK;
}

int upload_twiddles(pqg_ens* e, void* dst, int n) {
  std::vector<double> w(2 * (size_t)n);
  for (int m = 0; m < n; m++) {
    long double cr, sr;
    cos_sin(n, m, cr, sr);
    w[2 * m] = (double)cr;
    w[2 * m + 1] = -(double)sr;
  }
  return upload_scalars(e, dst, w.data(), w.size());
}

bool pow2(int n) { return n > 0 && (n & (n - 1)) == 0; }
int lg2(int n) { int l = 0; while ((1 << l) < n) l++; return l; }

#define E_LOGM(X) X(3) X(4) X(5) X(6) X(7) X(8) X(9)
#define E_LOGN(X) X(4) X(5) X(6) X(7) X(8) X(9) X(10)

template <class V>
struct EK {
  typedef typename Sc<V>::T S;
  typedef void (*Member)(EGeo, EConsts<S>, V*, V*, V*, S*, const V*, S, AbCoef<S>, int, int, int);
  static Member member(int N) {
    switch (lg2(N)) {
      case 4: return e_member_steps<V, 4>;
      case 5: return e_member_steps<V, 5>;
      case 6: return member64();
      default: return nullptr;
    }
  }
  static Member member64();
  typedef void (*RowAdv)(EGeo, EConsts<S>, V*, const S*, const V*, S, int, S*);
  typedef void (*ColFused)(EGeo, EConsts<S>, V*, V*, const V*, V*, const V*, S, S, S, int, int);
  typedef void (*ColInv)(EGeo, EConsts<S>, V*, const V*, const V*, int);
  typedef void (*RowC2r)(EGeo, const V*, int, S*, const V*, S, int);
  typedef void (*RowR2c)(EGeo, V*, const S*, const V*, int, int);
  typedef void (*ColFwd)(EGeo, const V*, V*, const V*, int);
  static RowAdv row_adv(int M) {
    switch (lg2(M)) {
#define C(L) case L: return e_row_adv<V, L>;
      E_LOGM(C)
#undef C
      default: return nullptr;
    }
  }
  static RowC2r row_c2r(int M) {
    switch (lg2(M)) {
#define C(L) case L: return e_row_c2r<V, L>;
      E_LOGM(C)
#undef C
      default: return nullptr;
    }
  }
  static RowR2c row_r2c(int M) {
    switch (lg2(M)) {
#define C(L) case L: return e_row_r2c<V, L>;
      E_LOGM(C)
#undef C
      default: return nullptr;
    }
  }
  static ColFused col_fused(int N) {
    switch (lg2(N)) {
#define C(L) case L: return e_col_fused<V, L>;
      E_LOGN(C)
#undef C
      default: return nullptr;
    }
  }
  static ColInv col_inv(int N) {
    switch (lg2(N)) {
#define C(L) case L: return e_col_invert<V, L>;
      E_LOGN(C)
#undef C
      default: return nullptr;
    }
  }
  static ColFwd col_fwd(int N) {
    switch (lg2(N)) {
#define C(L) case L: return e_col_fwd<V, L>;
      E_LOGN(C)
#undef C
      default: return nullptr;
    }
  }
};

template <class V>
EConsts<typename Sc<V>::T> econsts(const pqg_ens* e) {
  typedef typename Sc<V>::T S;
  EConsts<S> c;
  c.a = (const S*)e->a; c.kk = (const S*)e->kk; c.ll = (const S*)e->ll; c.k2l2 = (const S*)e->k2l2;
  c.filtr = (const S*)e->filtr; c.kQy = (const S*)e->kQy; c.Ubg = (const S*)e->Ubg; c.rek = (const S*)e->rek;
  return c;
}
EGeo egeo(const pqg_ens* e) {
  EGeo g;
  g.B = e->B; g.nz = e->nz; g.ny = e->ny; g.nx = e->nx; g.nk = e->nk; g.M = e->M;
  g.mstride = (size_t)e->nfield * e->nz * e->ny * e->nk;
  return g;
}
size_t vsz(const pqg_ens* e) { return 2 * e->esz; }

template <class V>
int launch_row_adv(pqg_ens* e, bool first, cudaStream_t st) {
  typedef typename Sc<V>::T S;
  const int nrows = e->B * e->nz * e->ny;
  const size_t smem = vsz(e) * ((size_t)e->nx + 3 * (size_t)e->rb * e->M);
  EK<V>::row_adv(e->M)<<<(nrows + e->rb - 1) / e->rb, e->T_row, smem, st>>>(
      egeo(e), econsts<V>(e), (V*)e->scratch, first ? (const S*)e->q : nullptr, (const V*)e->twx,
      (S)(1.0 / ((double)e->nx * e->ny)), e->rb, e->net ? (S*)e->qcur : nullptr);
  ECUDA(cudaGetLastError());
  return PQG_OK;
}

template <class V>
int launch_col_fused(pqg_ens* e, cudaStream_t st) {
  typedef typename Sc<V>::T S;
  double c1, c2, c3;
  if (e->ablevel <= 0) { c1 = e->dt; c2 = 0.0; c3 = 0.0; }
  else if (e->ablevel == 1) { c1 = 1.5 * e->dt; c2 = -0.5 * e->dt; c3 = 0.0; }
  else { c1 = 23. / 12. * e->dt; c2 = -16. / 12. * e->dt; c3 = 5. / 12. * e->dt; }
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(e->nz, (e->nk + e->C - 1) / e->C, e->B);
  cfg.blockDim = dim3(e->T_col, 1, 1);
  cfg.dynamicSmemBytes = vsz(e) * (size_t)e->ny * (1 + 4 * e->C);
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = e->nz;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  ECUDA(cudaLaunchKernelEx(&cfg, EK<V>::col_fused(e->ny), egeo(e), econsts<V>(e), (V*)e->scratch, (V*)e->qh,
                           (const V*)e->dq[e->role_p], (V*)e->dq[e->role_pp], (const V*)e->twy, (S)c1, (S)c2,
                           (S)c3, e->C, e->net ? 1 : 0));
  // rotation: newest tendency in the old pp buffer
  std::swap(e->role_p, e->role_pp);
  e->ablevel = e->ablevel >= 2 ? 2 : e->ablevel + 1;
  e->tc += 1;
  e->t += e->dt;
  return PQG_OK;
}

template <class V>
int launch_prologue(pqg_ens* e, cudaStream_t st) {
  EK<V>::col_inv(e->ny)<<<dim3(e->nz, (e->nk + e->C - 1) / e->C, e->B), e->T_col,
                           vsz(e) * (size_t)e->ny * (1 + 2 * e->C), st>>>(
      egeo(e), econsts<V>(e), (V*)e->scratch, (const V*)e->qh, (const V*)e->twy, e->C);
  ECUDA(cudaGetLastError());
  return PQG_OK;
}

template <class V>
int launch_epilogue(pqg_ens* e, cudaStream_t st) {
  typedef typename Sc<V>::T S;
  const int nrows = e->B * e->nz * e->ny;
  const size_t smem = vsz(e) * ((size_t)e->nx + (size_t)e->rb * e->M);
  EK<V>::row_c2r(e->M)<<<(nrows + e->rb - 1) / e->rb, e->T_row, smem, st>>>(
      egeo(e), (const V*)e->scratch, 2, (S*)e->q, (const V*)e->twx, (S)(1.0 / ((double)e->nx * e->ny)), e->rb);
  ECUDA(cudaGetLastError());
  return PQG_OK;
}

// closure: forcing = net(q) (physical), then its row transforms into mixed
// plane 3 (the column transforms run inside the fused column kernel)
template <class V>
int launch_closure(pqg_ens* e, cudaStream_t st) {
  typedef typename Sc<V>::T S;
  const int f64 = e->prec == 8 ? 1 : 0;
  if (pqg_cnn_forward(e->net, e->qcur, f64, e->dqf, f64, e->B, st) != PQG_OK)
    return efail(PQG_ERR_CUDA, std::string("closure network: ") + pqg_cnn_last_error());
  const int nrows = e->B * e->nz * e->ny;
  EK<V>::row_r2c(e->M)<<<(nrows + e->rb - 1) / e->rb, e->T_row, vsz(e) * ((size_t)e->nx + (size_t)e->rb * e->M),
                         st>>>(egeo(e), (V*)e->scratch, (const S*)e->dqf, (const V*)e->twx, e->rb, 3);
  ECUDA(cudaGetLastError());
  return PQG_OK;
}

// nx = 64 members only in FP32 (FP64 planes do not fit in shared memory)
template <>
EK<float2>::Member EK<float2>::member64() { return e_member_steps<float2, 6>; }
template <>
EK<double2>::Member EK<double2>::member64() { return nullptr; }

// Warp-owned FP32 row and column kernels (pqg_ens_warp.cuh): FP32 groups
// with 16 <= nx <= 256, 16 <= ny <= 256 and at most three layers.  Such a
// group always runs them (not the per-member kernel), so that its results
// do not depend on the launch choices; PQG_ENS_WARP=0 turns them off.
bool warp_on(const pqg_ens* e) {
  if (e->prec != 4 || e->nz > 3 || e->M < 8 || e->M > 128 || e->ny < 16 || e->ny > 256) return false;
  if (const char* s = getenv("PQG_ENS_WARP"))
    if (s[0] == '0') return false;
  return true;
}

typedef void (*RowW)(EGeo, EConsts<float>, float2*, const float*, const float2*, float, float*);
typedef void (*ColW)(EGeo, EConsts<float>, float2*, float2*, const float2*, float2*, const float2*, float, float,
                     float, int);
template <bool STAGE>
RowW row_w_s(int M) {
  switch (lg2(M)) {
    case 3: return e_row_w<3, STAGE>;
    case 4: return e_row_w<4, STAGE>;
    case 5: return e_row_w<5, STAGE>;
    case 6: return e_row_w<6, STAGE>;
    case 7: return e_row_w<7, STAGE>;
    default: return nullptr;
  }
}
// the staged row kernel: when chosen and the CTA's rows (warps x 256 / M)
// divide ny
bool row_staged(const pqg_ens* e) { return e->w_stage && e->ny % (e->w_row * 256 / e->M) == 0; }
template <int L>
ColW col_w_nz(int nz) {
  switch (nz) {
    case 1: return e_col_w<L, 1>;
    case 2: return e_col_w<L, 2>;
    case 3: return e_col_w<L, 3>;
    default: return nullptr;
  }
}
ColW col_w(int N, int nz) {
  switch (lg2(N)) {
    case 4: return col_w_nz<4>(nz);
    case 5: return col_w_nz<5>(nz);
    case 6: return col_w_nz<6>(nz);
    case 7: return col_w_nz<7>(nz);
    case 8: return col_w_nz<8>(nz);
    default: return nullptr;
  }
}

int launch_row_w(pqg_ens* e, bool first, cudaStream_t st) {
  const int G = e->M / 8, rpw = 32 / G, W = e->w_row;
  const long long nrows = (long long)e->B * e->nz * e->ny, per = (long long)W * rpw;
  const bool stage = row_staged(e);
  const size_t smem = sizeof(float2) * ((size_t)e->nx + (size_t)W * rpw * wg::wstride(e->M) +
                                        (stage ? (size_t)(e->M + 1) * (W * rpw + 1) : 0));
  (stage ? row_w_s<true>(e->M) : row_w_s<false>(e->M))<<<(unsigned)((nrows + per - 1) / per), 32 * W, smem, st>>>(
      egeo(e), econsts<float2>(e), (float2*)e->scratch, first ? (const float*)e->q : nullptr,
      (const float2*)e->twx, (float)(1.0 / ((double)e->nx * e->ny)), e->net ? (float*)e->qcur : nullptr);
  ECUDA(cudaGetLastError());
  return PQG_OK;
}

int launch_col_w(pqg_ens* e, cudaStream_t st) {
  double c1, c2, c3;
  if (e->ablevel <= 0) { c1 = e->dt; c2 = 0.0; c3 = 0.0; }
  else if (e->ablevel == 1) { c1 = 1.5 * e->dt; c2 = -0.5 * e->dt; c3 = 0.0; }
  else { c1 = 23. / 12. * e->dt; c2 = -16. / 12. * e->dt; c3 = 5. / 12. * e->dt; }
  const int G = e->ny / 8, upw = 32 / G, W = e->w_col;
  const long long nunits = (long long)e->B * e->nk, per = (long long)W * upw;
  const size_t smem = sizeof(float2) * ((size_t)e->ny + (size_t)W * upw * wg::wstride(e->ny));
  col_w(e->ny, e->nz)<<<(unsigned)((nunits + per - 1) / per), 32 * W, smem, st>>>(
      egeo(e), econsts<float2>(e), (float2*)e->scratch, (float2*)e->qh, (const float2*)e->dq[e->role_p],
      (float2*)e->dq[e->role_pp], (const float2*)e->twy, (float)c1, (float)c2, (float)c3, e->net ? 1 : 0);
  ECUDA(cudaGetLastError());
  std::swap(e->role_p, e->role_pp);
  e->ablevel = e->ablevel >= 2 ? 2 : e->ablevel + 1;
  e->tc += 1;
  e->t += e->dt;
  return PQG_OK;
}

// per-member kernel: rows per chunk and shared memory; 0 when the group's
// shape does not fit it (square, 16 <= nx <= 64, at most 4 layers, FP64
// only up to nx = 32, shared memory within the 200 KB the kernels opt in to)
int member_rb(const pqg_ens* e) { return std::min(e->ny, e->rb_mem); }
size_t member_smem(const pqg_ens* e) {
  if (e->nx != e->ny || e->nx < 16 || e->nx > 64 || e->nz > kMemberMaxZ || (e->prec == 8 && e->nx > 32)) return 0;
  const size_t n = (size_t)e->nx + 3 * (size_t)e->nz * e->nk * e->ny + 3 * (size_t)member_rb(e) * e->M;
  const size_t b = vsz(e) * n;
  return b <= 200 * 1024 ? b : 0;
}
bool member_on(const pqg_ens* e) {
  if (e->net || !member_smem(e) || warp_on(e)) return false;
  if (const char* env = getenv("PQG_ENS_FUSED")) {   // 1: always, 0: never
    if (env[0] == '1') return true;
    if (env[0] == '0') return false;
  }
  return e->fused;
}

// nsteps model steps of every member, one CTA per member (launches of at
// most 256 steps)
template <class V>
int launch_member(pqg_ens* e, int nsteps, cudaStream_t st) {
  typedef typename Sc<V>::T S;
  AbCoef<S> ab;
  const double dt = e->dt;
  const double c1[3] = {dt, 1.5 * dt, 23. / 12. * dt}, c2[3] = {0.0, -0.5 * dt, -16. / 12. * dt},
               c3[3] = {0.0, 0.0, 5. / 12. * dt};
  for (int i = 0; i < 3; i++) {
    ab.c1[i] = (S)c1[i];
    ab.c2[i] = (S)c2[i];
    ab.c3[i] = (S)c3[i];
  }
  const size_t smem = member_smem(e);
  auto fn = EK<V>::member(e->nx);
  if (!fn || !smem) return efail(PQG_ERR_UNSUPPORTED, "no per-member kernel for this shape");
  for (int done = 0; done < nsteps;) {
    const int n = std::min(256, nsteps - done);
    fn<<<e->B, e->T_mem, smem, st>>>(egeo(e), econsts<V>(e), (V*)e->qh, (V*)e->dq[e->role_p],
                                      (V*)e->dq[e->role_pp], (S*)e->q, (const V*)e->twy,
                                      (S)(1.0 / ((double)e->nx * e->ny)), ab, e->ablevel, n, member_rb(e));
    ECUDA(cudaGetLastError());
    // the same bookkeeping as n launches of the column kernel
    if (n & 1) std::swap(e->role_p, e->role_pp);
    e->ablevel = std::min(2, e->ablevel + n);
    e->tc += n;
    for (int i = 0; i < n; i++) e->t += e->dt;
    done += n;
  }
  return PQG_OK;
}

// the row and column kernels
template <class V>
int step_two(pqg_ens* e, int nsteps, cudaStream_t st) {
  int rc = launch_prologue<V>(e, st);
  const bool w = warp_on(e);
  for (int i = 0; i < nsteps && !rc; i++) {
    rc = w ? launch_row_w(e, i == 0, st) : launch_row_adv<V>(e, i == 0, st);
    if (!rc && e->net) rc = launch_closure<V>(e, st);
    if (!rc) rc = w ? launch_col_w(e, st) : launch_col_fused<V>(e, st);
  }
  if (!rc) rc = launch_epilogue<V>(e, st);
  return rc;
}

template <class V>
int step_impl(pqg_ens* e, int nsteps, cudaStream_t st) {
  return member_on(e) ? launch_member<V>(e, nsteps, st) : step_two<V>(e, nsteps, st);
}

template <class V>
int set_q_impl(pqg_ens* e, cudaStream_t st) {
  // staging FP64 q is in scratch; convert to the state precision, then
  // qh = rfft2(q) through mixed plane 0
  typedef typename Sc<V>::T S;
  const size_t n = (size_t)e->B * e->nz * e->ny * e->nx;
  e_from_f64<S><<<1024, 256, 0, st>>>((const double*)e->scratch, (S*)e->q, n);
  ECUDA(cudaGetLastError());
  const int nrows = e->B * e->nz * e->ny;
  EK<V>::row_r2c(e->M)<<<(nrows + e->rb - 1) / e->rb, e->T_row, vsz(e) * ((size_t)e->nx + (size_t)e->rb * e->M), st>>>(
      egeo(e), (V*)e->scratch, (const S*)e->q, (const V*)e->twx, e->rb, 0);
  ECUDA(cudaGetLastError());
  EK<V>::col_fwd(e->ny)<<<dim3(e->nz, (e->nk + e->C - 1) / e->C, e->B), e->T_col,
                           vsz(e) * (size_t)e->ny * (1 + e->C), st>>>(
      egeo(e), (const V*)e->scratch, (V*)e->qh, (const V*)e->twy, e->C);
  ECUDA(cudaGetLastError());
  return PQG_OK;
}

template <class V>
int set_attrs(pqg_ens* e) {
  const int big = 200 * 1024;
  ECUDA(cudaFuncSetAttribute(EK<V>::row_adv(e->M), cudaFuncAttributeMaxDynamicSharedMemorySize, big));
  ECUDA(cudaFuncSetAttribute(EK<V>::row_c2r(e->M), cudaFuncAttributeMaxDynamicSharedMemorySize, big));
  ECUDA(cudaFuncSetAttribute(EK<V>::row_r2c(e->M), cudaFuncAttributeMaxDynamicSharedMemorySize, big));
  ECUDA(cudaFuncSetAttribute(EK<V>::col_fused(e->ny), cudaFuncAttributeMaxDynamicSharedMemorySize, big));
  ECUDA(cudaFuncSetAttribute(EK<V>::col_inv(e->ny), cudaFuncAttributeMaxDynamicSharedMemorySize, big));
  ECUDA(cudaFuncSetAttribute(EK<V>::col_fwd(e->ny), cudaFuncAttributeMaxDynamicSharedMemorySize, big));
  if (member_smem(e))
    ECUDA(cudaFuncSetAttribute(EK<V>::member(e->nx), cudaFuncAttributeMaxDynamicSharedMemorySize, big));
  return PQG_OK;
}

}  // namespace

extern "C" {

PQG_API const char* pqg_ens_last_error(void) { return e_last_error.c_str(); }

PQG_API int pqg_ens_create(pqg_ens** out, int nmembers, int nz, int ny, int nx, int precision) {
  if (!out) return efail(PQG_ERR_INVALID, "output pointer is NULL");
  *out = nullptr;
  if (nmembers < 1 || nz < 1 || nz > 8) return efail(PQG_ERR_INVALID, "need nmembers >= 1 and 1 <= nz <= 8");
  if (precision != 4 && precision != 8) return efail(PQG_ERR_INVALID, "precision must be 4 (FP32) or 8 (FP64)");
  if (!pow2(nx) || !pow2(ny) || nx < 16 || nx > 1024 || ny < 16 || ny > 1024)
    return efail(PQG_ERR_UNSUPPORTED, "ensemble grids must be powers of two, 16..1024");
  pqg_ens* e = new pqg_ens();
  e->B = nmembers; e->nz = nz; e->ny = ny; e->nx = nx; e->nk = nx / 2 + 1; e->M = nx / 2;
  e->prec = precision; e->esz = precision;
  e->rb = std::max(1, std::min(std::min(16, ny), 256 / e->M));   // divides ny (powers of two)
  e->T_row = std::max(64, std::min(256, e->rb * e->M / 2));
  e->C = std::max(1, std::min(8, 512 / ny));
  e->T_col = std::max(64, std::min(256, ny * e->C / 2));
  if (const char* s = getenv("PQG_ENS_C")) e->C = atoi(s);
  if (const char* s = getenv("PQG_ENS_T_ROW")) e->T_row = atoi(s);
  if (const char* s = getenv("PQG_ENS_RB")) e->rb = std::max(1, std::min(ny, atoi(s)));
  if (ny % e->rb) { delete e; return efail(PQG_ERR_INVALID, "rows per block must divide ny"); }
  if (const char* s = getenv("PQG_ENS_T_COL")) e->T_col = atoi(s);
  const size_t S = (size_t)nmembers * nz * ny * e->nk, P = (size_t)nmembers * nz * ny * nx;
  const size_t V = 2 * e->esz;
  bool ok = true;
  auto alloc = [&](void** p, size_t bytes) {
    if (!ok) return;
    ok = cudaMalloc(p, bytes) == cudaSuccess && cudaMemset(*p, 0, bytes) == cudaSuccess;
  };
  alloc(&e->twx, V * nx); alloc(&e->twy, V * ny);
  alloc(&e->a, e->esz * nz * nz * ny * e->nk); alloc(&e->kk, e->esz * e->nk); alloc(&e->ll, e->esz * ny);
  alloc(&e->k2l2, e->esz * ny * e->nk); alloc(&e->filtr, e->esz * ny * e->nk);
  alloc(&e->kQy, e->esz * nmembers * nz * e->nk); alloc(&e->Ubg, e->esz * nmembers * nz);
  alloc(&e->rek, e->esz * nmembers);
  alloc(&e->q, e->esz * P); alloc(&e->qh, V * S);
  for (int i = 0; i < 3; i++) alloc(&e->dq[i], V * S);
  alloc(&e->scratch, std::max(V * 3 * S, sizeof(double) * P));
  alloc((void**)&e->d_red, sizeof(double) * 2 * nmembers * nz);
  if (!ok) { pqg_ens_destroy(e); return efail(PQG_ERR_NOMEM, "cudaMalloc failed in pqg_ens_create"); }
  int rc = upload_twiddles(e, e->twx, nx);
  if (!rc) rc = upload_twiddles(e, e->twy, ny);
  if (!rc) rc = precision == 4 ? set_attrs<float2>(e) : set_attrs<double2>(e);
  if (rc) { pqg_ens_destroy(e); return rc; }
  *out = e;
  return PQG_OK;
}

PQG_API int pqg_ens_destroy(pqg_ens* e) {
  if (!e) return PQG_OK;
  drop_graphs_of(e);
  void* ps[] = {e->twx, e->twy, e->a, e->kk, e->ll, e->k2l2, e->filtr, e->kQy, e->Ubg, e->rek, e->q,
                e->qh, e->dq[0], e->dq[1], e->dq[2], e->scratch, e->d_red, e->qcur, e->dqf};
  for (void* p : ps) cudaFree(p);
  delete e;
  return PQG_OK;
}

PQG_API int pqg_ens_set_constants(pqg_ens* e, const double* a, const double* kk, const double* ll,
                                  const double* filtr, double dt) {
  if (e) {
    e->version++;     // dt enters the captured AB coefficients
    drop_graphs_of(e);
  }
  if (!e || !a || !kk || !ll || !filtr) return efail(PQG_ERR_INVALID, "NULL argument");
  const int nk = e->nk, ny = e->ny, nz = e->nz;
  // device copies are k-major: (.., nk, ny)
  std::vector<double> at((size_t)nz * nz * ny * nk), ft((size_t)ny * nk);
  for (int zz = 0; zz < nz * nz; zz++)
    for (int j = 0; j < ny; j++)
      for (int i = 0; i < nk; i++)
        at[(size_t)zz * ny * nk + (size_t)i * ny + j] = a[(size_t)zz * ny * nk + (size_t)j * nk + i];
  for (int j = 0; j < ny; j++)
    for (int i = 0; i < nk; i++) ft[(size_t)i * ny + j] = filtr[(size_t)j * nk + i];
  int rc = upload_scalars(e, e->a, at.data(), at.size());
  if (!rc) rc = upload_scalars(e, e->kk, kk, nk);
  if (!rc) rc = upload_scalars(e, e->ll, ll, ny);
  if (!rc) rc = upload_scalars(e, e->filtr, ft.data(), ft.size());
  if (rc) return rc;
  std::vector<double> k2l2((size_t)ny * nk);
  for (int j = 0; j < ny; j++)
    for (int i = 0; i < nk; i++) {
      const double x = kk[i] * kk[i], y = ll[j] * ll[j];
      k2l2[(size_t)i * ny + j] = x + y;
    }
  rc = upload_scalars(e, e->k2l2, k2l2.data(), k2l2.size());
  if (rc) return rc;
  e->h_kk.assign(kk, kk + nk);
  e->dt = dt;
  e->ablevel = 0;
  e->have_consts = true;
  return PQG_OK;
}

PQG_API int pqg_ens_set_members(pqg_ens* e, const double* Ubg, const double* Qy, const double* rek) {
  if (!e || !Ubg || !Qy || !rek) return efail(PQG_ERR_INVALID, "NULL argument");
  if (!e->have_consts) return efail(PQG_ERR_STATE, "set the shared constants first");
  const int B = e->B, nz = e->nz, nk = e->nk;
  std::vector<double> kqy((size_t)B * nz * nk);
  for (int b = 0; b < B; b++)
    for (int z = 0; z < nz; z++)
      for (int i = 0; i < nk; i++) kqy[((size_t)b * nz + z) * nk + i] = e->h_kk[i] * Qy[(size_t)b * nz + z];
  int rc = upload_scalars(e, e->kQy, kqy.data(), kqy.size());
  if (!rc) rc = upload_scalars(e, e->Ubg, Ubg, (size_t)B * nz);
  if (!rc) rc = upload_scalars(e, e->rek, rek, B);
  if (!rc) e->have_members = true;
  return rc;
}

PQG_API int pqg_ens_set_q(pqg_ens* e, const double* q_host, void* stream) {
  if (!e || !q_host) return efail(PQG_ERR_INVALID, "NULL argument");
  cudaStream_t st = (cudaStream_t)stream;
  const size_t n = (size_t)e->B * e->nz * e->ny * e->nx;
  ECUDA(cudaMemcpyAsync(e->scratch, q_host, n * sizeof(double), cudaMemcpyHostToDevice, st));
  int rc = e->prec == 4 ? set_q_impl<float2>(e, st) : set_q_impl<double2>(e, st);
  if (rc) return rc;
  ECUDA(cudaStreamSynchronize(st));
  for (int i = 0; i < 3; i++) ECUDA(cudaMemset(e->dq[i], 0, 2 * e->esz * (size_t)e->B * e->nz * e->ny * e->nk));
  e->ablevel = 0;
  e->role_p = 1;
  e->role_pp = 2;
  return PQG_OK;
}

PQG_API int pqg_ens_get_q(pqg_ens* e, double* q_host, void* stream) {
  if (!e || !q_host) return efail(PQG_ERR_INVALID, "NULL argument");
  cudaStream_t st = (cudaStream_t)stream;
  const size_t n = (size_t)e->B * e->nz * e->ny * e->nx;
  if (e->prec == 4) e_to_f64<float><<<1024, 256, 0, st>>>((const float*)e->q, (double*)e->scratch, n);
  else e_to_f64<double><<<1024, 256, 0, st>>>((const double*)e->q, (double*)e->scratch, n);
  ECUDA(cudaGetLastError());
  ECUDA(cudaMemcpyAsync(q_host, e->scratch, n * sizeof(double), cudaMemcpyDeviceToHost, st));
  ECUDA(cudaStreamSynchronize(st));
  return PQG_OK;
}

PQG_API int pqg_ens_step(pqg_ens* e, int nsteps, void* stream) {
  if (!e || nsteps < 0) return efail(PQG_ERR_INVALID, "bad argument to pqg_ens_step");
  if (!e->have_consts || !e->have_members) return efail(PQG_ERR_STATE, "constants or members not set");
  if (nsteps == 0) return PQG_OK;
  return e->prec == 4 ? step_impl<float2>(e, nsteps, (cudaStream_t)stream)
                      : step_impl<double2>(e, nsteps, (cudaStream_t)stream);
}

}  // extern "C"

// groups on their own stream branches (fork / join through events), so that
// groups overlap on the GPU
static int run_many(pqg_ens** es, int count, int nsteps, cudaStream_t st) {
  if (count == 1) return pqg_ens_step(es[0], nsteps, st);
  std::vector<cudaStream_t> br(count);
  std::vector<cudaEvent_t> done(count);
  cudaEvent_t fork;
  ECUDA(cudaEventCreateWithFlags(&fork, cudaEventDisableTiming));
  for (int i = 0; i < count; i++) {
    ECUDA(cudaStreamCreateWithFlags(&br[i], cudaStreamNonBlocking));
    ECUDA(cudaEventCreateWithFlags(&done[i], cudaEventDisableTiming));
  }
  int rc = PQG_OK;
  ECUDA(cudaEventRecord(fork, st));
  for (int i = 0; i < count && !rc; i++) {
    ECUDA(cudaStreamWaitEvent(br[i], fork, 0));
    rc = pqg_ens_step(es[i], nsteps, br[i]);
    ECUDA(cudaEventRecord(done[i], br[i]));
  }
  for (int i = 0; i < count; i++) cudaStreamWaitEvent(st, done[i], 0);
  for (int i = 0; i < count; i++) {
    cudaStreamDestroy(br[i]);
    cudaEventDestroy(done[i]);
  }
  cudaEventDestroy(fork);
  return rc;
}

// CUDA graphs of K steps of a set of ensembles in the steady state
// (ablevel 2).  K is even, so the history roles return to their captured
// assignment after every replay; the key holds the ensembles, their
// versions and roles.
namespace {
constexpr int kGraphSteps = 16;
struct EnsGraph {
  std::vector<pqg_ens*> ens;
  std::vector<long long> ver;
  std::vector<int> role;
  cudaGraphExec_t exec = nullptr;
};
std::vector<EnsGraph> g_ens_graphs;
cudaStream_t g_cap_stream = nullptr;

bool graph_matches(const EnsGraph& g, pqg_ens** es, int count) {
  if ((int)g.ens.size() != count) return false;
  for (int i = 0; i < count; i++)
    if (g.ens[i] != es[i] || g.ver[i] != es[i]->version || g.role[i] != es[i]->role_p) return false;
  return true;
}

void drop_graphs_of(pqg_ens* e) {
  for (size_t i = 0; i < g_ens_graphs.size();) {
    bool hit = false;
    for (auto* x : g_ens_graphs[i].ens) hit |= x == e;
    if (hit) {
      cudaGraphExecDestroy(g_ens_graphs[i].exec);
      g_ens_graphs.erase(g_ens_graphs.begin() + i);
    } else {
      i++;
    }
  }
}
}  // namespace

static int graph_for(pqg_ens** es, int count, cudaGraphExec_t* out) {
  for (auto& g : g_ens_graphs)
    if (graph_matches(g, es, count)) { *out = g.exec; return PQG_OK; }
  if (!g_cap_stream) ECUDA(cudaStreamCreateWithFlags(&g_cap_stream, cudaStreamNonBlocking));
  // capturing runs the host bookkeeping of K steps without executing them:
  // save it and put it back afterwards
  struct Host { int rp, rpp, ab; long long tc; double t; };
  std::vector<Host> h(count);
  for (int i = 0; i < count; i++) h[i] = {es[i]->role_p, es[i]->role_pp, es[i]->ablevel, es[i]->tc, es[i]->t};
  ECUDA(cudaStreamBeginCapture(g_cap_stream, cudaStreamCaptureModeThreadLocal));
  int rc = run_many(es, count, kGraphSteps, g_cap_stream);
  cudaGraph_t graph = nullptr;
  cudaError_t ce = cudaStreamEndCapture(g_cap_stream, &graph);
  for (int i = 0; i < count; i++) {
    es[i]->role_p = h[i].rp;
    es[i]->role_pp = h[i].rpp;
    es[i]->ablevel = h[i].ab;
    es[i]->tc = h[i].tc;
    es[i]->t = h[i].t;
  }
  if (rc) { if (graph) cudaGraphDestroy(graph); return rc; }
  if (ce != cudaSuccess) return efail(PQG_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(ce));
  EnsGraph g;
  ce = cudaGraphInstantiate(&g.exec, graph, 0);
  cudaGraphDestroy(graph);
  if (ce != cudaSuccess) return efail(PQG_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(ce));
  for (int i = 0; i < count; i++) {
    g.ens.push_back(es[i]);
    g.ver.push_back(es[i]->version);
    g.role.push_back(es[i]->role_p);
  }
  if (g_ens_graphs.size() >= 16) {
    cudaGraphExecDestroy(g_ens_graphs.front().exec);
    g_ens_graphs.erase(g_ens_graphs.begin());
  }
  g_ens_graphs.push_back(g);
  *out = g.exec;
  return PQG_OK;
}

extern "C" {

// All groups advance `nsteps` steps.  Start-up steps (FE, AB2) run as plain
// launches; steady-state stretches of 16 steps replay a captured graph
// (PQG_ENS_NO_GRAPHS=1 disables the graphs).
PQG_API int pqg_ens_step_many(pqg_ens** es, int count, int nsteps, void* stream) {
  if (!es || count < 1 || nsteps < 0) return efail(PQG_ERR_INVALID, "bad argument to pqg_ens_step_many");
  for (int i = 0; i < count; i++)
    if (!es[i] || !es[i]->have_consts || !es[i]->have_members)
      return efail(PQG_ERR_STATE, "constants or members not set");
  cudaStream_t st = (cudaStream_t)stream;
  const char* ng = getenv("PQG_ENS_NO_GRAPHS");
  if (ng && ng[0] == '1') return run_many(es, count, nsteps, st);
  int done = 0;
  auto steady = [&]() {
    for (int i = 0; i < count; i++)
      if (es[i]->ablevel < 2) return false;
    return true;
  };
  while (done < nsteps && !steady()) {
    int rc = run_many(es, count, 1, st);
    if (rc) return rc;
    done++;
  }
  const int chunks = (nsteps - done) / kGraphSteps;
  if (chunks > 0) {
    cudaGraphExec_t exec;
    int rc = graph_for(es, count, &exec);
    if (rc) return rc;
    for (int c = 0; c < chunks; c++) ECUDA(cudaGraphLaunch(exec, st));
    for (int i = 0; i < count; i++) {
      es[i]->tc += (long long)chunks * kGraphSteps;
      es[i]->t += (double)chunks * kGraphSteps * es[i]->dt;
    }
    done += chunks * kGraphSteps;
  }
  if (done < nsteps) return run_many(es, count, nsteps - done, st);
  return PQG_OK;
}

}  // extern "C"

// --- autotuner ---------------------------------------------------------
// Times the row kernel over (rows per CTA, threads) and the fused column
// kernel over (columns per CTA, threads) on the ensemble's own state, keeps
// the fastest of each and restores the state.
template <class V>
int autotune_impl(pqg_ens* e, cudaStream_t st, double* out) {
  const size_t S = (size_t)e->B * e->nz * e->ny * e->nk, P = (size_t)e->B * e->nz * e->ny * e->nx;
  const size_t vb = 2 * e->esz * S, qb = e->esz * P;
  void* save = nullptr;
  if (cudaMalloc(&save, 4 * vb + qb) != cudaSuccess) return efail(PQG_ERR_NOMEM, "autotune: cudaMalloc failed");
  unsigned char* sv = (unsigned char*)save;
  ECUDA(cudaMemcpyAsync(sv, e->qh, vb, cudaMemcpyDeviceToDevice, st));
  for (int i = 0; i < 3; i++) ECUDA(cudaMemcpyAsync(sv + (1 + i) * vb, e->dq[i], vb, cudaMemcpyDeviceToDevice, st));
  ECUDA(cudaMemcpyAsync(sv + 4 * vb, e->q, qb, cudaMemcpyDeviceToDevice, st));
  const int rp = e->role_p, rpp = e->role_pp, ab = e->ablevel;
  const long long tc = e->tc;
  const double t = e->t;
  const size_t limit = 200 * 1024;
  cudaEvent_t a, b;
  ECUDA(cudaEventCreate(&a));
  ECUDA(cudaEventCreate(&b));
  auto time3 = [&](auto&& launch) -> float {
    launch();
    cudaEventRecord(a, st);
    for (int r = 0; r < 3; r++) launch();
    cudaEventRecord(b, st);
    if (cudaEventSynchronize(b) != cudaSuccess || cudaGetLastError() != cudaSuccess) return 1e30f;
    float ms = 0.f;
    cudaEventElapsedTime(&ms, a, b);
    return ms / 3;
  };
  int rc = launch_prologue<V>(e, st);
  const bool w = warp_on(e);
  // rows
  float best_r = 1e30f;
  int brb = e->rb, btr = e->T_row;
  if (w) {
    // warp-owned kernels: the warps per CTA, and staged tiles or not
    int bw = e->w_row;
    bool bs = e->w_stage;
    for (int stg = 0; stg < 2; stg++)
      for (int nw : {2, 4, 8}) {
        if (rc) break;
        e->w_row = nw;
        e->w_stage = stg == 1;
        if (e->w_stage && !row_staged(e)) continue;
        const float ms = time3([&]() { launch_row_w(e, false, st); });
        if (ms < best_r) { best_r = ms; bw = nw; bs = e->w_stage; }
      }
    e->w_row = bw;
    e->w_stage = bs;
  }
  for (int rb = 1; rb <= 16 && !rc && !w; rb *= 2) {
    if (e->ny % rb || vsz(e) * ((size_t)e->nx + 3 * (size_t)rb * e->M) > limit) continue;
    for (int tr : {64, 128, 256, 512}) {
      if (tr > 32 * ((rb * e->M + 31) / 32) * 2) continue;
      e->rb = rb;
      e->T_row = tr;
      const float ms = time3([&]() { launch_row_adv<V>(e, false, st); });
      if (ms < best_r) { best_r = ms; brb = rb; btr = tr; }
    }
  }
  e->rb = brb;
  e->T_row = btr;
  // columns (the fused kernel updates the state: restored below)
  float best_c = 1e30f;
  int bc = e->C, btc = e->T_col;
  if (w) {
    int bw = e->w_col;
    for (int nw : {2, 4, 8}) {
      if (rc) break;
      e->w_col = nw;
      const float ms = time3([&]() { launch_col_w(e, st); });
      if (ms < best_c) { best_c = ms; bw = nw; }
    }
    e->w_col = bw;
  }
  for (int C = 1; C <= 16 && !rc && !w; C *= 2) {
    if (C > e->nk || vsz(e) * (size_t)e->ny * (1 + 4 * C) > limit) continue;
    for (int tcn : {64, 128, 256, 512}) {
      if (tcn > 2 * e->ny * C) continue;
      e->C = C;
      e->T_col = tcn;
      const float ms = time3([&]() { launch_col_fused<V>(e, st); });
      if (ms < best_c) { best_c = ms; bc = C; btc = tcn; }
    }
  }
  e->C = bc;
  e->T_col = btc;
  // whole steps: the per-member kernel (threads 128 .. 512) against the
  // row and column kernels with the shapes just chosen
  float t_two = 0.f, best_m = 0.f;
  if (!rc && !e->net && member_smem(e) && !w) {
    t_two = time3([&]() { step_two<V>(e, 4, st); });
    best_m = 1e30f;
    int bt = e->T_mem, br = e->rb_mem;
    for (int rbm : {8, 16, 32}) {
      if (rbm > e->ny) continue;
      e->rb_mem = rbm;
      if (!member_smem(e)) continue;
      for (int tm : {128, 256, 512}) {
        if (tm > (e->prec == 4 ? 512 : 256)) continue;
        e->T_mem = tm;
        const float ms = time3([&]() { launch_member<V>(e, 4, st); });
        if (ms < best_m) { best_m = ms; bt = tm; br = rbm; }
      }
    }
    e->T_mem = bt;
    e->rb_mem = br;
    e->fused = best_m < t_two;
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  ECUDA(cudaMemcpyAsync(e->qh, sv, vb, cudaMemcpyDeviceToDevice, st));
  for (int i = 0; i < 3; i++) ECUDA(cudaMemcpyAsync(e->dq[i], sv + (1 + i) * vb, vb, cudaMemcpyDeviceToDevice, st));
  ECUDA(cudaMemcpyAsync(e->q, sv + 4 * vb, qb, cudaMemcpyDeviceToDevice, st));
  ECUDA(cudaStreamSynchronize(st));
  cudaFree(save);
  e->role_p = rp;
  e->role_pp = rpp;
  e->ablevel = ab;
  e->tc = tc;
  e->t = t;
  e->version++;
  drop_graphs_of(e);
  if (out && w) {
    out[0] = 32 / (e->M / 8) * e->w_row; out[1] = 32 * e->w_row; out[2] = best_r;
    out[3] = 32 / (e->ny / 8) * e->w_col; out[4] = 32 * e->w_col; out[5] = best_c;
    out[6] = 0.0; out[7] = 0.0; out[8] = 0.0; out[9] = 0.0;
  } else if (out) {
    out[0] = e->rb; out[1] = e->T_row; out[2] = best_r;
    out[3] = e->C; out[4] = e->T_col; out[5] = best_c;
    out[6] = member_smem(e) && e->fused && !e->net ? 1.0 : 0.0; out[7] = e->T_mem;
    out[8] = best_m; out[9] = t_two;
  }
  return rc;
}

extern "C" {

PQG_API int pqg_ens_autotune(pqg_ens* e, double* out, void* stream) {
  if (!e) return efail(PQG_ERR_INVALID, "NULL argument");
  if (!e->have_consts || !e->have_members) return efail(PQG_ERR_STATE, "constants or members not set");
  cudaStream_t st = (cudaStream_t)stream;
  return e->prec == 4 ? autotune_impl<float2>(e, st, out) : autotune_impl<double2>(e, st, out);
}

PQG_API int pqg_ens_energy(pqg_ens* e, double* ke, double* ens, void* stream) {
  if (!e || !ke || !ens) return efail(PQG_ERR_INVALID, "NULL argument");
  cudaStream_t st = (cudaStream_t)stream;
  const double m2 = (double)e->nx * e->ny;
  const double inv_m2 = 1.0 / (m2 * m2);
  double* dk = e->d_red;
  double* de = e->d_red + (size_t)e->B * e->nz;
  if (e->prec == 4)
    e_energy<float2><<<dim3(e->nz, e->B), 256, 0, st>>>(egeo(e), econsts<float2>(e), (const float2*)e->qh, dk, de, inv_m2);
  else
    e_energy<double2><<<dim3(e->nz, e->B), 256, 0, st>>>(egeo(e), econsts<double2>(e), (const double2*)e->qh, dk, de, inv_m2);
  ECUDA(cudaGetLastError());
  ECUDA(cudaMemcpyAsync(ke, dk, sizeof(double) * e->B * e->nz, cudaMemcpyDeviceToHost, st));
  ECUDA(cudaMemcpyAsync(ens, de, sizeof(double) * e->B * e->nz, cudaMemcpyDeviceToHost, st));
  ECUDA(cudaStreamSynchronize(st));
  return PQG_OK;
}

PQG_API int pqg_ens_set_closure(pqg_ens* e, pqg_cnn* net) {
  if (!e) return efail(PQG_ERR_INVALID, "NULL argument");
  if (cudaDeviceSynchronize() != cudaSuccess) return efail(PQG_ERR_CUDA, "device error before pqg_ens_set_closure");
  e->version++;
  drop_graphs_of(e);
  if (!net) {
    e->net = nullptr;
    return PQG_OK;
  }
  int cin = 0, cout = 0, ny = 0, nx = 0, maxb = 0;
  if (pqg_cnn_shape(net, &cin, &cout, &ny, &nx, &maxb) != PQG_OK) return efail(PQG_ERR_INVALID, "bad network");
  if (cin != e->nz || cout != e->nz || ny != e->ny || nx != e->nx)
    return efail(PQG_ERR_INVALID, "network channels / image size must match the members' (nz, ny, nx)");
  if (maxb < e->B) return efail(PQG_ERR_INVALID, "network batch capacity below the member count");
  const size_t S = (size_t)e->B * e->nz * e->ny * e->nk, P = (size_t)e->B * e->nz * e->ny * e->nx;
  const size_t V = 2 * e->esz;
  if (e->nfield < 4) {
    void* ns = nullptr;
    if (cudaMalloc(&ns, std::max(V * 4 * S, sizeof(double) * P)) != cudaSuccess)
      return efail(PQG_ERR_NOMEM, "cudaMalloc failed in pqg_ens_set_closure");
    cudaMemset(ns, 0, std::max(V * 4 * S, sizeof(double) * P));
    cudaFree(e->scratch);
    e->scratch = ns;
    e->nfield = 4;
  }
  if (!e->qcur && cudaMalloc(&e->qcur, e->esz * P) != cudaSuccess)
    return efail(PQG_ERR_NOMEM, "cudaMalloc failed in pqg_ens_set_closure");
  if (!e->dqf && cudaMalloc(&e->dqf, e->esz * P) != cudaSuccess)
    return efail(PQG_ERR_NOMEM, "cudaMalloc failed in pqg_ens_set_closure");
  e->net = net;
  return PQG_OK;
}

PQG_API int pqg_ens_state(pqg_ens* e, void** q, void** qh, long long* tc, double* t) {
  if (!e) return efail(PQG_ERR_INVALID, "NULL argument");
  if (q) *q = e->q;
  if (qh) *qh = e->qh;
  if (tc) *tc = e->tc;
  if (t) *t = e->t;
  return PQG_OK;
}

}  // extern "C"
