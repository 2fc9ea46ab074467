// Pointwise stages of the physical parameterizations on sm_103a
// (pyqg/parameterizations.py:132-366): Smagorinsky, BackscatterBiharmonic,
// ZannaBolton2020 and RingForcing.  Their transforms run on the library's
// CUDA FFT (pqg_rfft2 / pqg_irfft2); these kernels do everything between
// the transforms, in FP64, so no arithmetic of the closures runs in a
// framework's elementwise operators.
//
// Arrays are device pointers in the library's layouts: spectral fields
// (n, nl, nk) complex as interleaved (re, im) doubles, physical fields
// (n, ny, nx) doubles; kk (nk) and ll (nl) are the wavenumbers.  A "3n"
// argument holds three fields of n planes one after the other.  Products
// with i k and i l are the reference's complex products with a purely
// imaginary factor: (i k)(a + i b) = (-k b) + i (k a).
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>

#include "../../include/pyqg_gb300.h"

#define PQG_API extern "C" __attribute__((visibility("default")))

extern "C" int pqg_report_error(int code, const char* msg);   // pqg_step.cu (not part of the C API)

namespace {

constexpr int kThreads = 256;

int blocks_for(long long n) {
  const long long b = (n + kThreads - 1) / kThreads;
  return (int)(b < 152 * 16 ? (b > 0 ? b : 1) : 152 * 16);
}

int launch_check(const char* what) {
  const cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) return PQG_OK;
  static thread_local char msg[256];
  snprintf(msg, sizeof msg, "%s: %s", what, cudaGetErrorString(e));
  return pqg_report_error(PQG_ERR_CUDA, msg);
}

__device__ __forceinline__ double2 ld2(const double* p, long long i) {
  return reinterpret_cast<const double2*>(p)[i];
}
__device__ __forceinline__ void st2(double* p, long long i, double2 v) { reinterpret_cast<double2*>(p)[i] = v; }
// (i s) z for real s
__device__ __forceinline__ double2 imul(double s, double2 z) { return make_double2(-__dmul_rn(s, z.y), __dmul_rn(s, z.x)); }
__device__ __forceinline__ double2 cadd(double2 a, double2 b) { return make_double2(__dadd_rn(a.x, b.x), __dadd_rn(a.y, b.y)); }
__device__ __forceinline__ double2 csub(double2 a, double2 b) { return make_double2(__dsub_rn(a.x, b.x), __dsub_rn(a.y, b.y)); }
__device__ __forceinline__ double2 cscal(double s, double2 z) { return make_double2(__dmul_rn(s, z.x), __dmul_rn(s, z.y)); }

// Smagorinsky strain rates, spectral: ik uh, il vh, (il uh + ik vh) / 2
// (the halving is exact and commutes with the inverse transform)
__global__ void k_smag_strain(long long S, int nl, int nk, const double* kk, const double* ll, const double* uh,
                              const double* vh, double* out) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < S; i += (long long)gridDim.x * blockDim.x) {
    const int k = (int)(i % nk), l = (int)((i / nk) % nl);
    const double2 u = ld2(uh, i), v = ld2(vh, i);
    st2(out, i, imul(kk[k], u));
    st2(out, S + i, imul(ll[l], v));
    st2(out, 2 * S + i, cscal(0.5, cadd(imul(ll[l], u), imul(kk[k], v))));
  }
}

// viscosity nu = (C dx)^2 sqrt(2 (Sxx^2 + Syy^2 + 2 Sxy^2)) and the stresses
// nu Sxx, nu Sxy, nu Syy (reference operation order, no contraction)
__global__ void k_smag_stress(long long P, const double* s3, double c2dx2, double* nu, double* p3) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < P; i += (long long)gridDim.x * blockDim.x) {
    const double sxx = s3[i], syy = s3[P + i], sxy = s3[2 * P + i];
    double t = __dadd_rn(__dmul_rn(sxx, sxx), __dmul_rn(syy, syy));
    t = __dadd_rn(t, __dmul_rn(2.0, __dmul_rn(sxy, sxy)));
    const double v = __dmul_rn(c2dx2, __dsqrt_rn(__dmul_rn(2.0, t)));
    if (nu) nu[i] = v;
    if (p3) {
      p3[i] = __dmul_rn(v, sxx);
      p3[P + i] = __dmul_rn(v, sxy);
      p3[2 * P + i] = __dmul_rn(v, syy);
    }
  }
}

// divergence of the stresses, spectral: 2 (ik nSxx + il nSxy), 2 (ik nSxy + il nSyy)
__global__ void k_smag_div(long long S, int nl, int nk, const double* kk, const double* ll, const double* n3,
                           double* out) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < S; i += (long long)gridDim.x * blockDim.x) {
    const int k = (int)(i % nk), l = (int)((i / nk) % nl);
    const double2 a = ld2(n3, i), b = ld2(n3, S + i), c = ld2(n3, 2 * S + i);
    st2(out, i, cscal(2.0, cadd(imul(kk[k], a), imul(ll[l], b))));
    st2(out, S + i, cscal(2.0, cadd(imul(kk[k], b), imul(ll[l], c))));
  }
}

// velocity gradients, spectral: ik vh, il vh, ik uh, il uh (vx, vy, ux, uy)
__global__ void k_zb_grad(long long S, int nl, int nk, const double* kk, const double* ll, const double* uh,
                          const double* vh, double* out) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < S; i += (long long)gridDim.x * blockDim.x) {
    const int k = (int)(i % nk), l = (int)((i / nk) % nl);
    const double2 u = ld2(uh, i), v = ld2(vh, i);
    st2(out, i, imul(kk[k], v));
    st2(out, S + i, imul(ll[l], v));
    st2(out, 2 * S + i, imul(kk[k], u));
    st2(out, 3 * S + i, imul(ll[l], u));
  }
}

// relative vorticity rv = vx - uy, shearing sh = vx + uy, stretching
// st = ux - vy: rv st, rv sh, rv^2 + sh^2 + st^2
__global__ void k_zb_prod(long long P, const double* g4, double* out) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < P; i += (long long)gridDim.x * blockDim.x) {
    const double vx = g4[i], vy = g4[P + i], ux = g4[2 * P + i], uy = g4[3 * P + i];
    const double rv = __dsub_rn(vx, uy), sh = __dadd_rn(vx, uy), st = __dsub_rn(ux, vy);
    out[i] = __dmul_rn(rv, st);
    out[P + i] = __dmul_rn(rv, sh);
    out[2 * P + i] = __dadd_rn(__dadd_rn(__dmul_rn(rv, rv), __dmul_rn(sh, sh)), __dmul_rn(st, st));
  }
}

// kappa (ik (ss - rsh) + il rs), kappa (il (ss + rsh) + ik rs), ss = fft(sum
// of squares) / 2, from f3 = (rs, rsh, fft(sum of squares))
__global__ void k_zb_comb(long long S, int nl, int nk, const double* kk, const double* ll, const double* f3,
                          double kappa, double* out) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < S; i += (long long)gridDim.x * blockDim.x) {
    const int k = (int)(i % nk), l = (int)((i / nk) % nl);
    const double2 rs = ld2(f3, i), rsh = ld2(f3, S + i), ss = cscal(0.5, ld2(f3, 2 * S + i));
    st2(out, i, cscal(kappa, cadd(imul(kk[k], csub(ss, rsh)), imul(ll[l], rs))));
    st2(out, S + i, cscal(kappa, cadd(imul(ll[l], cadd(ss, rsh)), imul(kk[k], rs))));
  }
}

// out = scale (k^2 + l^2)^power in (power 1 or 2): the biharmonic operator
// lap^2 and -lap of the backscatter closure, with lap = (ik)^2 + (il)^2,
// and -wv2 ph of the diagnostics
__global__ void k_lap(long long S, int nl, int nk, const double* kk, const double* ll, int power, double scale,
                      const double* in, double* out) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < S; i += (long long)gridDim.x * blockDim.x) {
    const int k = (int)(i % nk), l = (int)((i / nk) % nl);
    const double w = __dadd_rn(__dmul_rn(kk[k], kk[k]), __dmul_rn(ll[l], ll[l]));
    st2(out, i, cscal(scale, cscal(power == 2 ? __dmul_rn(w, w) : w, ld2(in, i))));
  }
}

// out[i] = sum_j m[i][j] in[j] over planes of `plane` doubles (a complex
// plane counts its re and im), j in order
constexpr int kMixMax = 8;
struct Mix {
  double m[kMixMax * kMixMax];
};
__global__ void k_layer_mix(int nout, int nin, long long plane, Mix mx, const double* in, double* out) {
  const long long total = (long long)nout * plane;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
       t += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(t / plane);
    const long long p = t - (long long)i * plane;
    double acc = 0.0;
    for (int j = 0; j < nin; j++) acc = __dadd_rn(acc, __dmul_rn(mx.m[i * kMixMax + j], in[j * plane + p]));
    out[t] = acc;
  }
}

// out = (a s) b
__global__ void k_mul_scaled(long long P, const double* a, double s, const double* b, double* out) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < P; i += (long long)gridDim.x * blockDim.x)
    out[i] = __dmul_rn(__dmul_rn(a[i], s), b[i]);
}

// per plane (one CTA each): sums[z] = mean(a b), sums[n + z] = mean(a c)
// over ny nx points, a fixed summation order
__global__ void k_plane_means(int n, long long P1, const double* a, const double* b, const double* c, double* sums) {
  const int z = blockIdx.x;
  const double* pa = a + z * P1;
  const double* pb = b + z * P1;
  const double* pc = c + z * P1;
  double s1 = 0.0, s2 = 0.0;
  for (long long i = threadIdx.x; i < P1; i += blockDim.x) {
    s1 += pa[i] * pb[i];
    s2 += pa[i] * pc[i];
  }
  __shared__ double r1[32], r2[32];
  for (int off = 16; off > 0; off >>= 1) {
    s1 += __shfl_xor_sync(0xffffffffu, s1, off);
    s2 += __shfl_xor_sync(0xffffffffu, s2, off);
  }
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (lane == 0) { r1[w] = s1; r2[w] = s2; }
  __syncthreads();
  if (w == 0) {
    s1 = lane < (int)(blockDim.x >> 5) ? r1[lane] : 0.0;
    s2 = lane < (int)(blockDim.x >> 5) ? r2[lane] : 0.0;
    for (int off = 16; off > 0; off >>= 1) {
      s1 += __shfl_xor_sync(0xffffffffu, s1, off);
      s2 += __shfl_xor_sync(0xffffffffu, s2, off);
    }
    if (lane == 0) {
      sums[z] = s1 / (double)P1;
      sums[n + z] = s2 / (double)P1;
    }
  }
}

// backscatter: out = diss - Cb llp (num / den), num = sum_z Hi mean(psi
// diss), den = sum_z Hi mean(psi llp) + eps
__global__ void k_backscatter(int n, long long P, const double* diss, const double* llp, const double* sums,
                              const double* Hi, double cb, double eps, double* out) {
  double num = 0.0, den = 0.0;
  for (int z = 0; z < n; z++) {
    num += Hi[z] * sums[z];
    den += Hi[z] * sums[n + z];
  }
  const double ratio = num / (den + eps);
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < P; i += (long long)gridDim.x * blockDim.x)
    out[i] = __dsub_rn(diss[i], __dmul_rn(__dmul_rn(cb, llp[i]), ratio));
}

// ring forcing of one plane: m1 = mean(x), m2 = mean(|x - m1|) (one CTA),
// then out[z] = mag keep[z] (x - m1) / m2 for the kept layers and
// mag (0 - 0) / 0 = NaN for the others, as the reference's normalisation of
// an all-zero layer gives
__global__ void k_ring_moments(long long P1, const double* x, double* m) {
  __shared__ double red[32];
  double s = 0.0;
  for (long long i = threadIdx.x; i < P1; i += blockDim.x) s += x[i];
  for (int pass = 0; pass < 2; pass++) {
    for (int off = 16; off > 0; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0) red[w] = s;
    __syncthreads();
    if (w == 0) {
      s = lane < (int)(blockDim.x >> 5) ? red[lane] : 0.0;
      for (int off = 16; off > 0; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
      if (lane == 0) red[0] = s / (double)P1;
    }
    __syncthreads();
    const double mean = red[0];
    if (threadIdx.x == 0) m[pass] = mean;
    __syncthreads();
    if (pass == 0) {
      s = 0.0;
      for (long long i = threadIdx.x; i < P1; i += blockDim.x) s += fabs(x[i] - mean);
    }
  }
}

__global__ void k_ring_apply(int n, long long P1, const double* x, const double* m, const int* keep, double mag,
                             double* out) {
  const double m1 = m[0], m2 = m[1];
  const double nan = __longlong_as_double(0x7ff8000000000000ll);
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n * P1;
       i += (long long)gridDim.x * blockDim.x) {
    const int z = (int)(i / P1);
    out[i] = keep[z] ? __dmul_rn(mag, __ddiv_rn(__dsub_rn(x[i % P1], m1), m2)) : nan;
  }
}

}  // namespace

extern "C" {

PQG_API int pqg_smag_strain(int n, int nl, int nk, const double* kk, const double* ll, const double* uh,
                            const double* vh, double* out3, void* stream) {
  if (n < 1 || nl < 1 || nk < 1 || !kk || !ll || !uh || !vh || !out3)
    return pqg_report_error(PQG_ERR_INVALID, "pqg_smag_strain: bad argument");
  const long long S = (long long)n * nl * nk;
  k_smag_strain<<<blocks_for(S), kThreads, 0, (cudaStream_t)stream>>>(S, nl, nk, kk, ll, uh, vh, out3);
  return launch_check("pqg_smag_strain");
}

PQG_API int pqg_smag_stress(int n, int ny, int nx, const double* s3, double c2dx2, double* nu, double* p3,
                            void* stream) {
  if (n < 1 || ny < 1 || nx < 1 || !s3 || (!nu && !p3))
    return pqg_report_error(PQG_ERR_INVALID, "pqg_smag_stress: bad argument");
  const long long P = (long long)n * ny * nx;
  k_smag_stress<<<blocks_for(P), kThreads, 0, (cudaStream_t)stream>>>(P, s3, c2dx2, nu, p3);
  return launch_check("pqg_smag_stress");
}

PQG_API int pqg_smag_divergence(int n, int nl, int nk, const double* kk, const double* ll, const double* n3,
                                double* out2, void* stream) {
  if (n < 1 || nl < 1 || nk < 1 || !kk || !ll || !n3 || !out2)
    return pqg_report_error(PQG_ERR_INVALID, "pqg_smag_divergence: bad argument");
  const long long S = (long long)n * nl * nk;
  k_smag_div<<<blocks_for(S), kThreads, 0, (cudaStream_t)stream>>>(S, nl, nk, kk, ll, n3, out2);
  return launch_check("pqg_smag_divergence");
}

PQG_API int pqg_zb_gradients(int n, int nl, int nk, const double* kk, const double* ll, const double* uh,
                             const double* vh, double* out4, void* stream) {
  if (n < 1 || nl < 1 || nk < 1 || !kk || !ll || !uh || !vh || !out4)
    return pqg_report_error(PQG_ERR_INVALID, "pqg_zb_gradients: bad argument");
  const long long S = (long long)n * nl * nk;
  k_zb_grad<<<blocks_for(S), kThreads, 0, (cudaStream_t)stream>>>(S, nl, nk, kk, ll, uh, vh, out4);
  return launch_check("pqg_zb_gradients");
}

PQG_API int pqg_zb_products(int n, int ny, int nx, const double* g4, double* out3, void* stream) {
  if (n < 1 || ny < 1 || nx < 1 || !g4 || !out3) return pqg_report_error(PQG_ERR_INVALID, "pqg_zb_products: bad argument");
  const long long P = (long long)n * ny * nx;
  k_zb_prod<<<blocks_for(P), kThreads, 0, (cudaStream_t)stream>>>(P, g4, out3);
  return launch_check("pqg_zb_products");
}

PQG_API int pqg_zb_combine(int n, int nl, int nk, const double* kk, const double* ll, const double* f3, double kappa,
                           double* out2, void* stream) {
  if (n < 1 || nl < 1 || nk < 1 || !kk || !ll || !f3 || !out2)
    return pqg_report_error(PQG_ERR_INVALID, "pqg_zb_combine: bad argument");
  const long long S = (long long)n * nl * nk;
  k_zb_comb<<<blocks_for(S), kThreads, 0, (cudaStream_t)stream>>>(S, nl, nk, kk, ll, f3, kappa, out2);
  return launch_check("pqg_zb_combine");
}

PQG_API int pqg_lap_power(int n, int nl, int nk, const double* kk, const double* ll, int power, double scale,
                          const double* in, double* out, void* stream) {
  if (n < 1 || nl < 1 || nk < 1 || !kk || !ll || !in || !out || (power != 1 && power != 2))
    return pqg_report_error(PQG_ERR_INVALID, "pqg_lap_power: bad argument");
  const long long S = (long long)n * nl * nk;
  k_lap<<<blocks_for(S), kThreads, 0, (cudaStream_t)stream>>>(S, nl, nk, kk, ll, power, scale, in, out);
  return launch_check("pqg_lap_power");
}

PQG_API int pqg_layer_mix(int nout, int nin, long long plane, const double* m, const double* in, double* out,
                          void* stream) {
  if (nout < 1 || nin < 1 || nout > kMixMax || nin > kMixMax || plane < 1 || !m || !in || !out)
    return pqg_report_error(PQG_ERR_INVALID, "pqg_layer_mix: bad argument (at most 8 x 8 layers)");
  Mix mx = {};
  for (int i = 0; i < nout; i++)
    for (int j = 0; j < nin; j++) mx.m[i * kMixMax + j] = m[i * nin + j];
  k_layer_mix<<<blocks_for((long long)nout * plane), kThreads, 0, (cudaStream_t)stream>>>(nout, nin, plane, mx, in,
                                                                                        out);
  return launch_check("pqg_layer_mix");
}

PQG_API int pqg_mul_scaled(long long count, const double* a, double s, const double* b, double* out, void* stream) {
  if (count < 1 || !a || !b || !out) return pqg_report_error(PQG_ERR_INVALID, "pqg_mul_scaled: bad argument");
  k_mul_scaled<<<blocks_for(count), kThreads, 0, (cudaStream_t)stream>>>(count, a, s, b, out);
  return launch_check("pqg_mul_scaled");
}

PQG_API int pqg_backscatter(int n, int ny, int nx, const double* psi, const double* diss, const double* llp,
                            const double* Hi, double cb, double eps, double* sums, double* out, void* stream) {
  if (n < 1 || ny < 1 || nx < 1 || !psi || !diss || !llp || !Hi || !sums || !out)
    return pqg_report_error(PQG_ERR_INVALID, "pqg_backscatter: bad argument");
  const long long P1 = (long long)ny * nx;
  cudaStream_t st = (cudaStream_t)stream;
  k_plane_means<<<n, 1024, 0, st>>>(n, P1, psi, diss, llp, sums);
  int rc = launch_check("pqg_backscatter (means)");
  if (rc) return rc;
  k_backscatter<<<blocks_for(n * P1), kThreads, 0, st>>>(n, n * P1, diss, llp, sums, Hi, cb, eps, out);
  return launch_check("pqg_backscatter");
}

PQG_API int pqg_ring_normalize(int n, int ny, int nx, const double* x, const int* keep, double mag, double* moments,
                               double* out, void* stream) {
  if (n < 1 || ny < 1 || nx < 1 || !x || !keep || !moments || !out)
    return pqg_report_error(PQG_ERR_INVALID, "pqg_ring_normalize: bad argument");
  const long long P1 = (long long)ny * nx;
  cudaStream_t st = (cudaStream_t)stream;
  k_ring_moments<<<1, 1024, 0, st>>>(P1, x, moments);
  int rc = launch_check("pqg_ring_normalize (moments)");
  if (rc) return rc;
  k_ring_apply<<<blocks_for(n * P1), kThreads, 0, st>>>(n, P1, x, moments, keep, mag, out);
  return launch_check("pqg_ring_normalize");
}

}  // extern "C"
