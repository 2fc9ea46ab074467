// Device building blocks of the FP64 pseudo-spectral step on sm_103a:
// complex arithmetic with pinned rounding, radix-2/3/4/5/8 DFT kernels, and a
// mixed-radix Stockham FFT that transforms a batch of sequences held in
// shared memory by the whole thread block.
//
// Rounding is pinned with explicit intrinsics (__dadd_rn, __dmul_rn,
// __fma_rn) so that every kernel that shares these functions produces
// bit-identical results, whether the stages run one kernel per reference
// method or fused two kernels per step.
#pragma once
#include <cuda_runtime.h>

namespace pqg {

constexpr int kMaxStages = 16;

// Radix plan of one complex FFT length: n = prod of the stage radices,
// stage s radix = (code >> 4s) & 15 (kept in registers, no local arrays).
struct FftDesc {
  int n;
  int nst;
  unsigned long long code;
  __host__ __device__ int radix(int s) const { return (int)((code >> (4 * s)) & 15ull); }
};

// ---------------------------------------------------------------------------
// complex helpers (double2 = re, im)
// ---------------------------------------------------------------------------
__device__ __forceinline__ double2 cadd(double2 a, double2 b) {
  return make_double2(__dadd_rn(a.x, b.x), __dadd_rn(a.y, b.y));
}
__device__ __forceinline__ double2 csub(double2 a, double2 b) {
  return make_double2(__dsub_rn(a.x, b.x), __dsub_rn(a.y, b.y));
}
__device__ __forceinline__ double2 cscale(double2 a, double s) {
  return make_double2(__dmul_rn(a.x, s), __dmul_rn(a.y, s));
}
// a * w
__device__ __forceinline__ double2 cmul(double2 a, double2 w) {
  return make_double2(__fma_rn(a.x, w.x, -__dmul_rn(a.y, w.y)),
                      __fma_rn(a.x, w.y, __dmul_rn(a.y, w.x)));
}
// a * conj(w)
__device__ __forceinline__ double2 cmulc(double2 a, double2 w) {
  return make_double2(__fma_rn(a.x, w.x, __dmul_rn(a.y, w.y)),
                      __fma_rn(a.y, w.x, -__dmul_rn(a.x, w.y)));
}
// multiply by -i (forward) or +i (inverse)
template <bool INV>
__device__ __forceinline__ double2 rot(double2 a) {
  return INV ? make_double2(-a.y, a.x) : make_double2(a.y, -a.x);
}

// Scalar operations with pinned rounding, overloaded on the precision, and
// the float2 (FP32) counterparts of the complex helpers above.
__device__ __forceinline__ double sadd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double ssub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double smul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double sfma(double a, double b, double c) { return __fma_rn(a, b, c); }
__device__ __forceinline__ float sadd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float ssub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float smul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float sfma(float a, float b, float c) { return __fmaf_rn(a, b, c); }
__device__ __forceinline__ double2 mk(double x, double y) { return make_double2(x, y); }
__device__ __forceinline__ float2 mk(float x, float y) { return make_float2(x, y); }

__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(__fadd_rn(a.x, b.x), __fadd_rn(a.y, b.y)); }
__device__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(__fsub_rn(a.x, b.x), __fsub_rn(a.y, b.y)); }
__device__ __forceinline__ float2 cscale(float2 a, float s) { return make_float2(__fmul_rn(a.x, s), __fmul_rn(a.y, s)); }
__device__ __forceinline__ float2 cmul(float2 a, float2 w) {
  return make_float2(__fmaf_rn(a.x, w.x, -__fmul_rn(a.y, w.y)), __fmaf_rn(a.x, w.y, __fmul_rn(a.y, w.x)));
}
__device__ __forceinline__ float2 cmulc(float2 a, float2 w) {
  return make_float2(__fmaf_rn(a.x, w.x, __fmul_rn(a.y, w.y)), __fmaf_rn(a.y, w.x, -__fmul_rn(a.x, w.y)));
}
template <bool INV>
__device__ __forceinline__ float2 rot(float2 a) {
  return INV ? make_float2(-a.y, a.x) : make_float2(a.y, -a.x);
}

// Correctly rounded constants.
constexpr double kSqrt3_2 = 0x1.bb67ae8584caap-1;  // sin(2 pi / 3)
constexpr double kSqrt2_2 = 0x1.6a09e667f3bcdp-1;  // cos(pi / 4)
constexpr double kC5_1 = 0x1.3c6ef372fe950p-2;     // cos(2 pi / 5)
constexpr double kC5_2 = -0x1.9e3779b97f4a8p-1;    // cos(4 pi / 5)
constexpr double kS5_1 = 0x1.e6f0e134454ffp-1;     // sin(2 pi / 5)
constexpr double kS5_2 = 0x1.2cf2304755a5ep-1;     // sin(4 pi / 5)

// ---------------------------------------------------------------------------
// radix-R DFTs in registers: v[r] <- sum_q v[q] exp(-+2 pi i q r / R)
// ---------------------------------------------------------------------------
template <int R, bool INV> struct Dft;

template <bool INV> struct Dft<2, INV> {
  template <class V>
  static __device__ __forceinline__ void run(V* v) {
    V a = v[0], b = v[1];
    v[0] = cadd(a, b);
    v[1] = csub(a, b);
  }
};

template <bool INV> struct Dft<4, INV> {
  template <class V>
  static __device__ __forceinline__ void run(V* v) {
    V a = cadd(v[0], v[2]), b = csub(v[0], v[2]);
    V c = cadd(v[1], v[3]), d = rot<INV>(csub(v[1], v[3]));
    v[0] = cadd(a, c);
    v[2] = csub(a, c);
    v[1] = cadd(b, d);
    v[3] = csub(b, d);
  }
};

template <bool INV> struct Dft<3, INV> {
  static __device__ __forceinline__ void run(double2* v) {
    double2 t1 = cadd(v[1], v[2]);
    double2 t2 = make_double2(__fma_rn(-0.5, t1.x, v[0].x),
                              __fma_rn(-0.5, t1.y, v[0].y));
    double2 d = rot<INV>(cscale(csub(v[1], v[2]), kSqrt3_2));
    v[0] = cadd(v[0], t1);
    v[1] = cadd(t2, d);
    v[2] = csub(t2, d);
  }
};

template <bool INV> struct Dft<5, INV> {
  static __device__ __forceinline__ void run(double2* v) {
    double2 a1 = cadd(v[1], v[4]), b1 = csub(v[1], v[4]);
    double2 a2 = cadd(v[2], v[3]), b2 = csub(v[2], v[3]);
    double2 x0 = v[0];
    double2 A = make_double2(__fma_rn(kC5_2, a2.x, __fma_rn(kC5_1, a1.x, x0.x)),
                             __fma_rn(kC5_2, a2.y, __fma_rn(kC5_1, a1.y, x0.y)));
    double2 C = make_double2(__fma_rn(kC5_1, a2.x, __fma_rn(kC5_2, a1.x, x0.x)),
                             __fma_rn(kC5_1, a2.y, __fma_rn(kC5_2, a1.y, x0.y)));
    double2 B = make_double2(__fma_rn(kS5_2, b2.x, __dmul_rn(kS5_1, b1.x)),
                             __fma_rn(kS5_2, b2.y, __dmul_rn(kS5_1, b1.y)));
    double2 D = make_double2(__fma_rn(-kS5_1, b2.x, __dmul_rn(kS5_2, b1.x)),
                             __fma_rn(-kS5_1, b2.y, __dmul_rn(kS5_2, b1.y)));
    B = rot<INV>(B);
    D = rot<INV>(D);
    v[0] = cadd(x0, cadd(a1, a2));
    v[1] = cadd(A, B);
    v[4] = csub(A, B);
    v[2] = cadd(C, D);
    v[3] = csub(C, D);
  }
};

template <bool INV> struct Dft<8, INV> {
  template <class V>
  static __device__ __forceinline__ void run(V* v) {
    typedef decltype(v[0].x) S;
    const S h = (S)kSqrt2_2;
    V e[4] = {v[0], v[2], v[4], v[6]};
    V o[4] = {v[1], v[3], v[5], v[7]};
    Dft<4, INV>::run(e);
    Dft<4, INV>::run(o);
    // o1 *= w8, o2 *= w8^2 (= -+i), o3 *= w8^3, w8 = exp(-+ i pi / 4)
    V t = o[1];
    o[1] = INV ? mk(smul(ssub(t.x, t.y), h), smul(sadd(t.x, t.y), h))
               : mk(smul(sadd(t.x, t.y), h), smul(ssub(t.y, t.x), h));
    o[2] = rot<INV>(o[2]);
    t = o[3];
    o[3] = INV ? mk(smul(-sadd(t.x, t.y), h), smul(ssub(t.x, t.y), h))
               : mk(smul(ssub(t.y, t.x), h), smul(-sadd(t.x, t.y), h));
#pragma unroll
    for (int r = 0; r < 4; r++) {
      v[r] = cadd(e[r], o[r]);
      v[r + 4] = csub(e[r], o[r]);
    }
  }
};

// Butterflies a thread keeps in registers per stage for radix R: the block
// must satisfy blockDim.x * MaxIt<R> >= n / R for every stage.
template <int R> struct MaxIt { static constexpr int value = R == 2 ? 4 : (R == 8 || R == 5 ? 1 : 2); };
// (blockDim >= n / 8 covers radix 2, 4 and 8 stages; radix 3 needs n / 6,
// radix 5 needs n / 5)

// One Stockham stage (radix R, Ns = product of earlier radices) on `nseq`
// sequences of length n at buf + s*stride, in place through registers.
// Twiddles come from a table tw[m*twstep] = exp(-2 pi i m / n).
template <int R, bool INV, class V>
__device__ __forceinline__ void fft_stage(V* buf, int stride, int nseq,
                                          int n, int Ns,
                                          const V* __restrict__ tw,
                                          int twstep) {
  constexpr int IT = MaxIt<R>::value;
  const int nb = n / R;
  const int T = blockDim.x;
  const int tid = threadIdx.x;
  const int per_round = max(1, (IT * T) / nb);
  const int tscale = (n / (Ns * R)) * twstep;
  for (int s0 = 0; s0 < nseq; s0 += per_round) {
    const int total = min(per_round, nseq - s0) * nb;
    V v[IT][R];
#pragma unroll
    for (int it = 0; it < IT; it++) {
      const int p = tid + it * T;
      if (p < total) {
        const int sq = s0 + p / nb, j = p - (p / nb) * nb;
        const V* src = buf + sq * stride + j;
#pragma unroll
        for (int r = 0; r < R; r++) v[it][r] = src[r * nb];
      }
    }
    __syncthreads();
#pragma unroll
    for (int it = 0; it < IT; it++) {
      const int p = tid + it * T;
      if (p < total) {
        const int sq = s0 + p / nb, j = p - (p / nb) * nb;
        const int jm = j % Ns;
        if (Ns > 1) {
          const int ts = tscale * jm;
#pragma unroll
          for (int r = 1; r < R; r++) {
            const V w = tw[r * ts];
            v[it][r] = INV ? cmulc(v[it][r], w) : cmul(v[it][r], w);
          }
        }
        Dft<R, INV>::run(v[it]);
        V* dst = buf + sq * stride + (j - jm) * R + jm;
#pragma unroll
        for (int r = 0; r < R; r++) dst[r * Ns] = v[it][r];
      }
    }
    __syncthreads();
  }
}

// Unnormalised complex FFT (forward: exp(-2 pi i ...), inverse: exp(+...))
// of `nseq` sequences in shared memory.  All threads of the block must call.
template <bool INV>
__device__ void fft_run(double2* buf, int stride, int nseq, const FftDesc& d,
                        const double2* __restrict__ tw, int twstep) {
  int Ns = 1;
  for (int s = 0; s < d.nst; s++) {
    const int R = d.radix(s);
    switch (R) {
      case 2: fft_stage<2, INV>(buf, stride, nseq, d.n, Ns, tw, twstep); break;
      case 3: fft_stage<3, INV>(buf, stride, nseq, d.n, Ns, tw, twstep); break;
      case 4: fft_stage<4, INV>(buf, stride, nseq, d.n, Ns, tw, twstep); break;
      case 5: fft_stage<5, INV>(buf, stride, nseq, d.n, Ns, tw, twstep); break;
      default: fft_stage<8, INV>(buf, stride, nseq, d.n, Ns, tw, twstep); break;
    }
    Ns *= R;
  }
}

// ---------------------------------------------------------------------------
// Compile-time plans for power-of-two lengths n = 2^a: radix 8 stages, then
// radix 4 (two instead of a final 8*2), then a radix 2 only for n = 2, 8*2...
// The host-side factorisation produces the same radix order, so the runtime
// and compile-time paths run the same stages and give identical results.
// ---------------------------------------------------------------------------
__host__ __device__ constexpr int pow2_eights(int a) { return (a % 3 == 1 && a >= 4) ? a / 3 - 1 : a / 3; }
__host__ __device__ constexpr int pow2_fours(int a) { return (a % 3 == 1) ? (a >= 4 ? 2 : 0) : (a % 3 == 2 ? 1 : 0); }
__host__ __device__ constexpr int pow2_radix(int a, int s) {
  // radix of the stage that starts at Ns = 2^s
  return s < 3 * pow2_eights(a) ? 8 : (s < 3 * pow2_eights(a) + 2 * pow2_fours(a) ? 4 : 2);
}
__host__ __device__ constexpr int ilog2(int n) { return n <= 1 ? 0 : 1 + ilog2(n / 2); }

template <int N, int NS, bool INV, class V = double2>
struct Pow2Fft {
  static constexpr int R = pow2_radix(ilog2(N), ilog2(NS));
  static __device__ __forceinline__ void run(V* buf, int stride, int nseq,
                                             const V* __restrict__ tw, int twstep) {
    fft_stage<R, INV>(buf, stride, nseq, N, NS, tw, twstep);
    Pow2Fft<N, NS * R, INV, V>::run(buf, stride, nseq, tw, twstep);
  }
};
template <int N, bool INV, class V>
struct Pow2Fft<N, N, INV, V> {
  static __device__ __forceinline__ void run(V*, int, int, const V*, int) {}
};

// FFT engines used as kernel template arguments: a runtime mixed-radix plan,
// or a compile-time power-of-two plan of length 2^LOGN.
struct FftRuntime {
  template <bool INV>
  static __device__ __forceinline__ void run(double2* buf, int stride, int nseq, const FftDesc& d,
                                             const double2* __restrict__ tw, int twstep) {
    fft_run<INV>(buf, stride, nseq, d, tw, twstep);
  }
};
template <int LOGN>
struct FftPow2 {
  template <bool INV>
  static __device__ __forceinline__ void run(double2* buf, int stride, int nseq, const FftDesc&,
                                             const double2* __restrict__ tw, int twstep) {
    Pow2Fft<(1 << LOGN), 1, INV>::run(buf, stride, nseq, tw, twstep);
  }
};

// ---------------------------------------------------------------------------
// real <-> half-length complex packing for the row transforms (length N = 2M)
// tw is the length-N table exp(-2 pi i m / N).
// ---------------------------------------------------------------------------

// C2R pre-processing, task k in [0, M/2]: from the half spectrum X[0..M]
// (global) build Z'[k] and Z'[M-k] such that the unnormalised inverse
// length-M FFT of Z' gives N * (x[2m] + i x[2m+1]).  The imaginary parts of
// X[0] and X[M] are ignored (numpy.fft.irfft / FFTW c2r behaviour).
template <class V>
__device__ __forceinline__ void c2r_pre(const V* __restrict__ X,
                                        V* z, int M, int k,
                                        const V* __restrict__ tw) {
  if (k == 0) {
    const auto x0 = X[0].x, xm = X[M].x;
    z[0] = mk(sadd(x0, xm), ssub(x0, xm));
    return;
  }
  const V a = X[k], bb = X[M - k];
  const V b = mk(bb.x, -bb.y);
  const V A = cadd(a, b), B = csub(a, b);
  const V D = cmulc(B, tw[k]);
  z[k] = mk(ssub(A.x, D.y), sadd(A.y, D.x));
  if (k != M - k) z[M - k] = mk(sadd(A.x, D.y), ssub(D.x, A.y));
}

// R2C post-processing, task k in [0, M/2]: from Z = FFT_M(x[2m] + i x[2m+1])
// (shared) write the half spectrum X[k], X[M-k] (and X[0], X[M] for k = 0).
template <class V>
__device__ __forceinline__ void r2c_post(const V* z,
                                         V* __restrict__ X, int M, int k,
                                         const V* __restrict__ tw) {
  typedef decltype(z[0].x) S;
  const S half = (S)0.5;
  if (k == 0) {
    const V z0 = z[0];
    X[0] = mk(sadd(z0.x, z0.y), (S)0);
    X[M] = mk(ssub(z0.x, z0.y), (S)0);
    return;
  }
  const V a = z[k], bb = z[M - k];
  const V b = mk(bb.x, -bb.y);
  const V A = cadd(a, b), B = csub(a, b);
  const V C = cmul(B, tw[k]);
  X[k] = mk(smul(half, sadd(A.x, C.y)), smul(half, ssub(A.y, C.x)));
  if (k != M - k)
    X[M - k] = mk(smul(half, ssub(A.x, C.y)), smul(-half, sadd(A.y, C.x)));
}

// The same packing with the half spectrum at stride `sx` (X[k * sx]), for
// layouts where a row's spectral values are not contiguous.
template <class V>
__device__ __forceinline__ void c2r_pre_s(const V* __restrict__ X, int sx, V* z, int M, int k,
                                          const V* __restrict__ tw) {
  if (k == 0) {
    const auto x0 = X[0].x, xm = X[(size_t)M * sx].x;
    z[0] = mk(sadd(x0, xm), ssub(x0, xm));
    return;
  }
  const V a = X[(size_t)k * sx], bb = X[(size_t)(M - k) * sx];
  const V b = mk(bb.x, -bb.y);
  const V A = cadd(a, b), B = csub(a, b);
  const V D = cmulc(B, tw[k]);
  z[k] = mk(ssub(A.x, D.y), sadd(A.y, D.x));
  if (k != M - k) z[M - k] = mk(sadd(A.x, D.y), ssub(D.x, A.y));
}

template <class V>
__device__ __forceinline__ void r2c_post_s(const V* z, V* __restrict__ X, int sx, int M, int k,
                                           const V* __restrict__ tw) {
  typedef decltype(z[0].x) S;
  const S half = (S)0.5;
  if (k == 0) {
    const V z0 = z[0];
    X[0] = mk(sadd(z0.x, z0.y), (S)0);
    X[(size_t)M * sx] = mk(ssub(z0.x, z0.y), (S)0);
    return;
  }
  const V a = z[k], bb = z[M - k];
  const V b = mk(bb.x, -bb.y);
  const V A = cadd(a, b), B = csub(a, b);
  const V C = cmul(B, tw[k]);
  X[(size_t)k * sx] = mk(smul(half, sadd(A.x, C.y)), smul(half, ssub(A.y, C.x)));
  if (k != M - k)
    X[(size_t)(M - k) * sx] = mk(smul(half, ssub(A.x, C.y)), smul(-half, sadd(A.y, C.x)));
}

// ---------------------------------------------------------------------------
// pointwise physics (reference expressions, evaluated with fused
// multiply-adds; complex products with purely real / imaginary factors
// reduce to the real products below)
// ---------------------------------------------------------------------------

// ph = sum_{z'} a[z, z'] qh[z'] accumulated from zero in z' order
// (pyqg/kernel.pyx:323-338).
__device__ __forceinline__ double2 ph_acc(double2 acc, double a, double2 qh) {
  return make_double2(__fma_rn(a, qh.x, acc.x), __fma_rn(a, qh.y, acc.y));
}
// uh = -il ph (pyqg/kernel.pyx:346)
__device__ __forceinline__ double2 uh_of(double l, double2 ph) {
  return make_double2(__dmul_rn(l, ph.y), -__dmul_rn(l, ph.x));
}
// vh = ik ph (pyqg/kernel.pyx:347)
__device__ __forceinline__ double2 vh_of(double k, double2 ph) {
  return make_double2(-__dmul_rn(k, ph.y), __dmul_rn(k, ph.x));
}
// dqhdt = -(ik uqh + il vqh + ikQy ph) (pyqg/kernel.pyx:392-394)
__device__ __forceinline__ double2 tendency(double k, double l, double kQy,
                                            double2 uqh, double2 vqh,
                                            double2 ph) {
  const double re = __fma_rn(kQy, ph.y, __fma_rn(l, vqh.y, __dmul_rn(k, uqh.y)));
  const double im = __fma_rn(kQy, ph.x, __fma_rn(l, vqh.x, __dmul_rn(k, uqh.x)));
  return make_double2(re, -im);
}
// dqhdt += (rek k2l2) ph (pyqg/kernel.pyx:456-460)
__device__ __forceinline__ double2 friction(double2 dq, double rk2, double2 ph) {
  return make_double2(__fma_rn(rk2, ph.x, dq.x), __fma_rn(rk2, ph.y, dq.y));
}
// dqhdt += -il duh + ik dvh (pyqg/kernel.pyx:417-421)
__device__ __forceinline__ double2 uv_curl_add(double2 dq, double k, double l,
                                               double2 duh, double2 dvh) {
  // -il duh = (l duh.y, -l duh.x); ik dvh = (-k dvh.y, k dvh.x)
  const double re = __fma_rn(-k, dvh.y, __dmul_rn(l, duh.y));
  const double im = __fma_rn(k, dvh.x, -__dmul_rn(l, duh.x));
  return make_double2(__dadd_rn(dq.x, re), __dadd_rn(dq.y, im));
}
// qh_new = filtr (qh + c1 dq + c2 dq_p + c3 dq_pp) (pyqg/kernel.pyx:502-507)
__device__ __forceinline__ double2 ab_update(double f, double2 qh, double2 dq,
                                             double2 dqp, double2 dqpp,
                                             double c1, double c2, double c3) {
  const double re = __fma_rn(c3, dqpp.x, __fma_rn(c2, dqp.x, __fma_rn(c1, dq.x, qh.x)));
  const double im = __fma_rn(c3, dqpp.y, __fma_rn(c2, dqp.y, __fma_rn(c1, dq.y, qh.y)));
  return make_double2(__dmul_rn(f, re), __dmul_rn(f, im));
}

}  // namespace pqg
