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
  static __device__ __forceinline__ void run(double2* v) {
    double2 a = v[0], b = v[1];
    v[0] = cadd(a, b);
    v[1] = csub(a, b);
  }
};

template <bool INV> struct Dft<4, INV> {
  static __device__ __forceinline__ void run(double2* v) {
    double2 a = cadd(v[0], v[2]), b = csub(v[0], v[2]);
    double2 c = cadd(v[1], v[3]), d = rot<INV>(csub(v[1], v[3]));
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
  static __device__ __forceinline__ void run(double2* v) {
    double2 e[4] = {v[0], v[2], v[4], v[6]};
    double2 o[4] = {v[1], v[3], v[5], v[7]};
    Dft<4, INV>::run(e);
    Dft<4, INV>::run(o);
    // o1 *= w8, o2 *= w8^2 (= -+i), o3 *= w8^3, w8 = exp(-+ i pi / 4)
    double2 t = o[1];
    o[1] = INV ? make_double2(__dmul_rn(__dsub_rn(t.x, t.y), kSqrt2_2),
                              __dmul_rn(__dadd_rn(t.x, t.y), kSqrt2_2))
               : make_double2(__dmul_rn(__dadd_rn(t.x, t.y), kSqrt2_2),
                              __dmul_rn(__dsub_rn(t.y, t.x), kSqrt2_2));
    o[2] = rot<INV>(o[2]);
    t = o[3];
    o[3] = INV ? make_double2(__dmul_rn(-__dadd_rn(t.x, t.y), kSqrt2_2),
                              __dmul_rn(__dsub_rn(t.x, t.y), kSqrt2_2))
               : make_double2(__dmul_rn(__dsub_rn(t.y, t.x), kSqrt2_2),
                              __dmul_rn(-__dadd_rn(t.x, t.y), kSqrt2_2));
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
template <int R, bool INV>
__device__ __forceinline__ void fft_stage(double2* buf, int stride, int nseq,
                                          int n, int Ns,
                                          const double2* __restrict__ tw,
                                          int twstep) {
  constexpr int IT = MaxIt<R>::value;
  const int nb = n / R;
  const int T = blockDim.x;
  const int tid = threadIdx.x;
  const int per_round = max(1, (IT * T) / nb);
  const int tscale = (n / (Ns * R)) * twstep;
  for (int s0 = 0; s0 < nseq; s0 += per_round) {
    const int total = min(per_round, nseq - s0) * nb;
    double2 v[IT][R];
#pragma unroll
    for (int it = 0; it < IT; it++) {
      const int p = tid + it * T;
      if (p < total) {
        const int sq = s0 + p / nb, j = p - (p / nb) * nb;
        const double2* src = buf + sq * stride + j;
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
            const double2 w = tw[r * ts];
            v[it][r] = INV ? cmulc(v[it][r], w) : cmul(v[it][r], w);
          }
        }
        Dft<R, INV>::run(v[it]);
        double2* dst = buf + sq * stride + (j - jm) * R + jm;
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

template <int N, int NS, bool INV>
struct Pow2Fft {
  static constexpr int R = pow2_radix(ilog2(N), ilog2(NS));
  static __device__ __forceinline__ void run(double2* buf, int stride, int nseq,
                                             const double2* __restrict__ tw, int twstep) {
    fft_stage<R, INV>(buf, stride, nseq, N, NS, tw, twstep);
    Pow2Fft<N, NS * R, INV>::run(buf, stride, nseq, tw, twstep);
  }
};
template <int N, bool INV>
struct Pow2Fft<N, N, INV> {
  static __device__ __forceinline__ void run(double2*, int, int, const double2*, int) {}
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
__device__ __forceinline__ void c2r_pre(const double2* __restrict__ X,
                                        double2* z, int M, int k,
                                        const double2* __restrict__ tw) {
  if (k == 0) {
    const double x0 = X[0].x, xm = X[M].x;
    z[0] = make_double2(__dadd_rn(x0, xm), __dsub_rn(x0, xm));
    return;
  }
  const double2 a = X[k], bb = X[M - k];
  const double2 b = make_double2(bb.x, -bb.y);
  const double2 A = cadd(a, b), B = csub(a, b);
  const double2 D = cmulc(B, tw[k]);
  z[k] = make_double2(__dsub_rn(A.x, D.y), __dadd_rn(A.y, D.x));
  if (k != M - k) z[M - k] = make_double2(__dadd_rn(A.x, D.y), __dsub_rn(D.x, A.y));
}

// R2C post-processing, task k in [0, M/2]: from Z = FFT_M(x[2m] + i x[2m+1])
// (shared) write the half spectrum X[k], X[M-k] (and X[0], X[M] for k = 0).
__device__ __forceinline__ void r2c_post(const double2* z,
                                         double2* __restrict__ X, int M, int k,
                                         const double2* __restrict__ tw) {
  if (k == 0) {
    const double2 z0 = z[0];
    X[0] = make_double2(__dadd_rn(z0.x, z0.y), 0.0);
    X[M] = make_double2(__dsub_rn(z0.x, z0.y), 0.0);
    return;
  }
  const double2 a = z[k], bb = z[M - k];
  const double2 b = make_double2(bb.x, -bb.y);
  const double2 A = cadd(a, b), B = csub(a, b);
  const double2 C = cmul(B, tw[k]);
  X[k] = make_double2(__dmul_rn(0.5, __dadd_rn(A.x, C.y)),
                      __dmul_rn(0.5, __dsub_rn(A.y, C.x)));
  if (k != M - k)
    X[M - k] = make_double2(__dmul_rn(0.5, __dsub_rn(A.x, C.y)),
                            __dmul_rn(-0.5, __dadd_rn(A.y, C.x)));
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
