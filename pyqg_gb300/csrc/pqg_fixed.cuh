// 64-bit block-fixed-point FFT engine for sm_103a.
//
// GB300 runs FP64 at 1/58 of its FP32 rate (1.26 TFLOP/s measured), and the
// FFT butterflies are most of the FP64 work of a step.  This engine moves
// the transforms off the FP64 pipe: each sequence (row or column) is scaled
// by a power of two chosen from its largest element and converted to int64,
// the butterflies add exactly in integers, twiddles are Q62 integers and each
// twiddle product is rounded to nearest, and the result is converted back to
// FP64.  Conversions use integer bit operations only.
//
// Precision: a length-n transform keeps 62 - G bits below the sequence's
// largest element, G = log2(n) + 2..4 headroom bits for the growth of the
// transform (no overflow is possible), i.e. 50-52 bits, with exact additions
// and one rounding per twiddle product: normwise errors of the order of an
// FP64 transform's.
#pragma once
#include <cuda_runtime.h>

#include "pqg_fft.cuh"

namespace pqg {
namespace fx {

typedef long long i64;
typedef unsigned long long u64;

constexpr i64 kQ62One = 4611686018427387904LL;       // 2^62
constexpr i64 kQ62H8 = 3260954456333195553LL;        // round(2^62 sqrt(2)/2)
constexpr int kNanShift = -1000000;                  // marks a sequence with Inf/NaN

// round(x * w / 2^62), |w| <= 2^62, ties rounded up: floor((x w + 2^61) / 2^62)
// of the signed 128-bit product.  The product is formed from 32-bit limbs
// with carry chains (mad.lo/hi.cc), the high half corrected for the signs,
// then rounded at bit 61 and shifted by funnel shifts; the lowest partial
// product only feeds the carries, so only its high word is formed.  Equal
// bit for bit to the formulation (u64)x * w for the low and __mul64hi for
// the high half, and measured 17 % faster on sm_103a.
__device__ __forceinline__ i64 q62(i64 x, i64 w) {
  typedef unsigned int u32;
  const u32 x0 = (u32)x, x1 = (u32)((u64)x >> 32), w0 = (u32)w, w1 = (u32)((u64)w >> 32);
  u32 r1, r2, r3;   // words 1..3 of the unsigned product (word 0 does not reach bit 61)
  asm("{\n\t"
      "mul.hi.u32 %0, %3, %5;\n\t"
      "mad.lo.cc.u32 %0, %3, %6, %0;\n\t"
      "madc.hi.u32 %1, %3, %6, 0;\n\t"
      "mad.lo.cc.u32 %0, %4, %5, %0;\n\t"
      "madc.hi.cc.u32 %1, %4, %5, %1;\n\t"
      "madc.hi.u32 %2, %4, %6, 0;\n\t"
      "mad.lo.cc.u32 %1, %4, %6, %1;\n\t"
      "addc.u32 %2, %2, 0;\n\t"
      "}" : "=r"(r1), "=r"(r2), "=r"(r3) : "r"(x0), "r"(x1), "r"(w0), "r"(w1));
  // signed product = unsigned product - 2^64 (x < 0 ? w : 0) - 2^64 (w < 0 ? x : 0)
  u64 hi = ((u64)r3 << 32) | r2;
  hi -= (u64)(w & (x >> 63)) + (u64)(x & (w >> 63));
  u32 lo1 = r1, h0 = (u32)hi, h1 = (u32)(hi >> 32);
  asm("{\n\tadd.cc.u32 %0, %0, 0x20000000;\n\taddc.cc.u32 %1, %1, 0;\n\taddc.u32 %2, %2, 0;\n\t}"
      : "+r"(lo1), "+r"(h0), "+r"(h1));
  return (i64)(((u64)__funnelshift_l(h0, h1, 2) << 32) | __funnelshift_l(lo1, h0, 2));
}

__device__ __forceinline__ longlong2 fadd(longlong2 a, longlong2 b) {
  return make_longlong2(a.x + b.x, a.y + b.y);
}
__device__ __forceinline__ longlong2 fsub(longlong2 a, longlong2 b) {
  return make_longlong2(a.x - b.x, a.y - b.y);
}
template <bool INV>
__device__ __forceinline__ longlong2 frot(longlong2 a) {  // * -i (fwd) / +i (inv)
  return INV ? make_longlong2(-a.y, a.x) : make_longlong2(a.y, -a.x);
}
__device__ __forceinline__ longlong2 fcmul(longlong2 a, longlong2 w) {
  return make_longlong2(q62(a.x, w.x) - q62(a.y, w.y), q62(a.x, w.y) + q62(a.y, w.x));
}
__device__ __forceinline__ longlong2 fcmulc(longlong2 a, longlong2 w) {  // a * conj(w)
  return make_longlong2(q62(a.x, w.x) + q62(a.y, w.y), q62(a.y, w.x) - q62(a.x, w.y));
}

template <int R, bool INV> struct FDft;
template <bool INV> struct FDft<2, INV> {
  static __device__ __forceinline__ void run(longlong2* v) {
    const longlong2 a = v[0], b = v[1];
    v[0] = fadd(a, b);
    v[1] = fsub(a, b);
  }
};
template <bool INV> struct FDft<4, INV> {
  static __device__ __forceinline__ void run(longlong2* v) {
    const longlong2 a = fadd(v[0], v[2]), b = fsub(v[0], v[2]);
    const longlong2 c = fadd(v[1], v[3]), d = frot<INV>(fsub(v[1], v[3]));
    v[0] = fadd(a, c);
    v[2] = fsub(a, c);
    v[1] = fadd(b, d);
    v[3] = fsub(b, d);
  }
};
template <bool INV> struct FDft<8, INV> {
  static __device__ __forceinline__ void run(longlong2* v) {
    longlong2 e[4] = {v[0], v[2], v[4], v[6]};
    longlong2 o[4] = {v[1], v[3], v[5], v[7]};
    FDft<4, INV>::run(e);
    FDft<4, INV>::run(o);
    longlong2 t = o[1];
    o[1] = INV ? make_longlong2(q62(t.x - t.y, kQ62H8), q62(t.x + t.y, kQ62H8))
               : make_longlong2(q62(t.x + t.y, kQ62H8), q62(t.y - t.x, kQ62H8));
    o[2] = frot<INV>(o[2]);
    t = o[3];
    o[3] = INV ? make_longlong2(q62(-(t.x + t.y), kQ62H8), q62(t.x - t.y, kQ62H8))
               : make_longlong2(q62(t.y - t.x, kQ62H8), q62(-(t.x + t.y), kQ62H8));
#pragma unroll
    for (int r = 0; r < 4; r++) {
      v[r] = fadd(e[r], o[r]);
      v[r + 4] = fsub(e[r], o[r]);
    }
  }
};

// One Stockham stage on fixed-point sequences (same indexing as fft_stage).
template <int R, bool INV>
__device__ __forceinline__ void ffft_stage(longlong2* buf, int stride, int nseq, int n, int Ns,
                                           const longlong2* __restrict__ tw, int twstep) {
  constexpr int IT = MaxIt<R>::value;
  const int nb = n / R;
  const int T = blockDim.x;
  const int tid = threadIdx.x;
  const int per_round = max(1, (IT * T) / nb);
  const int tscale = (n / (Ns * R)) * twstep;
  for (int s0 = 0; s0 < nseq; s0 += per_round) {
    const int total = min(per_round, nseq - s0) * nb;
    longlong2 v[IT][R];
#pragma unroll
    for (int it = 0; it < IT; it++) {
      const int p = tid + it * T;
      if (p < total) {
        const int sq = s0 + p / nb, j = p - (p / nb) * nb;
        const longlong2* src = buf + sq * stride + j;
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
            const longlong2 w = tw[r * ts];
            v[it][r] = INV ? fcmulc(v[it][r], w) : fcmul(v[it][r], w);
          }
        }
        FDft<R, INV>::run(v[it]);
        longlong2* dst = buf + sq * stride + (j - jm) * R + jm;
#pragma unroll
        for (int r = 0; r < R; r++) dst[r * Ns] = v[it][r];
      }
    }
    __syncthreads();
  }
}

template <int N, int NS, bool INV>
struct FPow2Fft {
  static constexpr int R = pow2_radix(ilog2(N), ilog2(NS));
  static __device__ __forceinline__ void run(longlong2* buf, int stride, int nseq,
                                             const longlong2* __restrict__ tw, int twstep) {
    ffft_stage<R, INV>(buf, stride, nseq, N, NS, tw, twstep);
    FPow2Fft<N, NS * R, INV>::run(buf, stride, nseq, tw, twstep);
  }
};
template <int N, bool INV>
struct FPow2Fft<N, N, INV> {
  static __device__ __forceinline__ void run(longlong2*, int, int, const longlong2*, int) {}
};

// ---------------------------------------------------------------------------
// conversions (integer bit operations only)
// ---------------------------------------------------------------------------

// biased binary exponent of max(|v.x|, |v.y|) (2047 for Inf/NaN)
__device__ __forceinline__ int bexp(double2 v) {
  const u64 a = (u64)__double_as_longlong(v.x) & 0x7fffffffffffffffull;
  const u64 b = (u64)__double_as_longlong(v.y) & 0x7fffffffffffffffull;
  return (int)((a > b ? a : b) >> 52);
}
__device__ __forceinline__ int bexp1(double v) {
  return (int)(((u64)__double_as_longlong(v) & 0x7fffffffffffffffull) >> 52);
}

// Power-of-two shift S for a sequence whose largest biased exponent is emax:
// |v| 2^S < 2^(62 - G) for every element.
__device__ __forceinline__ int block_shift(int emax, int G) {
  return emax >= 2047 ? kNanShift : 1084 - G - emax;
}

// round(v * 2^S) as int64 (ties away from zero)
__device__ __forceinline__ i64 to_fixed(double v, int S) {
  const u64 b = (u64)__double_as_longlong(v);
  int E = (int)((b >> 52) & 0x7ff);
  u64 m = b & 0xfffffffffffffull;
  if (E) m |= (1ull << 52); else E = 1;
  const int k = E - 1075 + S;
  i64 r;
  if (k >= 0) {
    r = (i64)(m << (k > 10 ? 10 : k));
  } else {
    const int sh = -k;
    r = sh >= 63 ? 0 : (i64)((m + (1ull << (sh - 1))) >> sh);
  }
  return (b >> 63) ? -r : r;
}

// f * 2^-S as a double, rounded to nearest even (results below the normal
// range flush to zero)
__device__ __forceinline__ double from_fixed(i64 f, int S) {
  if (S == kNanShift) return __longlong_as_double(0x7ff8000000000000LL);
  if (f == 0) return 0.0;
  const u64 sign = f < 0 ? (1ull << 63) : 0ull;
  const u64 a = f < 0 ? (u64)(-f) : (u64)f;
  const int lz = __clzll((i64)a);
  const u64 n = a << lz;                  // leading one at bit 63
  u64 mant = n >> 11;                     // 53 bits
  const u64 rem = n & 0x7ffull;
  if (rem > 0x400ull || (rem == 0x400ull && (mant & 1ull))) mant++;
  int e = 63 - lz - S;
  if (mant == (1ull << 53)) { mant >>= 1; e++; }
  const int E = e + 1023;
  if (E <= 0) return sign ? -0.0 : 0.0;
  return __longlong_as_double((i64)(sign | ((u64)E << 52) | (mant & 0xfffffffffffffull)));
}

// Max biased exponent per sequence of `nseq` double2 sequences of length n
// at buf + s*stride into ex[s] (shared).  All threads call; ends synced.
__device__ __forceinline__ void seq_max_exp(const double2* buf, int stride, int nseq, int n, int* ex) {
  for (int i = threadIdx.x; i < nseq; i += blockDim.x) ex[i] = 0;
  __syncthreads();
  const int total = nseq * n;
  const int lane = threadIdx.x & 31;
  for (int t0 = threadIdx.x - lane; t0 < total; t0 += blockDim.x) {
    const int t = t0 + lane;
    int s = -1, e = 0;
    if (t < total) {
      s = t / n;
      e = bexp(buf[s * stride + (t - s * n)]);
    }
    const int s0 = __shfl_sync(0xffffffffu, s, 0);
    if (__all_sync(0xffffffffu, s == s0 || s < 0)) {
      const int m = __reduce_max_sync(0xffffffffu, e);
      if (lane == 0 && s0 >= 0) atomicMax(&ex[s0], m);
    } else if (s >= 0) {
      atomicMax(&ex[s], e);
    }
  }
  __syncthreads();
}

// In place double2 -> fixed of `nseq` sequences with shifts sh[s].
__device__ __forceinline__ void seq_to_fixed(double2* buf, int stride, int nseq, int n, const int* sh) {
  for (int t = threadIdx.x; t < nseq * n; t += blockDim.x) {
    const int s = t / n, j = t - s * n;
    double2* p = buf + s * stride + j;
    const double2 v = *p;
    const int S = sh[s];
    *reinterpret_cast<longlong2*>(p) = S == kNanShift ? make_longlong2(0, 0)
                                                      : make_longlong2(to_fixed(v.x, S), to_fixed(v.y, S));
  }
  __syncthreads();
}

// In place fixed -> double2 with shifts sh[s] + extra.
__device__ __forceinline__ void seq_from_fixed(double2* buf, int stride, int nseq, int n, const int* sh,
                                               int extra) {
  for (int t = threadIdx.x; t < nseq * n; t += blockDim.x) {
    const int s = t / n, j = t - s * n;
    double2* p = buf + s * stride + j;
    const longlong2 f = *reinterpret_cast<const longlong2*>(p);
    const int S = sh[s] == kNanShift ? kNanShift : sh[s] + extra;
    *p = make_double2(from_fixed(f.x, S), from_fixed(f.y, S));
  }
  __syncthreads();
}

}  // namespace fx
}  // namespace pqg
