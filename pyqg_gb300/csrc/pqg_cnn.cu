// pqg_cnn.cu -- the learned subgrid closure: a fully convolutional network of
// 5x5 periodic convolutions with ReLU between layers, run on the tcgen05
// tensor cores in BF16 with FP32 accumulation in TMEM, trained with Adam.
//
// No counterpart in the reference; it plugs into the model through the
// q_parameterization hook (pyqg/model.py:203-212, pyqg/kernel.pyx:424-442).
//
// Every convolution is an implicit GEMM over K = (tap, channel):
//   forward  out[p][co] = sum_{tap,ci} in[p + off(tap)][ci] w[co][tap][ci]
//   dgrad    din[p][ci] = sum_{tap,co} g[p + off(tap)][co] w[co][24-tap][ci]
//            (the forward kernel with flipped, channel-transposed weights)
//   wgrad    dw[co][tap][ci] = sum_p x[p + off(tap)][ci] g[p][co]
// with off(tap) = (tap / 5 - 2, tap % 5 - 2) taken periodically.
// Activations are NHWC BF16 (channels contiguous); master weights are FP32
// w[co][tap][ci]; packed BF16 copies hold each K chunk of 64 as one
// contiguous block in the tensor core's K-major core-matrix layout.
//
// A CTA of 128 threads owns a tile of 128 rows (pixels for forward/dgrad,
// (tap, channel) pairs for wgrad) and all N columns.  K advances in chunks of
// 64 through two shared-memory stages: the threads gather a chunk, one
// thread issues four 128xNx16 MMAs and commits them to the stage's mbarrier,
// and the stage is refilled once that barrier completes.  The epilogue reads
// the accumulator with tcgen05.ld (warp w owns TMEM lanes 32w..32w+31).
#include <cuda_runtime.h>
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "pyqg_gb300.h"
#include "pqg_tc.cuh"

#define PQG_API __attribute__((visibility("default")))

typedef __nv_bfloat16 bf16;
namespace tc = pqg::tc;

namespace {

constexpr int KC = 64;     // K elements per chunk
constexpr int TM = 128;    // tile rows
constexpr int NTAP = 25;   // 5 x 5 taps
constexpr int CHUNK_A = TM * KC * 2;   // bytes of one A stage

thread_local std::string c_last_error;

int cfail(int code, const std::string& msg) {
  c_last_error = msg;
  return code;
}

#define CCUDA(call)                                                                  \
  do {                                                                               \
    cudaError_t _e = (call);                                                         \
    if (_e != cudaSuccess) return cfail(PQG_ERR_CUDA, std::string(#call ": ") + cudaGetErrorString(_e)); \
  } while (0)

__host__ __device__ inline int pad16(int n) { return (n + 15) & ~15; }

__device__ __forceinline__ int wrap(int i, int n) { return i < 0 ? i + n : (i >= n ? i - n : i); }

// ---------------------------------------------------------------------------
// forward / dgrad convolution
// ---------------------------------------------------------------------------
struct ConvArgs {
  const bf16* in;        // NHWC, cin channels
  int cin;
  const bf16* wpk;       // nchunk blocks of N x KC (K-major core matrices)
  int N, nchunk, cout;   // N = pad16(cout)
  const float* bias;     // (cout) or null
  int H, W, npix;
  int mode;              // 0: bias+ReLU -> out_bf; 1: affine -> out (NCHW); 2: ReLU mask -> out_bf
  bf16* out_bf;          // NHWC, cout channels (cout multiple of 8)
  void* out;             // NCHW float or double
  int out_f64;
  const float* oscale;   // mode 1: out = (acc + bias) * oscale + oshift
  const float* oshift;
  const bf16* mask;      // mode 2: NHWC, cout channels
  int* err;
};

__device__ __forceinline__ uint32_t tmem_cols(int N) { return N <= 32 ? 32u : (N <= 64 ? 64u : (N <= 128 ? 128u : 256u)); }

template <bool VEC>
__global__ void __launch_bounds__(128) k_conv(ConvArgs a) {
  extern __shared__ __align__(1024) unsigned char csm[];
  __shared__ __align__(8) uint64_t mbar[2];
  __shared__ uint32_t tslot;
  const int tid = threadIdx.x, warp = tid >> 5;
  const int N = a.N;
  unsigned char* sA0 = csm;
  unsigned char* sB0 = csm + 2 * CHUNK_A;
  const int bbytes = N * KC * 2;
  const uint32_t ncols = tmem_cols(N);
  if (warp == 0) tc::tmem_alloc(&tslot, ncols);
  if (tid == 0) {
    tc::mbar_init(&mbar[0], 1);
    tc::mbar_init(&mbar[1], 1);
    tc::mbar_fence_init();
  }
  tc::fence_before();
  __syncthreads();
  tc::fence_after();
  const uint32_t tmem = tslot;
  const uint32_t idesc = tc::idesc_bf16(TM, N);

  const int p = blockIdx.x * TM + tid;           // this thread's pixel (tile row)
  const int HW = a.H * a.W;
  const int b = p / HW, rem = p - b * HW, y = rem / a.W, x = rem - (rem / a.W) * a.W;
  const bf16* img = a.in + (size_t)b * HW * a.cin;
  bool failed = false;
  for (int c = 0; c < a.nchunk; c++) {
    const int s = c & 1;
    if (c >= 2) {
      const bool to = !tc::mbar_wait(&mbar[s], ((c - 2) >> 1) & 1);
      if (__syncthreads_or(to)) { failed = true; break; }
    }
    unsigned char* sA = sA0 + s * CHUNK_A;
    unsigned char* sB = sB0 + s * bbytes;
    if (VEC) {
#pragma unroll
      for (int g = 0; g < KC / 8; g++) {
        const int k0 = c * KC + g * 8;
        const int tap = k0 / a.cin, ci0 = k0 - tap * a.cin;
        uint4 v = make_uint4(0, 0, 0, 0);
        if (tap < NTAP) {
          const int yy = wrap(y + tap / 5 - 2, a.H), xx = wrap(x + tap % 5 - 2, a.W);
          v = __ldg(reinterpret_cast<const uint4*>(img + ((size_t)yy * a.W + xx) * a.cin + ci0));
        }
        *reinterpret_cast<uint4*>(sA + tc::kmajor_off(tid, g * 8, KC)) = v;
      }
    } else {
#pragma unroll 1
      for (int g = 0; g < KC / 8; g++) {
        unsigned short h[8];
#pragma unroll
        for (int j = 0; j < 8; j++) {
          const int k = c * KC + g * 8 + j;
          const int tap = k / a.cin, ci = k - tap * a.cin;
          unsigned short val = 0;
          if (tap < NTAP) {
            const int yy = wrap(y + tap / 5 - 2, a.H), xx = wrap(x + tap % 5 - 2, a.W);
            val = __ldg(reinterpret_cast<const unsigned short*>(img + ((size_t)yy * a.W + xx) * a.cin + ci));
          }
          h[j] = val;
        }
        uint4 v;
        v.x = h[0] | ((uint32_t)h[1] << 16);
        v.y = h[2] | ((uint32_t)h[3] << 16);
        v.z = h[4] | ((uint32_t)h[5] << 16);
        v.w = h[6] | ((uint32_t)h[7] << 16);
        *reinterpret_cast<uint4*>(sA + tc::kmajor_off(tid, g * 8, KC)) = v;
      }
    }
    const uint4* src = reinterpret_cast<const uint4*>(a.wpk + (size_t)c * N * KC);
    for (int i = tid; i < N * KC / 8; i += TM) reinterpret_cast<uint4*>(sB)[i] = __ldg(src + i);
    tc::fence_proxy_async();
    __syncthreads();
    if (tid == 0) {
      tc::fence_after();
      const uint32_t aa = tc::smem_u32(sA), bb = tc::smem_u32(sB);
#pragma unroll
      for (int ks = 0; ks < KC / 16; ks++)
        tc::mma_bf16(tmem, tc::sdesc(aa + ks * 256, 128, KC * 16), tc::sdesc(bb + ks * 256, 128, KC * 16), idesc,
                     (c | ks) ? 1u : 0u);
      tc::mma_commit(&mbar[s]);
    }
  }
  if (!failed) {
    const int L = a.nchunk - 1;
    const bool to = !tc::mbar_wait(&mbar[L & 1], (L >> 1) & 1);
    failed = __syncthreads_or(to);
  }
  if (failed) {
    if (tid == 0) atomicExch(a.err, 1);
    // give any MMA still in flight a bounded time to finish before freeing TMEM
    tc::mbar_wait(&mbar[0], 0, 10000000ull);
    tc::mbar_wait(&mbar[1], 0, 10000000ull);
  } else {
    tc::fence_after();
    const uint32_t trow = tmem + ((uint32_t)(warp * 32) << 16);
    for (int n0 = 0; n0 < N; n0 += 8) {
      float v[8];
      tc::tmem_ld8(trow + n0, v);
      if (n0 >= a.cout) continue;
      if (a.mode == 0 || a.mode == 2) {
        unsigned short h[8];
        uint4 mk = make_uint4(0, 0, 0, 0);
        if (a.mode == 2) mk = __ldg(reinterpret_cast<const uint4*>(a.mask + (size_t)p * a.cout + n0));
        const unsigned short* mh = reinterpret_cast<const unsigned short*>(&mk);
#pragma unroll
        for (int j = 0; j < 8; j++) {
          float t = v[j];
          if (a.mode == 0) {
            t += a.bias[n0 + j];
            t = t > 0.f ? t : 0.f;
          } else {
            // ReLU derivative of the saved activation (positive BF16: sign bit clear, nonzero)
            const bool pos = (mh[j] & 0x8000u) == 0 && mh[j] != 0;
            t = pos ? t : 0.f;
          }
          h[j] = __bfloat16_as_ushort(__float2bfloat16_rn(t));
        }
        uint4 o;
        o.x = h[0] | ((uint32_t)h[1] << 16);
        o.y = h[2] | ((uint32_t)h[3] << 16);
        o.z = h[4] | ((uint32_t)h[5] << 16);
        o.w = h[6] | ((uint32_t)h[7] << 16);
        *reinterpret_cast<uint4*>(a.out_bf + (size_t)p * a.cout + n0) = o;
      } else {
#pragma unroll
        for (int j = 0; j < 8; j++) {
          const int n = n0 + j;
          if (n < a.cout) {
            const float t = (v[j] + (a.bias ? a.bias[n] : 0.f)) * a.oscale[n] + a.oshift[n];
            const size_t o = (((size_t)b * a.cout + n) * a.H + y) * a.W + x;
            if (a.out_f64) static_cast<double*>(a.out)[o] = (double)t;
            else static_cast<float*>(a.out)[o] = t;
          }
        }
      }
    }
  }
  tc::fence_before();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(tmem, ncols);
}

// ---------------------------------------------------------------------------
// weight gradient: rows m = (tap, ci) (tile of 128), columns n = co, K =
// pixels, one image row (W = 64 pixels) per chunk; each CTA sums a range of
// image rows and adds its partial sums atomically into dw[co][tap][ci].
// ---------------------------------------------------------------------------
struct WgradArgs {
  const bf16* x;   // layer input NHWC (cin)
  int cin;
  const bf16* g;   // gradient of the pre-activation output NHWC (cout)
  int cout, N, M;  // N = pad16(cout), M = 25 cin
  int H, W, nrows, rows_per_cta;
  float* dw;
  int* err;
};

template <bool VECX, bool VECG>
__global__ void __launch_bounds__(128) k_wgrad(WgradArgs a) {
  extern __shared__ __align__(1024) unsigned char csm[];
  __shared__ __align__(8) uint64_t mbar[2];
  __shared__ uint32_t tslot;
  const int tid = threadIdx.x, warp = tid >> 5;
  const int N = a.N;
  unsigned char* sA0 = csm;
  unsigned char* sB0 = csm + 2 * CHUNK_A;
  const int bbytes = N * KC * 2;
  const uint32_t ncols = tmem_cols(N);
  if (warp == 0) tc::tmem_alloc(&tslot, ncols);
  if (tid == 0) {
    tc::mbar_init(&mbar[0], 1);
    tc::mbar_init(&mbar[1], 1);
    tc::mbar_fence_init();
  }
  tc::fence_before();
  __syncthreads();
  tc::fence_after();
  const uint32_t tmem = tslot;
  const uint32_t idesc = tc::idesc_bf16(TM, N);
  const int m0 = blockIdx.x * TM;
  const int r0 = blockIdx.y * a.rows_per_cta;
  const int r1 = min(a.nrows, r0 + a.rows_per_cta);
  const int nchunk = r1 - r0;
  bool failed = false;
  for (int c = 0; c < nchunk; c++) {
    const int s = c & 1;
    if (c >= 2) {
      const bool to = !tc::mbar_wait(&mbar[s], ((c - 2) >> 1) & 1);
      if (__syncthreads_or(to)) { failed = true; break; }
    }
    unsigned char* sA = sA0 + s * CHUNK_A;
    unsigned char* sB = sB0 + s * bbytes;
    const int rr = r0 + c;
    const int b = rr / a.H, y = rr - (rr / a.H) * a.H;
    const bf16* img = a.x + (size_t)b * a.H * a.W * a.cin;
    // A[m][k] = x[b][y + dy][k + dx][ci]
    if (VECX) {
      const int k = tid & 63;
      for (int mg = tid >> 6; mg < TM / 8; mg += 2) {
        const int m = m0 + mg * 8;
        const int tap = m / a.cin, ci0 = m - tap * a.cin;
        uint4 v = make_uint4(0, 0, 0, 0);
        if (tap < NTAP) {
          const int yy = wrap(y + tap / 5 - 2, a.H), xx = wrap(k + tap % 5 - 2, a.W);
          v = __ldg(reinterpret_cast<const uint4*>(img + ((size_t)yy * a.W + xx) * a.cin + ci0));
        }
        const unsigned short* h = reinterpret_cast<const unsigned short*>(&v);
#pragma unroll
        for (int j = 0; j < 8; j++)
          *reinterpret_cast<unsigned short*>(sA + tc::kmajor_off(mg * 8 + j, k, KC)) = h[j];
      }
    } else {
      for (int i = tid; i < TM * KC; i += TM) {
        const int k = i & 63, r = i >> 6;
        const int m = m0 + r;
        const int tap = m / a.cin, ci = m - tap * a.cin;
        unsigned short val = 0;
        if (tap < NTAP) {
          const int yy = wrap(y + tap / 5 - 2, a.H), xx = wrap(k + tap % 5 - 2, a.W);
          val = __ldg(reinterpret_cast<const unsigned short*>(img + ((size_t)yy * a.W + xx) * a.cin + ci));
        }
        *reinterpret_cast<unsigned short*>(sA + tc::kmajor_off(r, k, KC)) = val;
      }
    }
    // B[n][k] = g[b][y][k][n]
    const bf16* grow = a.g + ((size_t)rr * a.W) * a.cout;
    if (VECG) {
      for (int i = tid; i < (N / 8) * KC; i += TM) {
        const int k = i & 63, ng = i >> 6;
        uint4 v = make_uint4(0, 0, 0, 0);
        if (ng * 8 < a.cout) v = __ldg(reinterpret_cast<const uint4*>(grow + (size_t)k * a.cout + ng * 8));
        const unsigned short* h = reinterpret_cast<const unsigned short*>(&v);
#pragma unroll
        for (int j = 0; j < 8; j++)
          *reinterpret_cast<unsigned short*>(sB + tc::kmajor_off(ng * 8 + j, k, KC)) = h[j];
      }
    } else {
      for (int i = tid; i < N * KC; i += TM) {
        const int k = i & 63, n = i >> 6;
        unsigned short val = 0;
        if (n < a.cout) val = __ldg(reinterpret_cast<const unsigned short*>(grow + (size_t)k * a.cout + n));
        *reinterpret_cast<unsigned short*>(sB + tc::kmajor_off(n, k, KC)) = val;
      }
    }
    tc::fence_proxy_async();
    __syncthreads();
    if (tid == 0) {
      tc::fence_after();
      const uint32_t aa = tc::smem_u32(sA), bb = tc::smem_u32(sB);
#pragma unroll
      for (int ks = 0; ks < KC / 16; ks++)
        tc::mma_bf16(tmem, tc::sdesc(aa + ks * 256, 128, KC * 16), tc::sdesc(bb + ks * 256, 128, KC * 16), idesc,
                     (c | ks) ? 1u : 0u);
      tc::mma_commit(&mbar[s]);
    }
  }
  if (!failed && nchunk > 0) {
    const int L = nchunk - 1;
    const bool to = !tc::mbar_wait(&mbar[L & 1], (L >> 1) & 1);
    failed = __syncthreads_or(to);
  }
  if (failed) {
    if (tid == 0) atomicExch(a.err, 1);
    tc::mbar_wait(&mbar[0], 0, 10000000ull);
    tc::mbar_wait(&mbar[1], 0, 10000000ull);
  } else if (nchunk > 0) {
    tc::fence_after();
    const uint32_t trow = tmem + ((uint32_t)(warp * 32) << 16);
    const int m = m0 + tid;
    for (int n0 = 0; n0 < N; n0 += 8) {
      float v[8];
      tc::tmem_ld8(trow + n0, v);
      if (m < a.M) {
#pragma unroll
        for (int j = 0; j < 8; j++)
          if (n0 + j < a.cout) atomicAdd(a.dw + (size_t)(n0 + j) * a.M + m, v[j]);
      }
    }
  }
  tc::fence_before();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(tmem, ncols);
}

// ---------------------------------------------------------------------------
// small kernels: layout conversion, packing, loss, bias gradient, Adam
// ---------------------------------------------------------------------------
// NCHW (float or double) -> NHWC BF16 with (x - mean[c]) * inv_std[c]
template <class T>
__global__ void k_to_nhwc(const T* __restrict__ x, bf16* __restrict__ out, int B, int C, int HW,
                          const float* __restrict__ mean, const float* __restrict__ inv_std) {
  const size_t n = (size_t)B * C * HW;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const int c = (int)(i % C);
    const size_t pix = i / C;
    const size_t b = pix / HW, hw = pix - b * HW;
    const float v = (float)x[(b * C + c) * HW + hw];
    out[i] = __float2bfloat16_rn((v - mean[c]) * inv_std[c]);
  }
}

// packed weights: forward (transpose = 0) or dgrad (transpose = 1)
__global__ void k_pack(const float* __restrict__ w, int cin, int cout, int transpose, bf16* __restrict__ out,
                       int N, int nchunk) {
  const int kin = transpose ? cout : cin;      // channels along K
  const int nreal = transpose ? cin : cout;    // real columns
  const size_t total = (size_t)nchunk * N * KC;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
    const int c = (int)(i / ((size_t)N * KC));
    const int rem = (int)(i - (size_t)c * N * KC);
    const int n = rem / KC, kk = rem - n * KC;
    const int k = c * KC + kk;
    const int tap = k / kin, ch = k - tap * kin;
    float v = 0.f;
    if (n < nreal && tap < NTAP) {
      if (!transpose) v = w[((size_t)n * NTAP + tap) * cin + ch];
      else v = w[((size_t)ch * NTAP + (NTAP - 1 - tap)) * cin + n];
    }
    const size_t o = (size_t)c * N * KC + tc::kmajor_off(n, kk, KC) / 2;
    out[o] = __float2bfloat16_rn(v);
  }
}

// MSE loss of y (NCHW FP32) against t; gradient 2 (y - t) / count as NHWC BF16
__global__ void k_mse(const float* __restrict__ y, const float* __restrict__ t, bf16* __restrict__ g, int B, int C,
                      int HW, float* __restrict__ loss_sum) {
  const size_t n = (size_t)B * C * HW;
  const float sc = 2.f / (float)n;
  float acc = 0.f;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const size_t b = i / ((size_t)C * HW);
    const size_t r = i - b * C * HW;
    const int c = (int)(r / HW);
    const size_t hw = r - (size_t)c * HW;
    const float d = y[i] - t[i];
    acc += d * d;
    g[(b * HW + hw) * C + c] = __float2bfloat16_rn(sc * d);
  }
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) atomicAdd(loss_sum, acc / (float)n);
}

// db[c] += sum over pixels of g[p][c]
__global__ void k_bias_grad(const bf16* __restrict__ g, int npix, int C, float* __restrict__ db) {
  __shared__ float acc[128];
  for (int i = threadIdx.x; i < C; i += blockDim.x) acc[i] = 0.f;
  __syncthreads();
  const size_t n = (size_t)npix * C;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    atomicAdd(&acc[i % C], __bfloat162float(g[i]));
  __syncthreads();
  for (int i = threadIdx.x; i < C; i += blockDim.x) atomicAdd(&db[i], acc[i]);
}

__global__ void k_adam(float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m,
                       float* __restrict__ v, size_t n, float lr, float b1, float b2, float eps, float c1, float c2) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
  }
}

struct CnnLayer {
  int cin, cout;
  int Nf, nchf;      // forward packing
  int Nd, nchd;      // dgrad packing
  size_t woff, boff; // offsets into the parameter vector
  bf16* wf;
  bf16* wd;
};

}  // namespace

struct pqg_cnn {
  int nl = 0, H = 0, W = 0, maxB = 0;
  std::vector<CnnLayer> L;
  size_t nparams = 0;
  float* params = nullptr;
  float* grads = nullptr;
  float* m = nullptr;
  float* v = nullptr;
  std::vector<bf16*> act;     // act[0] input, act[l] output of layer l-1 (post-ReLU)
  float* out = nullptr;       // last layer, NCHW FP32 (training)
  bf16* ga = nullptr;
  bf16* gb = nullptr;
  float* norm = nullptr;      // in_mean, in_inv_std, out_scale, out_shift, id_scale(1), id_shift(0)
  int cmax = 0;
  float* loss = nullptr;
  int* err = nullptr;
  long long adam_t = 0;
};

namespace {

size_t conv_smem(int N) { return 2 * (size_t)CHUNK_A + 2 * (size_t)N * KC * 2; }

int launch_conv(pqg_cnn* net, const CnnLayer& l, bool dgrad, const bf16* in, int batch, int mode, bf16* out_bf,
                void* out, int out_f64, const float* oscale, const float* oshift, const bf16* mask,
                cudaStream_t st) {
  ConvArgs a;
  a.in = in;
  a.cin = dgrad ? l.cout : l.cin;
  a.wpk = dgrad ? l.wd : l.wf;
  a.N = dgrad ? l.Nd : l.Nf;
  a.nchunk = dgrad ? l.nchd : l.nchf;
  a.cout = dgrad ? l.cin : l.cout;
  a.bias = dgrad ? nullptr : net->params + l.boff;
  a.H = net->H;
  a.W = net->W;
  a.npix = batch * net->H * net->W;
  a.mode = mode;
  a.out_bf = out_bf;
  a.out = out;
  a.out_f64 = out_f64;
  a.oscale = oscale;
  a.oshift = oshift;
  a.mask = mask;
  a.err = net->err;
  const size_t smem = conv_smem(a.N);
  const dim3 grid(a.npix / TM);
  if (a.cin % 8 == 0) k_conv<true><<<grid, TM, smem, st>>>(a);
  else k_conv<false><<<grid, TM, smem, st>>>(a);
  CCUDA(cudaGetLastError());
  return PQG_OK;
}

int launch_wgrad(pqg_cnn* net, const CnnLayer& l, const bf16* x, const bf16* g, int batch, cudaStream_t st) {
  WgradArgs a;
  a.x = x;
  a.cin = l.cin;
  a.g = g;
  a.cout = l.cout;
  a.N = l.Nf;
  a.M = NTAP * l.cin;
  a.H = net->H;
  a.W = net->W;
  a.nrows = batch * net->H;
  const int mt = (a.M + TM - 1) / TM;
  const int target = 4 * 152;
  int ks = std::max(1, std::min(a.nrows, (target + mt - 1) / mt));
  a.rows_per_cta = (a.nrows + ks - 1) / ks;
  ks = (a.nrows + a.rows_per_cta - 1) / a.rows_per_cta;
  a.dw = net->grads + l.woff;
  a.err = net->err;
  const size_t smem = conv_smem(a.N);
  const dim3 grid(mt, ks);
  const bool vx = l.cin % 8 == 0, vg = l.cout % 8 == 0;
#define WG(X, G) k_wgrad<X, G><<<grid, TM, smem, st>>>(a)
  if (vx && vg) WG(true, true);
  else if (vx) WG(true, false);
  else if (vg) WG(false, true);
  else WG(false, false);
#undef WG
  CCUDA(cudaGetLastError());
  return PQG_OK;
}

// the largest tile (N = 128) needs 64 KiB of dynamic shared memory
int set_attrs() {
  const int big = (int)conv_smem(128);
  CCUDA(cudaFuncSetAttribute(k_conv<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, big));
  CCUDA(cudaFuncSetAttribute(k_conv<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, big));
  CCUDA(cudaFuncSetAttribute(k_wgrad<true, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, big));
  CCUDA(cudaFuncSetAttribute(k_wgrad<true, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, big));
  CCUDA(cudaFuncSetAttribute(k_wgrad<false, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, big));
  CCUDA(cudaFuncSetAttribute(k_wgrad<false, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, big));
  return PQG_OK;
}

int grid_for(size_t n) { return (int)std::min<size_t>((n + 255) / 256, 152 * 16); }

int repack(pqg_cnn* net, cudaStream_t st) {
  for (auto& l : net->L) {
    k_pack<<<grid_for((size_t)l.nchf * l.Nf * KC), 256, 0, st>>>(net->params + l.woff, l.cin, l.cout, 0, l.wf, l.Nf,
                                                               l.nchf);
    k_pack<<<grid_for((size_t)l.nchd * l.Nd * KC), 256, 0, st>>>(net->params + l.woff, l.cin, l.cout, 1, l.wd, l.Nd,
                                                               l.nchd);
  }
  CCUDA(cudaGetLastError());
  return PQG_OK;
}

int check_err(pqg_cnn* net, cudaStream_t st) {
  int h = 0;
  CCUDA(cudaMemcpyAsync(&h, net->err, sizeof(int), cudaMemcpyDeviceToHost, st));
  CCUDA(cudaStreamSynchronize(st));
  if (h) {
    cudaMemsetAsync(net->err, 0, sizeof(int), st);
    return cfail(PQG_ERR_TIMEOUT, "tensor-core pipeline wait timed out");
  }
  return PQG_OK;
}

// forward through all layers; input already in act[0]
int forward_layers(pqg_cnn* net, int batch, void* out, int out_f64, const float* oscale, const float* oshift,
                   cudaStream_t st) {
  for (int i = 0; i < net->nl; i++) {
    const CnnLayer& l = net->L[i];
    const bool last = i == net->nl - 1;
    int rc = launch_conv(net, l, false, net->act[i], batch, last ? 1 : 0, last ? nullptr : net->act[i + 1],
                         last ? out : nullptr, out_f64, oscale, oshift, nullptr, st);
    if (rc) return rc;
  }
  return PQG_OK;
}

}  // namespace

extern "C" {

PQG_API const char* pqg_cnn_last_error(void) { return c_last_error.c_str(); }

PQG_API int pqg_cnn_create(pqg_cnn** out, int nlayers, const int* channels, int height, int width, int max_batch) {
  if (!out || !channels || nlayers < 1 || nlayers > 16) return cfail(PQG_ERR_INVALID, "bad layer count");
  if (width != KC) return cfail(PQG_ERR_UNSUPPORTED, "image width must be 64");
  if (height < 5 || max_batch < 1 || ((size_t)height * width * max_batch) % TM)
    return cfail(PQG_ERR_INVALID, "batch * height * width must be a multiple of 128");
  for (int i = 0; i <= nlayers; i++)
    if (channels[i] < 1 || channels[i] > 128) return cfail(PQG_ERR_UNSUPPORTED, "channels must be in 1..128");
  for (int i = 1; i < nlayers; i++)
    if (channels[i] % 8) return cfail(PQG_ERR_UNSUPPORTED, "hidden channel counts must be multiples of 8");
  pqg_cnn* net = new pqg_cnn();
  net->nl = nlayers;
  net->H = height;
  net->W = width;
  net->maxB = max_batch;
  size_t off = 0;
  for (int i = 0; i < nlayers; i++) {
    CnnLayer l{};
    l.cin = channels[i];
    l.cout = channels[i + 1];
    l.Nf = pad16(l.cout);
    l.nchf = (NTAP * l.cin + KC - 1) / KC;
    l.Nd = pad16(l.cin);
    l.nchd = (NTAP * l.cout + KC - 1) / KC;
    l.woff = off;
    off += (size_t)l.cout * NTAP * l.cin;
    l.boff = off;
    off += l.cout;
    net->L.push_back(l);
    net->cmax = std::max(net->cmax, std::max(l.cin, l.cout));
  }
  net->nparams = off;
  const size_t npix = (size_t)max_batch * height * width;
  auto fail = [&](const char* what) {
    pqg_cnn_destroy(net);
    return cfail(PQG_ERR_CUDA, std::string("allocation failed: ") + what);
  };
  if (cudaMalloc(&net->params, 4 * off) || cudaMalloc(&net->grads, 4 * off) || cudaMalloc(&net->m, 4 * off) ||
      cudaMalloc(&net->v, 4 * off))
    return fail("parameters");
  cudaMemset(net->params, 0, 4 * off);
  cudaMemset(net->m, 0, 4 * off);
  cudaMemset(net->v, 0, 4 * off);
  for (auto& l : net->L) {
    if (cudaMalloc(&l.wf, (size_t)l.nchf * l.Nf * KC * 2) || cudaMalloc(&l.wd, (size_t)l.nchd * l.Nd * KC * 2))
      return fail("packed weights");
  }
  net->act.assign(nlayers, nullptr);
  for (int i = 0; i < nlayers; i++)
    if (cudaMalloc(&net->act[i], npix * net->L[i].cin * 2)) return fail("activations");
  if (cudaMalloc(&net->out, npix * net->L.back().cout * 4) || cudaMalloc(&net->ga, npix * net->cmax * 2) ||
      cudaMalloc(&net->gb, npix * net->cmax * 2) || cudaMalloc(&net->norm, 4 * 6 * 128) ||
      cudaMalloc(&net->loss, 4) || cudaMalloc(&net->err, 4))
    return fail("buffers");
  std::vector<float> nm(6 * 128, 0.f);
  for (int c = 0; c < 128; c++) {
    nm[128 + c] = 1.f;
    nm[256 + c] = 1.f;
    nm[512 + c] = 1.f;
  }
  cudaMemcpy(net->norm, nm.data(), 4 * nm.size(), cudaMemcpyHostToDevice);
  cudaMemset(net->err, 0, 4);
  if (set_attrs() != PQG_OK || cudaDeviceSynchronize() != cudaSuccess) return fail("initialisation");
  *out = net;
  return PQG_OK;
}

PQG_API int pqg_cnn_destroy(pqg_cnn* net) {
  if (!net) return PQG_OK;
  cudaFree(net->params);
  cudaFree(net->grads);
  cudaFree(net->m);
  cudaFree(net->v);
  for (auto& l : net->L) {
    cudaFree(l.wf);
    cudaFree(l.wd);
  }
  for (auto p : net->act) cudaFree(p);
  cudaFree(net->out);
  cudaFree(net->ga);
  cudaFree(net->gb);
  cudaFree(net->norm);
  cudaFree(net->loss);
  cudaFree(net->err);
  delete net;
  return PQG_OK;
}

PQG_API int pqg_cnn_shape(pqg_cnn* net, int* cin, int* cout, int* ny, int* nx, int* max_batch) {
  if (!net) return cfail(PQG_ERR_INVALID, "NULL argument");
  if (cin) *cin = net->L.front().cin;
  if (cout) *cout = net->L.back().cout;
  if (ny) *ny = net->H;
  if (nx) *nx = net->W;
  if (max_batch) *max_batch = net->maxB;
  return PQG_OK;
}

PQG_API int pqg_cnn_nparams(pqg_cnn* net, long long* n) {
  if (!net || !n) return cfail(PQG_ERR_INVALID, "NULL argument");
  *n = (long long)net->nparams;
  return PQG_OK;
}

PQG_API int pqg_cnn_set_params(pqg_cnn* net, const float* host, void* stream) {
  if (!net || !host) return cfail(PQG_ERR_INVALID, "NULL argument");
  cudaStream_t st = (cudaStream_t)stream;
  CCUDA(cudaMemcpyAsync(net->params, host, 4 * net->nparams, cudaMemcpyHostToDevice, st));
  CCUDA(cudaMemsetAsync(net->m, 0, 4 * net->nparams, st));
  CCUDA(cudaMemsetAsync(net->v, 0, 4 * net->nparams, st));
  net->adam_t = 0;
  int rc = repack(net, st);
  if (rc) return rc;
  CCUDA(cudaStreamSynchronize(st));
  return PQG_OK;
}

PQG_API int pqg_cnn_get_params(pqg_cnn* net, float* host, void* stream) {
  if (!net || !host) return cfail(PQG_ERR_INVALID, "NULL argument");
  cudaStream_t st = (cudaStream_t)stream;
  CCUDA(cudaMemcpyAsync(host, net->params, 4 * net->nparams, cudaMemcpyDeviceToHost, st));
  CCUDA(cudaStreamSynchronize(st));
  return PQG_OK;
}

PQG_API int pqg_cnn_get_grads(pqg_cnn* net, float* host, void* stream) {
  if (!net || !host) return cfail(PQG_ERR_INVALID, "NULL argument");
  cudaStream_t st = (cudaStream_t)stream;
  CCUDA(cudaMemcpyAsync(host, net->grads, 4 * net->nparams, cudaMemcpyDeviceToHost, st));
  CCUDA(cudaStreamSynchronize(st));
  return PQG_OK;
}

PQG_API int pqg_cnn_set_norm(pqg_cnn* net, const float* in_mean, const float* in_std, const float* out_mean,
                             const float* out_std) {
  if (!net || !in_mean || !in_std || !out_mean || !out_std) return cfail(PQG_ERR_INVALID, "NULL argument");
  std::vector<float> nm(4 * 128, 0.f);
  const int ci = net->L[0].cin, co = net->L.back().cout;
  for (int c = 0; c < 128; c++) {
    nm[128 + c] = 1.f;
    nm[256 + c] = 1.f;
  }
  for (int c = 0; c < ci; c++) {
    if (!(in_std[c] > 0.f)) return cfail(PQG_ERR_INVALID, "input std must be positive");
    nm[c] = in_mean[c];
    nm[128 + c] = 1.f / in_std[c];
  }
  for (int c = 0; c < co; c++) {
    nm[256 + c] = out_std[c];
    nm[384 + c] = out_mean[c];
  }
  CCUDA(cudaMemcpy(net->norm, nm.data(), 4 * nm.size(), cudaMemcpyHostToDevice));
  return PQG_OK;
}

// y = net((x - in_mean) / in_std) * out_std + out_mean; x (batch, cin, H, W)
// and y (batch, cout, H, W) are device arrays, FP32 or FP64.
PQG_API int pqg_cnn_forward(pqg_cnn* net, const void* x, int x_f64, void* y, int y_f64, int batch, void* stream) {
  if (!net || !x || !y) return cfail(PQG_ERR_INVALID, "NULL argument");
  if (batch < 1 || batch > net->maxB || ((size_t)batch * net->H * net->W) % TM)
    return cfail(PQG_ERR_INVALID, "bad batch size");
  cudaStream_t st = (cudaStream_t)stream;
  const size_t n = (size_t)batch * net->L[0].cin * net->H * net->W;
  if (x_f64)
    k_to_nhwc<double><<<grid_for(n), 256, 0, st>>>((const double*)x, net->act[0], batch, net->L[0].cin,
                                                   net->H * net->W, net->norm, net->norm + 128);
  else
    k_to_nhwc<float><<<grid_for(n), 256, 0, st>>>((const float*)x, net->act[0], batch, net->L[0].cin,
                                                  net->H * net->W, net->norm, net->norm + 128);
  CCUDA(cudaGetLastError());
  int rc = forward_layers(net, batch, y, y_f64, net->norm + 256, net->norm + 384, st);
  if (rc) return rc;
  return PQG_OK;
}

// gradients of the MSE loss of net(x) against t (both standardised, FP32
// NCHW device arrays) into the gradient vector; loss (host) if not NULL
PQG_API int pqg_cnn_backward(pqg_cnn* net, const float* x, const float* t, int batch, float* loss, void* stream) {
  if (!net || !x || !t) return cfail(PQG_ERR_INVALID, "NULL argument");
  if (batch < 1 || batch > net->maxB || ((size_t)batch * net->H * net->W) % TM)
    return cfail(PQG_ERR_INVALID, "bad batch size");
  cudaStream_t st = (cudaStream_t)stream;
  const int HW = net->H * net->W;
  const size_t npix = (size_t)batch * HW;
  const float* ident = net->norm + 512;   // 1 then 0 (norm + 640 holds zeros)
  k_to_nhwc<float><<<grid_for(npix * net->L[0].cin), 256, 0, st>>>(x, net->act[0], batch, net->L[0].cin, HW,
                                                                   net->norm + 640, ident);
  CCUDA(cudaGetLastError());
  int rc = forward_layers(net, batch, net->out, 0, ident, net->norm + 640, st);
  if (rc) return rc;
  CCUDA(cudaMemsetAsync(net->grads, 0, 4 * net->nparams, st));
  CCUDA(cudaMemsetAsync(net->loss, 0, 4, st));
  const int nl = net->nl;
  const int cl = net->L[nl - 1].cout;
  k_mse<<<grid_for(npix * cl), 256, 0, st>>>(net->out, t, net->ga, batch, cl, HW, net->loss);
  CCUDA(cudaGetLastError());
  bf16* g = net->ga;     // gradient of the current layer's pre-activation output
  bf16* gn = net->gb;
  for (int i = nl - 1; i >= 0; i--) {
    const CnnLayer& l = net->L[i];
    k_bias_grad<<<std::min<size_t>(1024, (npix * l.cout + 255) / 256), 256, 0, st>>>(g, (int)npix, l.cout,
                                                                                  net->grads + l.boff);
    CCUDA(cudaGetLastError());
    rc = launch_wgrad(net, l, net->act[i], g, batch, st);
    if (rc) return rc;
    if (i > 0) {
      // gradient of layer i's input, masked by the ReLU of layer i-1's output
      rc = launch_conv(net, l, true, g, batch, 2, gn, nullptr, 0, nullptr, nullptr, net->act[i], st);
      if (rc) return rc;
      std::swap(g, gn);
    }
  }
  rc = check_err(net, st);
  if (rc) return rc;
  if (loss) {
    CCUDA(cudaMemcpyAsync(loss, net->loss, 4, cudaMemcpyDeviceToHost, st));
    CCUDA(cudaStreamSynchronize(st));
  }
  return PQG_OK;
}

// one Adam update of the parameters from the gradient vector
PQG_API int pqg_cnn_adam(pqg_cnn* net, float lr, float beta1, float beta2, float eps, void* stream) {
  if (!net) return cfail(PQG_ERR_INVALID, "NULL argument");
  cudaStream_t st = (cudaStream_t)stream;
  net->adam_t++;
  const float c1 = 1.f - (float)std::pow((double)beta1, (double)net->adam_t);
  const float c2 = 1.f - (float)std::pow((double)beta2, (double)net->adam_t);
  k_adam<<<grid_for(net->nparams), 256, 0, st>>>(net->params, net->grads, net->m, net->v, net->nparams, lr, beta1,
                                                 beta2, eps, c1, c2);
  CCUDA(cudaGetLastError());
  return repack(net, st);
}

PQG_API int pqg_cnn_train_step(pqg_cnn* net, const float* x, const float* t, int batch, float lr, float* loss,
                               void* stream) {
  int rc = pqg_cnn_backward(net, x, t, batch, loss, stream);
  if (rc) return rc;
  return pqg_cnn_adam(net, lr, 0.9f, 0.999f, 1e-8f, stream);
}

}  // extern "C"
