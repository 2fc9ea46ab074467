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
//            (a forward convolution with flipped, channel-transposed weights)
//   wgrad    dw[co][tap][ci] = sum_p x[p + off(tap)][ci] g[p][co]
// with off(tap) = (tap / 5 - 2, tap % 5 - 2) taken periodically.
//
// Activations and gradients are BF16 NHWC images stored with a periodic
// halo of 2 pixels on each side ((ny + 4) x (nx + 4) pixels per image, the
// halo a copy of the opposite edge), written by every producer, so that no
// consumer wraps indices.  Master weights are FP32 w[co][tap][ci].
//
// Three convolution kernels:
//  * k_conv_halo (16, 32, 64 or 128 channels along K): every forward layer
//    (the network input is stored zero-padded to 16 channels) and the data
//    gradients with at least 16 channels.  A CTA computes a tile of 16 rows
//    x 8 SX columns.  TMA loads the input tile with its halo once into
//    shared memory as one slab per 8 channels (pixel-major, 16 bytes per
//    pixel); the A operand of tap (dy, dx) is then a shifted descriptor over
//    the same slabs (core matrix = 8 consecutive pixels of a row, next
//    8-pixel group = next image row).  The per-tap weight blocks stream
//    through a bulk-copy ring of `nst` stages (all 25 taps resident when
//    they fit); one thread per 8-column subtile issues its MMAs.
//  * k_conv_gather (few channels along K: the data gradient through the
//    2-channel output layer): threads gather a K-chunk of 64 (tap, channel)
//    pairs per pixel.
//  * k_conv_rows (opt-in, PQG_CNN_ROWS; measured slower than the halo
//    kernel on these layers): a tile is two full image rows, so every A
//    operand window is aligned, and the five horizontal taps are folded into
//    the MMA's N dimension (N = 5 x 32 for 32 output channels); the epilogue
//    sums the horizontally shifted columns.
// The weight gradient gathers (tap, channel) x pixel tiles (k_wgrad) and
// adds its partial sums atomically.
#include <cuda_runtime.h>
#include <cuda_bf16.h>
#include <cuda.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "pyqg_gb300.h"
#include "pqg_tc.cuh"

#define PQG_API __attribute__((visibility("default")))

typedef __nv_bfloat16 bf16;
namespace tc = pqg::tc;

namespace {

constexpr int KC = 64;     // K elements per chunk (gather kernels)
constexpr int TM = 128;    // tile rows
constexpr int NTAP = 25;   // 5 x 5 taps
constexpr int PAD = 2;     // halo width
constexpr int CHUNK_A = TM * KC * 2;   // bytes of one A stage (gather kernels)
constexpr int TY = 16;     // output rows of a halo-kernel tile
constexpr int TYH = TY + 2 * PAD;
constexpr int MAXST = 2 * NTAP;   // weight stages of the halo kernel (at most one per tap and unit)
constexpr int NEPI = 8;           // epilogue warps of the halo kernel (two per TMEM lane quarter)
constexpr int MAXH = 4;           // halo buffers of the halo kernel at most

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

struct Img {            // padded NHWC image geometry
  int H, W, Hp, Wp;
  __device__ __forceinline__ size_t pix(int b, int yp, int xp) const {
    return ((size_t)b * Hp + yp) * Wp + xp;
  }
};

// periodic images of interior coordinate y in padded coordinates
__device__ __forceinline__ int images(int y, int n, int* out) {
  int k = 0;
  out[k++] = y + PAD;
  if (y < PAD) out[k++] = y + PAD + n;
  else if (y >= n - PAD) out[k++] = y + PAD - n;
  return k;
}

// store 8 channels (16 bytes) of pixel (b, y, x) and its halo copies
__device__ __forceinline__ void store_px16(bf16* buf, int C, const Img& g, int b, int y, int x, int c0, uint4 v) {
  int ys[2], xs[2];
  const int ny = images(y, g.H, ys), nx = images(x, g.W, xs);
  for (int i = 0; i < ny; i++)
    for (int j = 0; j < nx; j++) *reinterpret_cast<uint4*>(buf + g.pix(b, ys[i], xs[j]) * C + c0) = v;
}
__device__ __forceinline__ void store_px1(bf16* buf, int C, const Img& g, int b, int y, int x, int c, bf16 v) {
  int ys[2], xs[2];
  const int ny = images(y, g.H, ys), nx = images(x, g.W, xs);
  for (int i = 0; i < ny; i++)
    for (int j = 0; j < nx; j++) buf[g.pix(b, ys[i], xs[j]) * C + c] = v;
}

// TMEM allocation: a power of two of at least 32 columns (n <= 512)
__device__ __forceinline__ uint32_t tmem_cols(int n) {
  return n <= 32 ? 32u : (n <= 64 ? 64u : (n <= 128 ? 128u : (n <= 256 ? 256u : 512u)));
}

__device__ __forceinline__ uint32_t bf2(float a, float b) {
  return (uint32_t)__bfloat16_as_ushort(__float2bfloat16_rn(a)) |
         ((uint32_t)__bfloat16_as_ushort(__float2bfloat16_rn(b)) << 16);
}

// epilogue shared by the convolution kernels: 8 accumulator columns n0.. of
// output pixel (b, y, x)
struct Epi {
  int mode;              // 0: bias+ReLU -> out_bf; 1: affine -> out (NCHW); 2: ReLU mask -> out_bf
  int cout;              // real output channels (multiple of 8 in modes 0 and 2)
  const float* bias;     // (cout) or null
  bf16* out_bf;          // padded NHWC, cout channels
  void* out;             // NCHW float or double, unpadded
  int out_f64;
  const float* oscale;   // mode 1: out = (acc + bias) * oscale + oshift
  const float* oshift;
  const bf16* mask;      // mode 2: padded NHWC, cout channels
};

// `bias` is the bias vector (global or shared memory) or null
__device__ __forceinline__ void epilogue8(const Epi& e, const float* bias, const Img& g, int b, int y, int x, int n0,
                                          const float* v) {
  if (n0 >= e.cout) return;
  if (e.mode == 0 || e.mode == 2) {
    float t[8];
    uint4 mk = make_uint4(0, 0, 0, 0);
    if (e.mode == 2) mk = __ldg(reinterpret_cast<const uint4*>(e.mask + g.pix(b, y + PAD, x + PAD) * e.cout + n0));
    const unsigned short* mh = reinterpret_cast<const unsigned short*>(&mk);
#pragma unroll
    for (int j = 0; j < 8; j++) {
      if (e.mode == 0) {
        const float s = v[j] + bias[n0 + j];
        t[j] = s > 0.f ? s : 0.f;
      } else {
        // ReLU derivative from the saved (post-ReLU) activation: positive BF16
        const bool pos = (mh[j] & 0x8000u) == 0 && mh[j] != 0;
        t[j] = pos ? v[j] : 0.f;
      }
    }
    store_px16(e.out_bf, e.cout, g, b, y, x, n0, make_uint4(bf2(t[0], t[1]), bf2(t[2], t[3]), bf2(t[4], t[5]),
                                                            bf2(t[6], t[7])));
  } else {
#pragma unroll
    for (int j = 0; j < 8; j++) {
      const int n = n0 + j;
      if (n < e.cout) {
        const float t = (v[j] + (bias ? bias[n] : 0.f)) * e.oscale[n] + e.oshift[n];
        const size_t o = (((size_t)b * e.cout + n) * g.H + y) * g.W + x;
        if (e.out_f64) static_cast<double*>(e.out)[o] = (double)t;
        else static_cast<float*>(e.out)[o] = t;
      }
    }
  }
}

// mode 0 (bias + ReLU -> padded NHWC BF16) without per-call address work:
// the store addresses of an output pixel and of its periodic halo copies,
// computed once per pixel
struct PixOut {
  bf16* p0;              // the pixel
  bf16* p1;              // x halo copy (h1)
  bf16* p2;              // y halo copy (h2)
  bf16* p3;              // corner copy (h1 && h2)
  bool h1, h2;
};

__device__ __forceinline__ PixOut pix_out(bf16* buf, int C, const Img& g, int b, int y, int x) {
  // padded coordinates of the pixel and of its periodic image (the same
  // when it has none)
  const int y0 = y + PAD, x0 = x + PAD;
  const int y1 = y < PAD ? y0 + g.H : (y >= g.H - PAD ? y0 - g.H : y0);
  const int x1 = x < PAD ? x0 + g.W : (x >= g.W - PAD ? x0 - g.W : x0);
  PixOut o;
  o.h1 = x1 != x0;
  o.h2 = y1 != y0;
  o.p0 = buf + g.pix(b, y0, x0) * C;
  o.p1 = buf + g.pix(b, y0, x1) * C;
  o.p2 = buf + g.pix(b, y1, x0) * C;
  o.p3 = buf + g.pix(b, y1, x1) * C;
  return o;
}

// K (multiple of 8) accumulator columns n0.. of one pixel: + bias, ReLU,
// BF16 (round to nearest even, as epilogue8), 16-byte stores; `bias` is a
// 16-byte aligned shared-memory vector
template <int K>
__device__ __forceinline__ void relu_store(const PixOut& o, const float* bias, int n0, const float* v) {
  uint32_t w[K / 2];
#pragma unroll
  for (int i = 0; i < K / 4; i++) {
    const float4 bb = *reinterpret_cast<const float4*>(bias + n0 + 4 * i);
    float t0 = v[4 * i] + bb.x, t1 = v[4 * i + 1] + bb.y, t2 = v[4 * i + 2] + bb.z, t3 = v[4 * i + 3] + bb.w;
    t0 = t0 > 0.f ? t0 : 0.f;
    t1 = t1 > 0.f ? t1 : 0.f;
    t2 = t2 > 0.f ? t2 : 0.f;
    t3 = t3 > 0.f ? t3 : 0.f;
    const __nv_bfloat162 h01 = __floats2bfloat162_rn(t0, t1), h23 = __floats2bfloat162_rn(t2, t3);
    w[2 * i] = *reinterpret_cast<const uint32_t*>(&h01);
    w[2 * i + 1] = *reinterpret_cast<const uint32_t*>(&h23);
  }
#pragma unroll
  for (int q = 0; q < K / 8; q++) {
    const uint4 u = make_uint4(w[4 * q], w[4 * q + 1], w[4 * q + 2], w[4 * q + 3]);
    *reinterpret_cast<uint4*>(o.p0 + n0 + 8 * q) = u;
    if (o.h1) *reinterpret_cast<uint4*>(o.p1 + n0 + 8 * q) = u;
    if (o.h2) *reinterpret_cast<uint4*>(o.p2 + n0 + 8 * q) = u;
    if (o.h1 && o.h2) *reinterpret_cast<uint4*>(o.p3 + n0 + 8 * q) = u;
  }
}

// ---------------------------------------------------------------------------
// halo-tile convolution (input channels 16, 32, 64 or 128), persistent and
// warp-specialised, one CTA per SM, 9 + SX warps:
//   warps 0-7     epilogue: TMEM -> registers -> global (warp w reads TMEM
//                 lanes 32 (w % 4) ..; the two warps of a lane quarter split
//                 the subtiles, or the columns of a single subtile)
//   warp 8        producer (one lane): TMA halo tiles into `nh` buffers,
//                 per-tap weight blocks into a ring of `nst` stages (loaded
//                 once when all 25 taps are resident)
//   warps 9..     one MMA issuer (one lane) per 8-column subtile: 25 taps x
//                 cin/16 MMAs per tile into the subtile's columns of one of
//                 two TMEM accumulators.
// Inputs of more than 64 channels are pipelined in units of 64 channels (a
// halo buffer and a weight block per unit), so that two half-size halo
// buffers overlap loads with MMAs.  Independent issuers keep several
//                 MMA streams in flight, which the shifted (not atom-aligned)
//                 operand windows need to reach the tensor pipe's rate.
// Barriers (parity = use count & 1): hfull / hempty per halo buffer, afull /
// aempty per accumulator, wfull / wempty per weight stage; hempty, wempty and
// afull count one arrival per issuer, aempty one per epilogue warp (lane 0,
// after the warp's TMEM loads and a __syncwarp).
// ---------------------------------------------------------------------------
struct HaloArgs {
  int cin;               // input channels
  const bf16* wpk;       // 25 per-tap blocks of N x cin (K-major core matrices)
  int N;                 // pad16(cout); 2 SX N <= 512
  int nst;               // weight stages (NTAP: resident)
  int nh;                // halo buffers (1 .. MAXH)
  int tiles_x;           // W / (8 SX)
  int ntiles;            // batch * (H / 16) * tiles_x
  Img g;
  Epi e;
  int* err;
  int stop_unit;         // >= 0: the producer issues no copy from this pipeline unit on (failure tests)
  unsigned long long wait_ns;   // bound of every pipeline wait
};

template <int SX, int KS, int KUM>
__global__ void __launch_bounds__(32 * (NEPI + 1 + SX)) k_conv_halo(const __grid_constant__ CUtensorMap tmap, HaloArgs a) {
  constexpr int TXH = 8 * SX + 2 * PAD;
  constexpr int SLAB = TXH * TYH * 16;     // bytes per 8 channels
  constexpr int CH = KS > KUM ? KS / KUM : 1;  // channel units per tile (at most 16 KUM channels each)
  constexpr int KU = KS / CH;              // K steps of 16 per unit
  constexpr int cu = 16 * KU, groups = 2 * KU;   // channels and 8-channel slabs per unit
  extern __shared__ __align__(1024) unsigned char csm[];
  __shared__ __align__(8) uint64_t hfull[MAXH], hempty[MAXH], afull[2], aempty[2], wfull[MAXST], wempty[MAXST];
  __shared__ __align__(8) uint64_t drain[SX];   // failure path: the MMAs of each issuer
  __shared__ uint32_t tslot;
  __shared__ int s_fail;
  __shared__ long long s_issued[2];   // copies the producer issued: halo units, weight blocks
  __shared__ __align__(16) float s_bias[256];
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int N = a.N, NST = a.nst, NH = a.nh;
  const bool resident = NST >= NTAP * CH;
  const uint32_t hbytes = (uint32_t)groups * SLAB;
  unsigned char* halo = csm;                        // NH buffers
  unsigned char* wst = csm + (size_t)NH * hbytes;   // NST stages
  const uint32_t wbytes = (uint32_t)N * cu * 2;
  const int per_img = (a.g.H / TY) * a.tiles_x;
  const uint32_t acc_cols = SX * N;
  const uint32_t ncols = tmem_cols(2 * acc_cols);
  if (warp == 0) tc::tmem_alloc(&tslot, ncols);
  if (tid == 0) {
    for (int i = 0; i < NH; i++) {
      tc::mbar_init(&hfull[i], 1);
      tc::mbar_init(&hempty[i], SX);
    }
    for (int i = 0; i < 2; i++) {
      tc::mbar_init(&afull[i], SX);
      tc::mbar_init(&aempty[i], NEPI);   // one arrival per epilogue warp
    }
    for (int s = 0; s < NST; s++) {
      tc::mbar_init(&wfull[s], 1);
      tc::mbar_init(&wempty[s], SX);
    }
    for (int i = 0; i < SX; i++) tc::mbar_init(&drain[i], 1);
    tc::mbar_fence_init();
    s_fail = 0;
    s_issued[0] = s_issued[1] = 0;
  }
  for (int i = tid; i < N; i += blockDim.x) s_bias[i] = (a.e.bias && i < a.e.cout) ? a.e.bias[i] : 0.f;
  tc::fence_before();
  __syncthreads();
  tc::fence_after();
  const uint32_t tmem = tslot;
  bool ok = true;
  if (warp == NEPI) {
    if (lane == 0) {
      // producer.  Ring positions are kept as (slot, round) counters: the
      // loop runs on one lane, where a division per tap would dominate.
      int wq = 0, ws = 0, wr = 0;   // weight blocks issued; ring slot and round
      int u = 0, hs = 0, hr = 0;    // pipeline unit (tile, channel unit); halo buffer and round
      bool stopped = false;
      for (int tile = blockIdx.x; tile < a.ntiles && ok && !stopped; tile += gridDim.x) {
        const int b = tile / per_img, r = tile - b * per_img;
        const int y0 = (r / a.tiles_x) * TY, x0 = (r % a.tiles_x) * 8 * SX;
        for (int h = 0; h < CH && ok; h++, u++) {
          if (u == a.stop_unit) { stopped = true; break; }
          if (hr > 0) ok = tc::mbar_wait(&hempty[hs], (hr - 1) & 1, a.wait_ns);
          if (!ok) break;
          tc::mbar_expect_tx(&hfull[hs], hbytes);
          for (int gq = 0; gq < groups; gq++)
            tc::tma_load_4d(halo + (size_t)hs * hbytes + (size_t)gq * SLAB, &tmap, cu * h + 8 * gq, x0, y0, b,
                            &hfull[hs]);
          if (resident) {
            if (u == 0)
              for (int blk = 0; blk < NTAP * CH; blk++) {
                tc::mbar_expect_tx(&wfull[blk], wbytes);
                tc::bulk_load(wst + (size_t)blk * wbytes, a.wpk + (size_t)blk * N * cu, wbytes, &wfull[blk]);
              }
          } else {
            for (int t = 0; t < NTAP && ok; t++, wq++) {
              if (wr > 0) ok = tc::mbar_wait(&wempty[ws], (wr - 1) & 1, a.wait_ns);
              if (!ok) break;
              tc::mbar_expect_tx(&wfull[ws], wbytes);
              tc::bulk_load(wst + (size_t)ws * wbytes, a.wpk + (size_t)(t * CH + h) * N * cu, wbytes, &wfull[ws]);
              if (++ws == NST) { ws = 0; wr++; }
            }
          }
          if (++hs == NH) { hs = 0; hr++; }
        }
      }
      s_issued[0] = u;
      s_issued[1] = resident ? (u > 0 ? NTAP * CH : 0) : wq;
    }
    __syncwarp();
  } else if (warp > NEPI) {
    if (lane == 0) {
      // MMA issuer of subtile sx.  Descriptors are linear in the start
      // address (field = address / 16): base descriptors plus offsets.
      const int sx = warp - NEPI - 1;
      const uint32_t idesc = tc::idesc_bf16(TM, N);
      const uint64_t ad0 = tc::sdesc(tc::smem_u32(halo), SLAB, TXH * 16) + (uint64_t)(8 * sx);
      const uint64_t bd0 = tc::sdesc(tc::smem_u32(wst), 128, cu * 16);
      int ws = 0, wr = 0;   // weight ring slot and round (streamed weights)
      int hs = 0, hr = 0;   // halo buffer and round
      int it = 0;
      for (int tile = blockIdx.x; tile < a.ntiles && ok; tile += gridDim.x, it++) {
        const int as = it & 1;
        const uint32_t acc = tmem + as * acc_cols + sx * N;
        for (int h = 0; h < CH && ok; h++) {
          ok = tc::mbar_wait(&hfull[hs], hr & 1, a.wait_ns);
          if (ok && h == 0 && it >= 2) ok = tc::mbar_wait(&aempty[as], ((it - 2) >> 1) & 1, a.wait_ns);
          if (!ok) break;
          tc::fence_after();
          const uint64_t adh = ad0 + (uint64_t)hs * (hbytes >> 4);
          if (KU >= 2 && resident && it > 0) {
            // steady state with resident weights and two or more MMAs per
            // tap: no waits or branches inside the tile (32 -> 32: 134
            // against 148 us; the one-MMA-per-tap first layer is slower this
            // way and keeps the general loop).  The loop stays rolled: fully
            // unrolled, the same body gave wrong results on a CTA's later
            // tiles, deterministically (the same error with a sleep after
            // every tap), so a code-generation effect rather than a race.
            const uint64_t bdh = bd0 + (uint64_t)h * (wbytes >> 4);
            const uint64_t wstep = (uint64_t)CH * (wbytes >> 4);
#pragma unroll 1
            for (int t = 0; t < NTAP; t++) {
              const uint64_t at = adh + (uint64_t)((t / 5) * TXH + t % 5);
              const uint64_t bt = bdh + (uint64_t)t * wstep;
#pragma unroll
              for (int kk = 0; kk < KU; kk++)
                tc::mma_bf16(acc, at + (uint64_t)(kk * (2 * SLAB / 16)), bt + (uint64_t)(16 * kk), idesc,
                             (t | kk | h) ? 1u : 0u);
            }
            tc::mma_commit(&hempty[hs]);
            if (++hs == NH) { hs = 0; hr++; }
            continue;
          }
          int dy = 0, dx = 0;
          for (int t = 0; t < NTAP && ok; t++) {
            const int wsl = resident ? t * CH + h : ws;
            // resident weights: waited for (and fenced) on the first tile only
            if (!resident || it == 0) {
              ok = tc::mbar_wait(&wfull[wsl], resident ? 0 : wr & 1, a.wait_ns);
              if (!ok) break;
              tc::fence_after();
            }
            const uint64_t at = adh + (uint64_t)(dy * TXH + dx);
            const uint64_t bt = bd0 + (uint64_t)wsl * (wbytes >> 4);
#pragma unroll
            for (int kk = 0; kk < KU; kk++)
              tc::mma_bf16(acc, at + (uint64_t)(kk * (2 * SLAB / 16)), bt + (uint64_t)(16 * kk), idesc,
                           (t | kk | h) ? 1u : 0u);
            if (!resident) {
              tc::mma_commit(&wempty[ws]);
              if (++ws == NST) { ws = 0; wr++; }
            }
            if (++dx == 5) { dx = 0; dy++; }
          }
          if (!ok) break;
          tc::mma_commit(&hempty[hs]);
          if (++hs == NH) { hs = 0; hr++; }
        }
        if (!ok) break;
        tc::mma_commit(&afull[as]);
      }
    }
    __syncwarp();
  } else {
    // epilogue warps
    const int quarter = warp & 3, half = warp >> 2;
    const uint32_t trow = tmem + ((uint32_t)(quarter * 32) << 16);
    const int sx0 = SX >= 2 ? half : 0, sxs = SX >= 2 ? 2 : 1;
    const int nlo = SX >= 2 ? 0 : half * (N / 2), nhi = SX >= 2 ? N : (half + 1) * (N / 2);
    int it = 0;
    for (int tile = blockIdx.x; tile < a.ntiles; tile += gridDim.x, it++) {
      const int as = it & 1;
      const bool got = __all_sync(0xffffffffu, tc::mbar_wait(&afull[as], (it >> 1) & 1, a.wait_ns));
      if (!got) { ok = false; break; }
      tc::fence_after();
      const int b = tile / per_img, r = tile - b * per_img;
      const int y = (r / a.tiles_x) * TY + 4 * quarter + (lane >> 3);
      const int x0 = (r % a.tiles_x) * 8 * SX;
      for (int sx = sx0; sx < SX; sx += sxs) {
        const int x = x0 + 8 * sx + (lane & 7);
        const bool fast = a.e.mode == 0;
        PixOut po{};
        if (fast) po = pix_out(a.e.out_bf, a.e.cout, a.g, b, y, x);
        int n0 = nlo;
        for (; n0 + 32 <= nhi; n0 += 32) {
          float v[32];
          tc::tmem_ld32(trow + as * acc_cols + sx * N + n0, v);
          if (fast && n0 + 32 <= a.e.cout) {
            relu_store<32>(po, s_bias, n0, v);
          } else {
#pragma unroll
            for (int q = 0; q < 4; q++) epilogue8(a.e, s_bias, a.g, b, y, x, n0 + 8 * q, v + 8 * q);
          }
        }
        for (; n0 < nhi; n0 += 8) {
          float v[8];
          tc::tmem_ld8(trow + as * acc_cols + sx * N + n0, v);
          if (fast && n0 + 8 <= a.e.cout) relu_store<8>(po, s_bias, n0, v);
          else epilogue8(a.e, s_bias, a.g, b, y, x, n0, v);
        }
      }
      tc::fence_before();
      __syncwarp();
      if (lane == 0) tc::mbar_arrive(&aempty[as]);
    }
  }
  if (!ok) s_fail = 1;
  __syncthreads();
  if (s_fail) {
    // every issuer waits (bounded) for its own MMAs, and the copies still in
    // flight get a bounded time, before TMEM is freed
    if (warp > NEPI && lane == 0) {
      tc::mma_commit(&drain[warp - NEPI - 1]);
      tc::mbar_wait(&drain[warp - NEPI - 1], 0, 10000000ull);
    }
    if (tid == 0) {
      atomicExch(a.err, 1);
      tc::drain_ring(hfull, NH, s_issued[0], 10000000ull);
      tc::drain_ring(wfull, resident ? NTAP * CH : NST, s_issued[1], 10000000ull);
    }
    __syncthreads();
  }
  tc::fence_before();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(tmem, ncols);
}

// ---------------------------------------------------------------------------
// row-tile convolution (image width 64, input channels 16, 32, 64 or 128),
// persistent and warp-specialised, one CTA per SM, 18 warps.
//
// A tile is two full image rows (M = 128 pixels, row-major), so the A
// operand of vertical offset dy is the aligned 128-pixel window starting at
// halo row dy: no operand window is shifted by a pixel.  The five horizontal
// taps are folded into N instead:
//     D[p][dx * CO + co] = sum_{dy, ci} in[p + (dy - 2, 0)][ci] w[co][dy][dx][ci]
//     out[y][x][co]      = sum_dx D[(y, (x + dx - 2) mod 64)][dx * CO + co]
// so one MMA of N = 5 CO (160 for 32 output channels) per (dy, 16 input
// channels) replaces five MMAs of N = CO, and the horizontal sum (periodic
// within the row) is done by the epilogue with warp shuffles.
//   warps 0-15  epilogue.  Warp w reads TMEM lanes 32 (w % 4) .., i.e. 32
//               pixels of one row half, and the 8-channel group w / 4 of the
//               output unit; w and w ^ 1 hold the two halves of a row and
//               swap, through shared memory, the few values that the lane
//               rotations of the horizontal sum carry across their edges.
//   warp 16     producer (one lane): TMA halo tiles (6 rows x 64 pixels x
//               up to 64 channels per channel unit) into `nh` buffers and
//               weight blocks (output unit, channel unit, dy) into a ring of
//               `nst` stages, or once when all blocks are resident.
//   warp 17     MMA issuer (one lane).
// Output channels are processed in units of CO (<= 32) into a ring of `nacc`
// TMEM accumulators of Nu = pad16(5 CO) columns.  Inputs of 128 channels are
// pipelined in two units of 64 channels, reloaded for every output unit.
// ---------------------------------------------------------------------------
constexpr int RT = 2;                  // image rows per tile
constexpr int RH = RT + 2 * PAD;       // halo rows
constexpr int RW = 64;                 // image width
constexpr int RSLAB = RH * RW * 16;    // bytes per 8 channels of a halo tile
constexpr int RMAXST = 40;             // weight stages / resident blocks
constexpr int RNACC = 4;               // accumulator slots at most
constexpr int REPI = 16;               // epilogue warps (four per TMEM lane quarter)
constexpr int RMAXH = 4;               // halo buffers at most
constexpr uint64_t kLimit = 1000000000ull;   // bound of every pipeline wait (ns)

struct RowArgs {
  const bf16* wpk;       // blocks ((o * CH + h) * 5 + dy) of Nu x cu, K-major core matrices
  int cout;              // real output channels
  int CO;                // output channels per unit (<= 32)
  int nuo;               // output units
  int Nu;                // pad16(5 CO)
  int nacc;              // accumulator slots (nacc Nu <= 512)
  int nst;               // weight stages (nuo CH 5: resident)
  int nh;                // halo buffers (1 .. RMAXH)
  int ntiles;            // batch * H / 2
  uint32_t hint;         // producer / issuer waits: sleep after every miss (ns)
  uint32_t ehint;        // epilogue waits: the same
  Img g;
  Epi e;
  int* err;
};

// x8 TMEM load without the wait (the caller waits once for several loads)
__device__ __forceinline__ void tmem_ld8_nw(uint32_t taddr, uint32_t* r) {
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
               : "r"(taddr));
}
// the wait, with 8 loaded registers passed through it
__device__ __forceinline__ void tmem_wait8(uint32_t* r) {
  asm volatile("tcgen05.wait::ld.sync.aligned;"
               : "+r"(r[0]), "+r"(r[1]), "+r"(r[2]), "+r"(r[3]), "+r"(r[4]), "+r"(r[5]), "+r"(r[6]), "+r"(r[7])
               :: "memory");
}
// no instruction: keeps the uses of r after the preceding wait
__device__ __forceinline__ void reg_after8(uint32_t* r) {
  asm volatile(""
               : "+r"(r[0]), "+r"(r[1]), "+r"(r[2]), "+r"(r[3]), "+r"(r[4]), "+r"(r[5]), "+r"(r[6]), "+r"(r[7])
               :: "memory");
}

// v[dx][c] = s[dx K + c] for the K (< 8) channels of a small output unit
template <int K>
__device__ __forceinline__ void spread_small(const uint32_t* s, uint32_t (*v)[8]) {
#pragma unroll
  for (int dx = 0; dx < 5; dx++)
#pragma unroll
    for (int c = 0; c < 8; c++) v[dx][c] = c < K ? s[dx * K + c] : 0u;
}

template <int KU, int CH, bool SMALL>
__global__ void __launch_bounds__(32 * (REPI + 2)) k_conv_rows(const __grid_constant__ CUtensorMap tmap, RowArgs a) {
  constexpr int cu = 16 * KU, groups = 2 * KU;   // channels and 8-channel slabs per channel unit
  constexpr uint32_t hbytes = (uint32_t)groups * RSLAB;
  extern __shared__ __align__(1024) unsigned char csm[];
  __shared__ __align__(8) uint64_t hfull[RMAXH], hempty[RMAXH], afull[RNACC], aempty[RNACC], wfull[RMAXST],
      wempty[RMAXST];
  __shared__ __align__(8) uint64_t xbar[2][REPI / 2];
  __shared__ __align__(8) uint64_t drain;   // failure path: the issuer's MMAs
  __shared__ __align__(16) float xbuf[2][REPI][4][16];   // edge values swapped between the two warps of a row
  __shared__ uint32_t tslot;
  __shared__ int s_fail;
  __shared__ long long s_issued[2];   // copies the producer issued: halo units, weight blocks
  __shared__ __align__(16) float s_bias[128];
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int Nu = a.Nu, CO = a.CO, NUO = a.nuo, NST = a.nst, NH = a.nh, NACC = a.nacc;
  const int nblk = NUO * CH * 5;
  const bool resident = NST >= nblk;
  unsigned char* halo = csm;                        // NH buffers
  unsigned char* wst = csm + (size_t)NH * hbytes;   // NST stages
  const uint32_t wbytes = (uint32_t)Nu * cu * 2;
  const int per_img = a.g.H / RT;
  const uint32_t ncols = tmem_cols(NACC * Nu);
  if (warp == 0) tc::tmem_alloc(&tslot, ncols);
  if (tid == 0) {
    for (int i = 0; i < RMAXH; i++) {
      tc::mbar_init(&hfull[i], 1);
      tc::mbar_init(&hempty[i], 1);
    }
    for (int i = 0; i < 2; i++)
      for (int p = 0; p < REPI / 2; p++) tc::mbar_init(&xbar[i][p], 2);   // one arrival per warp of the pair
    tc::mbar_init(&drain, 1);
    for (int i = 0; i < NACC; i++) {
      tc::mbar_init(&afull[i], 1);
      tc::mbar_init(&aempty[i], REPI);   // one arrival per epilogue warp
    }
    for (int s = 0; s < (resident ? nblk : NST); s++) {
      tc::mbar_init(&wfull[s], 1);
      tc::mbar_init(&wempty[s], 1);
    }
    tc::mbar_fence_init();
    s_fail = 0;
    s_issued[0] = s_issued[1] = 0;
  }
  for (int i = tid; i < 128; i += blockDim.x) s_bias[i] = (a.e.bias && i < a.e.cout) ? a.e.bias[i] : 0.f;
  tc::fence_before();
  __syncthreads();
  tc::fence_after();
  const uint32_t tmem = tslot;
  bool ok = true;
  if (warp == REPI) {
    if (lane == 0) {
      // producer (ring positions as slot / round counters, as in the halo kernel)
      int wq = 0, ws = 0, wr = 0;
      int hq = 0, hs = 0, hr = 0;
      bool first = true;
      for (int tile = blockIdx.x; tile < a.ntiles && ok; tile += gridDim.x) {
        const int b = tile / per_img, y0 = (tile - b * per_img) * RT;
        if (resident && first) {
          for (int blk = 0; blk < nblk; blk++) {
            tc::mbar_expect_tx(&wfull[blk], wbytes);
            tc::bulk_load(wst + (size_t)blk * wbytes, a.wpk + (size_t)blk * Nu * cu, wbytes, &wfull[blk]);
          }
        }
        first = false;
        for (int o = 0; o < NUO && ok; o++) {
          for (int h = 0; h < CH && ok; h++) {
            if (CH > 1 || o == 0) {
              if (hr > 0) ok = tc::mbar_wait(&hempty[hs], (hr - 1) & 1, kLimit, a.hint);
              if (!ok) break;
              tc::mbar_expect_tx(&hfull[hs], hbytes);
              // padded rows y0 .. y0 + 5 hold image rows y0 - 2 .. y0 + 3
              for (int gq = 0; gq < groups; gq++)
                tc::tma_load_4d(halo + (size_t)hs * hbytes + (size_t)gq * RSLAB, &tmap, cu * h + 8 * gq, PAD, y0, b,
                                &hfull[hs]);
              hq++;
              if (++hs == NH) { hs = 0; hr++; }
            }
            if (!resident) {
              for (int dy = 0; dy < 5 && ok; dy++, wq++) {
                if (wr > 0) ok = tc::mbar_wait(&wempty[ws], (wr - 1) & 1, kLimit, a.hint);
                if (!ok) break;
                tc::mbar_expect_tx(&wfull[ws], wbytes);
                tc::bulk_load(wst + (size_t)ws * wbytes, a.wpk + (size_t)((o * CH + h) * 5 + dy) * Nu * cu, wbytes,
                              &wfull[ws]);
                if (++ws == NST) { ws = 0; wr++; }
              }
            }
          }
        }
      }
      s_issued[0] = hq;
      s_issued[1] = resident ? (first ? 0 : nblk) : wq;
    }
    __syncwarp();
  } else if (warp == REPI + 1) {
    if (lane == 0) {
      // MMA issuer.  Descriptors are linear in the start address (field =
      // address / 16): base descriptors plus offsets.
      const uint32_t idesc = tc::idesc_bf16(TM, Nu);
      const uint64_t ad0 = tc::sdesc(tc::smem_u32(halo), RSLAB, 128);
      const uint64_t bd0 = tc::sdesc(tc::smem_u32(wst), 128, cu * 16);
      int ws = 0, wr = 0;       // weight ring slot and round
      int hs = 0, hr = 0;       // halo buffer and round (advanced after each halo unit's last use)
      int slot = 0, ar = 0;     // accumulator slot and round
      bool first = true;
      for (int tile = blockIdx.x; tile < a.ntiles && ok; tile += gridDim.x) {
        for (int o = 0; o < NUO && ok; o++) {
          if (ar > 0) ok = tc::mbar_wait(&aempty[slot], (ar - 1) & 1, kLimit, a.hint);
          if (!ok) break;
          tc::fence_after();
          const uint32_t acc = tmem + slot * Nu;
          for (int h = 0; h < CH && ok; h++) {
            if (CH > 1 || o == 0) {
              ok = tc::mbar_wait(&hfull[hs], hr & 1, kLimit, a.hint);
              if (!ok) break;
              tc::fence_after();
            }
            const uint64_t adh = ad0 + (uint64_t)hs * (hbytes >> 4);
            for (int dy = 0; dy < 5 && ok; dy++) {
              const int blk = (o * CH + h) * 5 + dy;
              const int wsl = resident ? blk : ws;
              if (!resident || first) {
                ok = tc::mbar_wait(&wfull[wsl], resident ? 0 : wr & 1, kLimit, a.hint);
                if (!ok) break;
                tc::fence_after();
              }
              const uint64_t at = adh + (uint64_t)(dy * RW);   // dy rows of 64 pixels x 16 bytes
              const uint64_t bt = bd0 + (uint64_t)wsl * (wbytes >> 4);
#pragma unroll
              for (int kk = 0; kk < KU; kk++)
                tc::mma_bf16(acc, at + (uint64_t)(kk * (2 * RSLAB / 16)), bt + (uint64_t)(16 * kk), idesc,
                             (dy | kk | h) ? 1u : 0u);
              if (!resident) {
                tc::mma_commit(&wempty[ws]);
                if (++ws == NST) { ws = 0; wr++; }
              }
            }
            if (!ok) break;
            if (CH > 1 || o == NUO - 1) {
              tc::mma_commit(&hempty[hs]);
              if (++hs == NH) { hs = 0; hr++; }
            }
          }
          if (!ok) break;
          tc::mma_commit(&afull[slot]);
          if (++slot == NACC) { slot = 0; ar++; }
        }
        first = false;
      }
    }
    __syncwarp();
  } else {
    // epilogue warps: `quarter` is the TMEM lane quarter (32 pixels of one
    // row half), `grp` the 8-channel group of the output unit
    const int quarter = warp & 3, grp = warp >> 2, pair = warp >> 1;
    const uint32_t trow = tmem + ((uint32_t)(quarter * 32) << 16);
    const int edge = lane < 2 ? lane : (lane >= 30 ? lane - 28 : -1);
    const bool active = SMALL ? grp == 0 : 8 * grp < CO;
    int aq = 0, slot = 0, ar = 0;   // accumulators used; slot and round
    for (int tile = blockIdx.x; tile < a.ntiles && ok; tile += gridDim.x) {
      const int b = tile / per_img;
      const int y = (tile - b * per_img) * RT + (quarter >> 1), x = 32 * (quarter & 1) + lane;
      const bool fast = a.e.mode == 0;
      PixOut po{};
      if (fast) po = pix_out(a.e.out_bf, a.e.cout, a.g, b, y, x);
      // (slot, ar) = (aq % NACC, aq / NACC), advanced with aq
      for (int o = 0; o < NUO; o++, aq++, slot = slot + 1 == NACC ? 0 : slot + 1, ar += slot == 0) {
        const int par = aq & 1;
        const bool got = __all_sync(0xffffffffu, tc::mbar_wait(&afull[slot], ar & 1, kLimit, a.ehint));
        if (!got) { ok = false; break; }
        tc::fence_after();
        const uint32_t tacc = trow + slot * Nu;
        uint32_t v[5][8];   // v[dx][c]: horizontal tap dx, channel 8 grp + c of this pixel
        if (active) {
          if (SMALL) {
            uint32_t s16[16];   // CO <= 3: the 5 CO used columns lie in the first 16
            tmem_ld8_nw(tacc, s16);
            tmem_ld8_nw(tacc + 8, s16 + 8);
            tmem_wait8(s16);
            reg_after8(s16 + 8);
            if (CO == 1) spread_small<1>(s16, v);
            else if (CO == 2) spread_small<2>(s16, v);
            else spread_small<3>(s16, v);
          } else {
#pragma unroll
            for (int dx = 0; dx < 5; dx++) tmem_ld8_nw(tacc + dx * CO + 8 * grp, v[dx]);
            tmem_wait8(v[0]);
#pragma unroll
            for (int dx = 1; dx < 5; dx++) reg_after8(v[dx]);
          }
        }
        tc::fence_before();
        __syncwarp();
        if (lane == 0) tc::mbar_arrive(&aempty[slot]);   // the accumulator is in registers
        // The horizontal sum rotates the 32 lanes by dx - 2.  The values
        // that the rotation wraps around (tap 0 of lanes 30-31, tap 1 of lane
        // 31, tap 3 of lane 0, tap 4 of lanes 0-1) are used only by pixels of
        // the partner warp (the other half of the row, periodically): swap
        // them with the partner first, then every rotation is exact.
        if (active && edge >= 0) {
          float4* xb = reinterpret_cast<float4*>(xbuf[par][warp][edge]);
          uint32_t sa[8], sb[8];
#pragma unroll
          for (int c = 0; c < 8; c++) {
            sa[c] = lane >= 30 ? v[0][c] : (lane == 0 ? v[3][c] : v[4][c]);
            sb[c] = lane == 31 ? v[1][c] : v[4][c];
          }
          xb[0] = make_float4(__uint_as_float(sa[0]), __uint_as_float(sa[1]), __uint_as_float(sa[2]), __uint_as_float(sa[3]));
          xb[1] = make_float4(__uint_as_float(sa[4]), __uint_as_float(sa[5]), __uint_as_float(sa[6]), __uint_as_float(sa[7]));
          xb[2] = make_float4(__uint_as_float(sb[0]), __uint_as_float(sb[1]), __uint_as_float(sb[2]), __uint_as_float(sb[3]));
          xb[3] = make_float4(__uint_as_float(sb[4]), __uint_as_float(sb[5]), __uint_as_float(sb[6]), __uint_as_float(sb[7]));
        }
        __syncwarp();   // the warp's edge values are written before its one arrival
        if (lane == 0) tc::mbar_arrive(&xbar[par][pair]);
        const bool swapped =
            __all_sync(0xffffffffu, tc::mbar_wait(&xbar[par][pair], (aq >> 1) & 1, kLimit, a.ehint));
        if (!swapped) { ok = false; break; }
        if (!active) continue;
        if (edge >= 0) {
          const float4* pb = reinterpret_cast<const float4*>(xbuf[par][warp ^ 1][edge]);
          const float4 q0 = pb[0], q1 = pb[1], q2 = pb[2], q3 = pb[3];
          const uint32_t ra[8] = {__float_as_uint(q0.x), __float_as_uint(q0.y), __float_as_uint(q0.z), __float_as_uint(q0.w),
                                  __float_as_uint(q1.x), __float_as_uint(q1.y), __float_as_uint(q1.z), __float_as_uint(q1.w)};
          const uint32_t rb[8] = {__float_as_uint(q2.x), __float_as_uint(q2.y), __float_as_uint(q2.z), __float_as_uint(q2.w),
                                  __float_as_uint(q3.x), __float_as_uint(q3.y), __float_as_uint(q3.z), __float_as_uint(q3.w)};
#pragma unroll
          for (int c = 0; c < 8; c++) {
            if (lane >= 30) v[0][c] = ra[c];
            if (lane == 31) v[1][c] = rb[c];
            if (lane == 0) { v[3][c] = ra[c]; v[4][c] = rb[c]; }
            if (lane == 1) v[4][c] = ra[c];
          }
        }
        float out[8];
#pragma unroll
        for (int c = 0; c < 8; c++) {
          const float t0 = __shfl_sync(0xffffffffu, __uint_as_float(v[0][c]), (lane + 30) & 31);
          const float t1 = __shfl_sync(0xffffffffu, __uint_as_float(v[1][c]), (lane + 31) & 31);
          const float t3 = __shfl_sync(0xffffffffu, __uint_as_float(v[3][c]), (lane + 1) & 31);
          const float t4 = __shfl_sync(0xffffffffu, __uint_as_float(v[4][c]), (lane + 2) & 31);
          out[c] = __uint_as_float(v[2][c]) + t0 + t1 + t3 + t4;
        }
        const int n0 = o * CO + 8 * grp;
        if (fast && n0 + 8 <= a.e.cout) relu_store<8>(po, s_bias, n0, out);
        else epilogue8(a.e, s_bias, a.g, b, y, x, n0, out);
      }
    }
  }
  if (!ok) s_fail = 1;
  __syncthreads();
  if (s_fail) {
    // the issuer waits (bounded) for its own MMAs, and the copies still in
    // flight get a bounded time, before TMEM is freed
    if (warp == REPI + 1 && lane == 0) {
      tc::mma_commit(&drain);
      tc::mbar_wait(&drain, 0, 10000000ull);
    }
    if (tid == 0) {
      atomicExch(a.err, 1);
      tc::drain_ring(hfull, NH, s_issued[0], 10000000ull);
      tc::drain_ring(wfull, resident ? nblk : NST, s_issued[1], 10000000ull);
    }
    __syncthreads();
  }
  tc::fence_before();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(tmem, ncols);
}

// ---------------------------------------------------------------------------
// gather convolution (few input channels): K chunks of 64 (tap, channel)
// ---------------------------------------------------------------------------
struct GatherArgs {
  const bf16* in;        // padded NHWC, cin channels
  int cin;
  const bf16* wpk;       // nchunk blocks of N x KC
  int N, nchunk;
  int npix;
  Img g;
  Epi e;
  int* err;
};

__global__ void __launch_bounds__(128) k_conv_gather(GatherArgs a) {
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
  const int HW = a.g.H * a.g.W;
  const int b = p / HW, rem = p - b * HW, y = rem / a.g.W, x = rem - (rem / a.g.W) * a.g.W;
  bool failed = false;
  int issued = 0;   // MMA commits issued (one per chunk)
  for (int c = 0; c < a.nchunk; c++) {
    const int s = c & 1;
    if (c >= 2) {
      const bool to = !tc::mbar_wait(&mbar[s], ((c - 2) >> 1) & 1);
      if (__syncthreads_or(to)) { failed = true; break; }
    }
    issued = c + 1;
    unsigned char* sA = sA0 + s * CHUNK_A;
    unsigned char* sB = sB0 + s * bbytes;
#pragma unroll 1
    for (int gq = 0; gq < KC / 8; gq++) {
      unsigned short u[8];
#pragma unroll
      for (int j = 0; j < 8; j++) {
        const int k = c * KC + gq * 8 + j;
        const int tap = k / a.cin, ci = k - tap * a.cin;
        unsigned short val = 0;
        if (tap < NTAP)
          val = __ldg(reinterpret_cast<const unsigned short*>(a.in + a.g.pix(b, y + tap / 5, x + tap % 5) * a.cin + ci));
        u[j] = val;
      }
      const uint4 v = make_uint4(u[0] | ((uint32_t)u[1] << 16), u[2] | ((uint32_t)u[3] << 16),
                                 u[4] | ((uint32_t)u[5] << 16), u[6] | ((uint32_t)u[7] << 16));
      *reinterpret_cast<uint4*>(sA + tc::kmajor_off(tid, gq * 8, KC)) = v;
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
    tc::drain_ring(mbar, 2, issued, 10000000ull);
  } else {
    tc::fence_after();
    const uint32_t trow = tmem + ((uint32_t)(warp * 32) << 16);
    for (int n0 = 0; n0 < N; n0 += 8) {
      float v[8];
      tc::tmem_ld8(trow + n0, v);
      epilogue8(a.e, a.e.bias, a.g, b, y, x, n0, v);
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
  const bf16* x;   // layer input, padded NHWC (xs channels per pixel, cin used)
  int cin, xs;
  const bf16* g;   // gradient of the pre-activation output, padded NHWC (cout)
  int cout, N, M;  // N = pad16(cout), M = 25 cin
  Img gm;
  int nrows, rows_per_cta;
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
  int issued = 0;   // MMA commits issued (one per chunk)
  for (int c = 0; c < nchunk; c++) {
    const int s = c & 1;
    if (c >= 2) {
      const bool to = !tc::mbar_wait(&mbar[s], ((c - 2) >> 1) & 1);
      if (__syncthreads_or(to)) { failed = true; break; }
    }
    issued = c + 1;
    unsigned char* sA = sA0 + s * CHUNK_A;
    unsigned char* sB = sB0 + s * bbytes;
    const int rr = r0 + c;
    const int b = rr / a.gm.H, y = rr - (rr / a.gm.H) * a.gm.H;
    // A[m][k] = x[b][y + dy][k + dx][ci] (padded coordinates)
    if (VECX) {
      const int k = tid & 63;
      for (int mg = tid >> 6; mg < TM / 8; mg += 2) {
        const int m = m0 + mg * 8;
        const int tap = m / a.cin, ci0 = m - tap * a.cin;
        uint4 v = make_uint4(0, 0, 0, 0);
        if (tap < NTAP)
          v = __ldg(reinterpret_cast<const uint4*>(a.x + a.gm.pix(b, y + tap / 5, k + tap % 5) * a.xs + ci0));
        const unsigned short* h = reinterpret_cast<const unsigned short*>(&v);
#pragma unroll
        for (int j = 0; j < 8; j++)
          *reinterpret_cast<unsigned short*>(sA + tc::kmajor_off(mg * 8 + j, k, KC)) = h[j];
      }
    } else {
      for (int i = tid; i < TM * KC; i += TM) {
        const int k = i & 63, rw = i >> 6;
        const int m = m0 + rw;
        const int tap = m / a.cin, ci = m - tap * a.cin;
        unsigned short val = 0;
        if (tap < NTAP)
          val = __ldg(reinterpret_cast<const unsigned short*>(a.x + a.gm.pix(b, y + tap / 5, k + tap % 5) * a.xs + ci));
        *reinterpret_cast<unsigned short*>(sA + tc::kmajor_off(rw, k, KC)) = val;
      }
    }
    // B[n][k] = g[b][y][k][n]
    const bf16* grow = a.g + a.gm.pix(b, y + PAD, PAD) * a.cout;
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
    tc::drain_ring(mbar, 2, issued, 10000000ull);
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
// NCHW (float or double) -> padded NHWC BF16 with (x - mean[c]) * inv_std[c]
// (out has Cs >= C channels per pixel; the others are left untouched)
template <class T>
__global__ void k_to_nhwc(const T* __restrict__ x, bf16* __restrict__ out, int B, int C, int Cs, Img g,
                          const float* __restrict__ mean, const float* __restrict__ inv_std) {
  const int HW = g.H * g.W;
  const size_t n = (size_t)B * C * HW;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const int c = (int)(i % C);
    const size_t pix = i / C;
    const int b = (int)(pix / HW), hw = (int)(pix - (size_t)b * HW);
    const float v = (float)x[((size_t)b * C + c) * HW + hw];
    store_px1(out, Cs, g, b, hw / g.W, hw % g.W, c, __float2bfloat16_rn((v - mean[c]) * inv_std[c]));
  }
}

// chunked packing for the gather kernel: forward (transpose = 0) or dgrad
__global__ void k_pack_chunks(const float* __restrict__ w, int cin, int cout, int transpose, bf16* __restrict__ out,
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
    out[(size_t)c * N * KC + tc::kmajor_off(n, kk, KC) / 2] = __float2bfloat16_rn(v);
  }
}

// packing for the halo kernel: blocks (tap, unit) of N x cu, cu = kpad / nu
// channels along K (kpad >= the real K channels; the padding is zero)
__global__ void k_pack_taps(const float* __restrict__ w, int cin, int cout, int transpose, bf16* __restrict__ out,
                            int N, int kpad, int nu) {
  const int kin = transpose ? cout : cin;
  const int nreal = transpose ? cin : cout;
  const int cu = kpad / nu;
  const size_t total = (size_t)NTAP * N * kpad;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
    const int blk = (int)(i / ((size_t)N * cu));
    const int rem = (int)(i - (size_t)blk * N * cu);
    const int n = rem / cu, cl = rem - n * cu;
    const int tap = blk / nu, ch = (blk - tap * nu) * cu + cl;
    float v = 0.f;
    if (n < nreal && ch < kin) {
      if (!transpose) v = w[((size_t)n * NTAP + tap) * cin + ch];
      else v = w[((size_t)ch * NTAP + (NTAP - 1 - tap)) * cin + n];
    }
    out[(size_t)blk * N * cu + tc::kmajor_off(n, cl, cu) / 2] = __float2bfloat16_rn(v);
  }
}

// packing for the row-tile kernel: blocks ((o * CH + h) * 5 + dy) of Nu x cu,
// row n = dx * CO + co of output unit o (rows 5 CO .. Nu - 1 zero), cu = kpad
// / CH channels along K (channels beyond the real K channels zero)
__global__ void k_pack_rows(const float* __restrict__ w, int cin, int cout, int transpose, bf16* __restrict__ out,
                            int CO, int Nu, int kpad, int CH, int nuo) {
  const int kin = transpose ? cout : cin;
  const int nreal = transpose ? cin : cout;
  const int cu = kpad / CH;
  const size_t total = (size_t)nuo * CH * 5 * Nu * cu;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
    const int blk = (int)(i / ((size_t)Nu * cu));
    const int rem = (int)(i - (size_t)blk * Nu * cu);
    const int n = rem / cu, cl = rem - n * cu;
    const int dy = blk % 5, oh = blk / 5, h = oh % CH, o = oh / CH;
    const int ch = h * cu + cl;
    float v = 0.f;
    if (n < 5 * CO) {
      const int dx = n / CO, co = o * CO + n % CO, tap = dy * 5 + dx;
      if (co < nreal && ch < kin) {
        if (!transpose) v = w[((size_t)co * NTAP + tap) * cin + ch];
        else v = w[((size_t)ch * NTAP + (NTAP - 1 - tap)) * cin + co];
      }
    }
    out[(size_t)blk * Nu * cu + tc::kmajor_off(n, cl, cu) / 2] = __float2bfloat16_rn(v);
  }
}

// MSE loss of y (NCHW FP32) against t; gradient 2 (y - t) / count as padded
// NHWC BF16
__global__ void k_mse(const float* __restrict__ y, const float* __restrict__ t, bf16* __restrict__ g, int B, int C,
                      Img gm, float* __restrict__ loss_sum) {
  const int HW = gm.H * gm.W;
  const size_t n = (size_t)B * C * HW;
  const float sc = 2.f / (float)n;
  float acc = 0.f;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const int b = (int)(i / ((size_t)C * HW));
    const int r = (int)(i - (size_t)b * C * HW);
    const int c = r / HW, hw = r - c * HW;
    const float d = y[i] - t[i];
    acc += d * d;
    store_px1(g, C, gm, b, hw / gm.W, hw % gm.W, c, __float2bfloat16_rn(sc * d));
  }
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) atomicAdd(loss_sum, acc / (float)n);
}

// db[c] += sum over interior pixels of g[p][c]
__global__ void k_bias_grad(const bf16* __restrict__ g, int B, int C, Img gm, float* __restrict__ db) {
  __shared__ float acc[128];
  for (int i = threadIdx.x; i < C; i += blockDim.x) acc[i] = 0.f;
  __syncthreads();
  const int HW = gm.H * gm.W;
  const size_t n = (size_t)B * HW * C;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const int c = (int)(i % C);
    const size_t pix = i / C;
    const int b = (int)(pix / HW), hw = (int)(pix - (size_t)b * HW);
    atomicAdd(&acc[c], __bfloat162float(g[gm.pix(b, hw / gm.W + PAD, hw % gm.W + PAD) * C + c]));
  }
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

// one convolution direction of a layer: packed weights and kernel choice
struct ConvPlan {
  int kin = 0, nout = 0;   // channels along K (input) and real output channels
  int N = 0;               // pad16(nout)
  bool halo = false;       // halo kernel (kin % 16 == 0) or gather kernel
  bool rows = false;       // row-tile kernel (width 64; replaces the halo kernel)
  int sx = 0;              // halo kernel tile width / 8
  int cu = 0;              // halo kernel: input channels per unit (64 or 32)
  int cps = 0;             // halo kernel: persistent CTAs per SM (0: the network's)
  int nst = 0;             // halo / row-tile kernel weight stages
  int nh = 0;              // halo / row-tile kernel halo buffers
  int co = 0, nuo = 0;     // row-tile kernel: output channels per unit, units
  int nun = 0, nacc = 0;   // row-tile kernel: MMA N per unit, accumulator slots
  int ch = 1;              // row-tile kernel: input channel units
  int nchunk = 0;          // gather kernel K chunks
  bf16* w = nullptr;
  size_t smem = 0;
};

struct CnnLayer {
  int cin, cout;
  int cs;              // channels of the stored input activation (cin, or 16 for 1..15 inputs)
  ConvPlan fwd, bwd;
  size_t woff, boff;   // offsets into the parameter vector
};

PFN_cuTensorMapEncodeTiled_v12000 g_encode = nullptr;

}  // namespace

struct pqg_cnn {
  int nl = 0, H = 0, W = 0, maxB = 0;
  int nsm = 1;                // SM count
  int cps = 1;                // persistent CTAs per SM
  uint32_t hint = 0;          // row-tile kernel: producer / issuer waits sleep this long after a miss (ns)
  uint32_t ehint = 0;         // row-tile kernel: epilogue waits, the same
  Img g{};
  std::vector<CnnLayer> L;
  size_t nparams = 0;
  float* params = nullptr;
  float* grads = nullptr;
  float* m = nullptr;
  float* v = nullptr;
  std::vector<bf16*> act;     // act[0] input, act[l] output of layer l-1 (post-ReLU); padded NHWC
  float* out = nullptr;       // last layer, NCHW FP32 (training)
  bf16* ga = nullptr;         // gradient ping-pong buffers, padded NHWC
  bf16* gb = nullptr;
  float* norm = nullptr;      // in_mean, in_inv_std, out_scale, out_shift, ones, zeros (128 each)
  int cmax = 0;
  float* loss = nullptr;
  int* err = nullptr;
  long long adam_t = 0;
  int stop_unit = -1;                          // failure tests (pqg_cnn_set_fault)
  unsigned long long wait_ns = 1000000000ull;  // bound of the halo-tile kernel's pipeline waits
};

namespace {

size_t gather_smem(int N) { return 2 * (size_t)CHUNK_A + 2 * (size_t)N * KC * 2; }

size_t halo_bytes(int sx, int kin) { return (size_t)(kin / 8) * (8 * sx + 2 * PAD) * TYH * 16; }

size_t rows_halo_bytes(int cu) { return (size_t)(cu / 8) * RSLAB; }

// row-tile kernel plan: false if the layer does not take it.  By default
// only 64 input channels and one output unit of at most 32 channels: there
// the MMA saving outweighs the longer epilogue (5 TMEM columns and 4 lane
// shuffles per output instead of 1 column), measured 277 us against 432 us
// for the 64 -> 32 layer at batch 512; for 16 or 32 input channels, or
// several output units, the epilogue's instruction issue bounds the kernel
// above the halo kernel's time.  PQG_CNN_ROWS=2 takes every layer that fits,
// PQG_CNN_ROWS=0 none.
// PQG_CNN_ROWS: 0 (default) no layer, 1 the 64 -> (<= 32) layers, 2 every
// layer the row-tile kernel takes.  With the halo kernel's issue loop free of
// divisions, the halo kernel measured faster on every layer (64 -> 32: 271
// against 290 us at batch 512).
bool plan_rows(ConvPlan& c, int W, int kin, int nout) {
  int mode = 0;
  if (const char* e = getenv("PQG_CNN_ROWS")) mode = atoi(e);
  if (mode <= 0) return false;
  if (W != RW || !(kin == 16 || kin == 32 || kin == 64 || kin == 128)) return false;
  if (!((nout <= 32 && (nout % 8 == 0 || nout <= 3)) || nout % 32 == 0)) return false;
  if (mode == 1 && !(kin == 64 && nout <= 32)) return false;
  c.ch = kin > 64 ? 2 : 1;
  const int cu = kin / c.ch;
  c.co = std::min(nout, 32);
  c.nuo = (nout + c.co - 1) / c.co;
  c.nun = pad16(5 * c.co);
  c.nacc = std::min(RNACC, 512 / c.nun);
  if (const char* e = getenv("PQG_CNN_NACC")) c.nacc = std::max(1, std::min(c.nacc, atoi(e)));
  const int nblk = c.nuo * c.ch * 5;
  const size_t wb = (size_t)c.nun * cu * 2, hb = rows_halo_bytes(cu);
  const size_t budget = 212 * 1024;   // + the kernel's static shared memory (10 KB)
  c.nst = 0;
  int nhmax = RMAXH;
  if (const char* e = getenv("PQG_CNN_NH")) nhmax = std::max(1, std::min(RMAXH, atoi(e)));
  for (int nh = nhmax; nh >= 1; nh--) {
    if (nblk <= RMAXST && nh * hb + nblk * wb <= budget) { c.nh = nh; c.nst = nblk; break; }
    const int nst = (int)std::min<size_t>(std::min(RMAXST, nblk - 1), (budget - nh * hb) / wb);
    if (nh * hb < budget && nst >= 4) { c.nh = nh; c.nst = nst; break; }
  }
  if (!c.nst) return false;
  c.smem = c.nh * hb + (size_t)c.nst * wb;
  // more than half of TMEM per CTA: keep one CTA per SM through shared memory
  if (c.nacc * c.nun > 256) c.smem = std::max<size_t>(c.smem, 120 * 1024);
  c.rows = true;
  return true;
}

void plan_conv(ConvPlan& c, int W, int kin, int nout) {
  c.kin = kin;
  c.nout = nout;
  c.N = pad16(nout);
  c.nchunk = (NTAP * kin + KC - 1) / KC;
  if (plan_rows(c, W, kin, nout)) return;
  c.halo = kin == 16 || kin == 32 || kin == 64 || kin == 128;
  if (c.halo) {
    // One persistent CTA per SM.  Prefer wide tiles (one MMA issuer per 8
    // columns: more independent MMA streams measured faster than deeper
    // weight rings, also for N = 64), then two halo buffers, then resident
    // weights; otherwise the deepest weight ring (at least 4 stages) within
    // about 224 KiB of shared memory.  Two accumulators of SX N columns must
    // fit in TMEM (512).  PQG_CNN_SX caps the width (tuning).
    const size_t budget = 224 * 1024;
    int cap = 8;
    if (const char* e = getenv("PQG_CNN_SX")) cap = std::max(1, atoi(e));
    // channel units of at most 64 (PQG_CNN_UNIT=32: of at most 32, for a
    // deeper weight ring beside two halo buffers)
    // 64 input channels in two units of 32: the weights fit resident beside
    // two halo buffers (64 -> 32: 244 against 269 us with one unit of 64)
    int umax = kin == 64 ? 32 : 64;
    if (const char* e = getenv("PQG_CNN_UNIT")) umax = atoi(e) == 32 ? 32 : 64;
    const int nu = kin > umax ? kin / umax : 1, cu = kin / nu;
    c.cu = cu;
    const size_t wb = (size_t)c.N * cu * 2;
    int best = -1;
    for (int sx : {8, 4, 2, 1}) {
      if (sx > cap || (W % (8 * sx)) || 2 * sx * c.N > 512) continue;
      // eight subtiles: instantiated for 32 input channels; measured faster
      // than four for N = 16 (the 32 -> 2 output layer) and slower for N = 32
      if (sx == 8 && (kin != 32 || c.N > 16)) continue;
      for (int nh : {2, 1}) {
        const size_t h = (size_t)nh * halo_bytes(sx, cu);
        if (h >= budget) continue;
        int nst, res;
        if (NTAP * nu <= MAXST && h + (size_t)NTAP * nu * wb <= budget) { nst = NTAP * nu; res = 1; }
        else if ((nst = (int)std::min<size_t>(std::min(MAXST, NTAP * nu - 1), (budget - h) / wb)) >= 4) res = 0;
        else continue;
        const int score = 4 * sx + 2 * nh + res;
        if (score > best) { best = score; c.sx = sx; c.nh = nh; c.nst = nst; }
      }
    }
    // tuning override for one layer shape:
    // PQG_CNN_HALO_<kin>_<nout>=<sx>,<nh>[,<CTAs per SM>]
    char key[64];
    snprintf(key, sizeof key, "PQG_CNN_HALO_%d_%d", kin, nout);
    if (const char* e = getenv(key)) {
      int sx = 0, nh = 0, cps = 0;
      const int nread = sscanf(e, "%d,%d,%d", &sx, &nh, &cps);
      if (nread == 3 && cps >= 1 && cps <= 4) c.cps = cps;
      if (nread >= 2 && (sx == 1 || sx == 2 || sx == 4 || (sx == 8 && kin == 32)) && nh >= 1 && nh <= MAXH &&
          W % (8 * sx) == 0 && 2 * sx * c.N <= 512) {
        const size_t h = (size_t)nh * halo_bytes(sx, cu);
        if (NTAP * nu <= MAXST && h + (size_t)NTAP * nu * wb <= budget) {
          best = 1; c.sx = sx; c.nh = nh; c.nst = NTAP * nu;
        } else if (h < budget && (budget - h) / wb >= 4) {
          best = 1; c.sx = sx; c.nh = nh;
          c.nst = (int)std::min<size_t>(std::min(MAXST, NTAP * nu - 1), (budget - h) / wb);
        }
      }
    }
    if (best < 0) c.halo = false;
  }
  c.smem = c.halo ? (size_t)c.nh * halo_bytes(c.sx, c.cu) + (size_t)c.nst * c.N * c.cu * 2 : gather_smem(c.N);
}

size_t plan_weight_elems(const ConvPlan& c) {
  if (c.rows) return (size_t)c.nuo * 5 * c.nun * c.kin;
  return c.halo ? (size_t)NTAP * c.N * c.kin : (size_t)c.nchunk * c.N * KC;
}

// 4-D map of a padded NHWC buffer; boxes of 8 channels x bw pixels x bh rows
int encode_map(CUtensorMap* m, const bf16* buf, int C, const pqg_cnn* net, int bw, int bh) {
  if (!g_encode) {
    void* fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess || !fn)
      return cfail(PQG_ERR_CUDA, "cuTensorMapEncodeTiled unavailable");
    g_encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
  }
  cuuint64_t dims[4] = {(cuuint64_t)C, (cuuint64_t)net->g.Wp, (cuuint64_t)net->g.Hp, (cuuint64_t)net->maxB};
  cuuint64_t strides[3] = {(cuuint64_t)C * 2, (cuuint64_t)net->g.Wp * C * 2, (cuuint64_t)net->g.Hp * net->g.Wp * C * 2};
  cuuint32_t box[4] = {8, (cuuint32_t)bw, (cuuint32_t)bh, 1};
  cuuint32_t es[4] = {1, 1, 1, 1};
  CUresult r = g_encode(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, const_cast<bf16*>(buf), dims, strides, box, es,
                        CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                        CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return cfail(PQG_ERR_CUDA, "cuTensorMapEncodeTiled failed");
  return PQG_OK;
}

typedef void (*HaloFn)(const __grid_constant__ CUtensorMap, HaloArgs);
// ks = input channels / 16, cu = channels per unit (64, or 32 for 64 and
// 128 input channels)
HaloFn halo_kernel(int sx, int ks, int cu) {
#define HK(S)                                                              \
  switch (ks) {                                                            \
    case 1: return k_conv_halo<S, 1, 4>;                                   \
    case 2: return k_conv_halo<S, 2, 4>;                                   \
    case 4: return cu == 32 ? k_conv_halo<S, 4, 2> : k_conv_halo<S, 4, 4>; \
    case 8: return cu == 32 ? k_conv_halo<S, 8, 2> : k_conv_halo<S, 8, 4>; \
    default: return nullptr;                                               \
  }
  if (sx == 8) return ks == 2 ? k_conv_halo<8, 2, 4> : nullptr;   // full 64-pixel rows, 32 input channels
  if (sx == 4) { HK(4) }
  if (sx == 2) { HK(2) }
  if (sx == 1) { HK(1) }
#undef HK
  return nullptr;
}

typedef void (*RowFn)(const __grid_constant__ CUtensorMap, RowArgs);
RowFn rows_kernel(int kin, bool small) {
#define RK(KU, CH)                                                     \
  return small ? k_conv_rows<KU, CH, true> : k_conv_rows<KU, CH, false>;
  switch (kin) {
    case 16: RK(1, 1)
    case 32: RK(2, 1)
    case 64: RK(4, 1)
    case 128: RK(4, 2)
    default: return nullptr;
  }
#undef RK
}

int launch_conv(pqg_cnn* net, const CnnLayer& l, bool dgrad, const bf16* in, int batch, const Epi& e,
                cudaStream_t st) {
  const ConvPlan& c = dgrad ? l.bwd : l.fwd;
  if (c.rows) {
    const bool small = c.co < 8;
    if (small && e.mode != 1) return cfail(PQG_ERR_UNSUPPORTED, "fewer than 8 channels only at the network output");
    CUtensorMap m;
    int rc = encode_map(&m, in, c.kin, net, RW, RH);
    if (rc) return rc;
    RowArgs a;
    a.wpk = c.w;
    a.cout = c.nout;
    a.CO = c.co;
    a.nuo = c.nuo;
    a.Nu = c.nun;
    a.nacc = c.nacc;
    a.nst = c.nst;
    a.nh = c.nh;
    a.ntiles = batch * (net->H / RT);
    a.hint = net->hint;
    a.ehint = net->ehint;
    a.g = net->g;
    a.e = e;
    a.err = net->err;
    const dim3 grid(std::min(a.ntiles, net->nsm * net->cps));
    auto fn = rows_kernel(c.kin, small);
    if (!fn) return cfail(PQG_ERR_UNSUPPORTED, "no convolution kernel for this channel count");
    fn<<<grid, 32 * (REPI + 2), c.smem, st>>>(m, a);
  } else if (c.halo) {
    CUtensorMap m;
    int rc = encode_map(&m, in, c.kin, net, 8 * c.sx + 2 * PAD, TYH);
    if (rc) return rc;
    HaloArgs a;
    a.cin = c.kin;
    a.wpk = c.w;
    a.N = c.N;
    a.nst = c.nst;
    a.nh = c.nh;
    a.tiles_x = net->W / (8 * c.sx);
    a.ntiles = batch * (net->H / TY) * a.tiles_x;
    a.g = net->g;
    a.e = e;
    a.err = net->err;
    a.stop_unit = net->stop_unit;
    a.wait_ns = net->wait_ns;
    const dim3 grid(std::min(a.ntiles, net->nsm * (c.cps ? c.cps : net->cps)));
    auto fn = halo_kernel(c.sx, c.kin / 16, c.cu);
    if (!fn) return cfail(PQG_ERR_UNSUPPORTED, "no convolution kernel for this channel count");
    fn<<<grid, 32 * (NEPI + 1 + c.sx), c.smem, st>>>(m, a);
  } else {
    GatherArgs a;
    a.in = in;
    a.cin = c.kin;
    a.wpk = c.w;
    a.N = c.N;
    a.nchunk = c.nchunk;
    a.npix = batch * net->H * net->W;
    a.g = net->g;
    a.e = e;
    a.err = net->err;
    k_conv_gather<<<a.npix / TM, TM, c.smem, st>>>(a);
  }
  CCUDA(cudaGetLastError());
  return PQG_OK;
}

int launch_wgrad(pqg_cnn* net, const CnnLayer& l, const bf16* x, const bf16* g, int batch, cudaStream_t st) {
  WgradArgs a;
  a.x = x;
  a.cin = l.cin;
  a.xs = l.cs;
  a.g = g;
  a.cout = l.cout;
  a.N = pad16(l.cout);
  a.M = NTAP * l.cin;
  a.gm = net->g;
  a.nrows = batch * net->H;
  const int mt = (a.M + TM - 1) / TM;
  const int target = 4 * 152;
  int ks = std::max(1, std::min(a.nrows, (target + mt - 1) / mt));
  a.rows_per_cta = (a.nrows + ks - 1) / ks;
  ks = (a.nrows + a.rows_per_cta - 1) / a.rows_per_cta;
  a.dw = net->grads + l.woff;
  a.err = net->err;
  const size_t smem = gather_smem(a.N);
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

// dynamic shared memory limit of every kernel: the device's opt-in maximum
// less room for the kernels' static shared memory
int set_attrs() {
  int dev = 0, optin = 0;
  CCUDA(cudaGetDevice(&dev));
  CCUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
  const int big = optin - 2048;
  for (int sx : {1, 2, 4})
    for (int ks : {1, 2, 4, 8})
      for (int cu : {64, 32})
        if (cu == 64 || ks >= 4)
          CCUDA(cudaFuncSetAttribute(halo_kernel(sx, ks, cu), cudaFuncAttributeMaxDynamicSharedMemorySize, big));
  CCUDA(cudaFuncSetAttribute(halo_kernel(8, 2, 32), cudaFuncAttributeMaxDynamicSharedMemorySize, big));
  for (int kin : {16, 32, 64, 128})
    for (bool small : {false, true})
      CCUDA(cudaFuncSetAttribute(rows_kernel(kin, small), cudaFuncAttributeMaxDynamicSharedMemorySize, optin - 12288));
  CCUDA(cudaFuncSetAttribute(k_conv_gather, cudaFuncAttributeMaxDynamicSharedMemorySize, big));
  CCUDA(cudaFuncSetAttribute(k_wgrad<true, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, big));
  CCUDA(cudaFuncSetAttribute(k_wgrad<true, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, big));
  CCUDA(cudaFuncSetAttribute(k_wgrad<false, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, big));
  CCUDA(cudaFuncSetAttribute(k_wgrad<false, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, big));
  return PQG_OK;
}

int grid_for(size_t n) { return (int)std::min<size_t>((n + 255) / 256, 152 * 16); }

int repack(pqg_cnn* net, cudaStream_t st) {
  for (auto& l : net->L) {
    for (int d = 0; d < 2; d++) {
      const ConvPlan& c = d ? l.bwd : l.fwd;
      if (c.rows)
        k_pack_rows<<<grid_for(plan_weight_elems(c)), 256, 0, st>>>(net->params + l.woff, l.cin, l.cout, d, c.w, c.co,
                                                                    c.nun, c.kin, c.ch, c.nuo);
      else if (c.halo)
        k_pack_taps<<<grid_for(plan_weight_elems(c)), 256, 0, st>>>(net->params + l.woff, l.cin, l.cout, d, c.w, c.N,
                                                                   c.kin, c.kin / c.cu);
      else
        k_pack_chunks<<<grid_for(plan_weight_elems(c)), 256, 0, st>>>(net->params + l.woff, l.cin, l.cout, d, c.w,
                                                                     c.N, c.nchunk);
    }
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
    Epi e{};
    e.cout = l.cout;
    e.bias = net->params + l.boff;
    if (i < net->nl - 1) {
      e.mode = 0;
      e.out_bf = net->act[i + 1];
    } else {
      e.mode = 1;
      e.out = out;
      e.out_f64 = out_f64;
      e.oscale = oscale;
      e.oshift = oshift;
    }
    int rc = launch_conv(net, l, false, net->act[i], batch, e, st);
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
  if (height < TY || height % TY || max_batch < 1)
    return cfail(PQG_ERR_UNSUPPORTED, "image height must be a positive multiple of 16");
  for (int i = 0; i <= nlayers; i++)
    if (channels[i] < 1 || channels[i] > 128) return cfail(PQG_ERR_UNSUPPORTED, "channels must be in 1..128");
  for (int i = 1; i < nlayers; i++)
    if (channels[i] % 8) return cfail(PQG_ERR_UNSUPPORTED, "hidden channel counts must be multiples of 8");
  pqg_cnn* net = new pqg_cnn();
  net->nl = nlayers;
  net->H = height;
  net->W = width;
  net->maxB = max_batch;
  net->g = Img{height, width, height + 2 * PAD, width + 2 * PAD};
  {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&net->nsm, cudaDevAttrMultiProcessorCount, dev);
    if (net->nsm < 1) net->nsm = 1;
    if (const char* e = getenv("PQG_CNN_CPS")) net->cps = std::max(1, std::min(4, atoi(e)));
    if (const char* e = getenv("PQG_CNN_HINT")) net->hint = (uint32_t)std::max(0, atoi(e));
    if (const char* e = getenv("PQG_CNN_EHINT")) net->ehint = (uint32_t)std::max(0, atoi(e));
  }
  size_t off = 0;
  for (int i = 0; i < nlayers; i++) {
    CnnLayer l{};
    l.cin = channels[i];
    l.cout = channels[i + 1];
    // the network input (few channels) is stored zero-padded to 16 channels
    // so that the first layer runs on the halo kernel
    l.cs = (i == 0 && l.cin < 16) ? 16 : l.cin;
    plan_conv(l.fwd, width, l.cs, l.cout);
    plan_conv(l.bwd, width, l.cout, l.cin);
    l.woff = off;
    off += (size_t)l.cout * NTAP * l.cin;
    l.boff = off;
    off += l.cout;
    net->L.push_back(l);
    net->cmax = std::max(net->cmax, std::max(l.cin, l.cout));
  }
  net->nparams = off;
  const size_t npad = (size_t)max_batch * net->g.Hp * net->g.Wp;
  const size_t npix = (size_t)max_batch * height * width;
  auto fail = [&](const char* what) {
    pqg_cnn_destroy(net);
    return cfail(PQG_ERR_NOMEM, std::string("allocation failed: ") + what);
  };
  if (cudaMalloc(&net->params, 4 * off) || cudaMalloc(&net->grads, 4 * off) || cudaMalloc(&net->m, 4 * off) ||
      cudaMalloc(&net->v, 4 * off))
    return fail("parameters");
  cudaMemset(net->params, 0, 4 * off);
  cudaMemset(net->m, 0, 4 * off);
  cudaMemset(net->v, 0, 4 * off);
  for (auto& l : net->L) {
    if (cudaMalloc(&l.fwd.w, 2 * plan_weight_elems(l.fwd)) || cudaMalloc(&l.bwd.w, 2 * plan_weight_elems(l.bwd)))
      return fail("packed weights");
  }
  net->act.assign(nlayers, nullptr);
  for (int i = 0; i < nlayers; i++)
    if (cudaMalloc(&net->act[i], npad * net->L[i].cs * 2) || cudaMemset(net->act[i], 0, npad * net->L[i].cs * 2))
      return fail("activations");
  if (cudaMalloc(&net->out, npix * net->L.back().cout * 4) || cudaMalloc(&net->ga, npad * net->cmax * 2) ||
      cudaMalloc(&net->gb, npad * net->cmax * 2) || cudaMalloc(&net->norm, 4 * 6 * 128) ||
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
  if (set_attrs() != PQG_OK) {
    const std::string msg = c_last_error;
    pqg_cnn_destroy(net);
    return cfail(PQG_ERR_CUDA, "initialisation failed: " + msg);
  }
  if (cudaDeviceSynchronize() != cudaSuccess) {
    pqg_cnn_destroy(net);
    return cfail(PQG_ERR_CUDA, "initialisation failed");
  }
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
    cudaFree(l.fwd.w);
    cudaFree(l.bwd.w);
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
// Failure tests: from pipeline unit `stop_unit` on (a unit is one tile and
// input-channel block of a CTA; < 0: never) the producer of the halo-tile
// convolutions issues no more copies, so the other warps' waits run out
// after `wait_ns` nanoseconds (0: the default of one second) and the kernel
// takes its failure path.
PQG_API int pqg_cnn_set_fault(pqg_cnn* net, int stop_unit, unsigned long long wait_ns) {
  if (!net) return cfail(PQG_ERR_INVALID, "NULL network");
  net->stop_unit = stop_unit;
  net->wait_ns = wait_ns ? wait_ns : 1000000000ull;
  return PQG_OK;
}

// Synchronizes `stream`; PQG_ERR_TIMEOUT if a pipeline wait of the
// network's kernels gave up since the last check (the flag is cleared).
PQG_API int pqg_cnn_status(pqg_cnn* net, void* stream) {
  if (!net) return cfail(PQG_ERR_INVALID, "NULL network");
  return check_err(net, (cudaStream_t)stream);
}

PQG_API int pqg_cnn_forward(pqg_cnn* net, const void* x, int x_f64, void* y, int y_f64, int batch, void* stream) {
  if (!net || !x || !y) return cfail(PQG_ERR_INVALID, "NULL argument");
  if (batch < 1 || batch > net->maxB) return cfail(PQG_ERR_INVALID, "bad batch size");
  cudaStream_t st = (cudaStream_t)stream;
  const size_t n = (size_t)batch * net->L[0].cin * net->H * net->W;
  if (x_f64)
    k_to_nhwc<double><<<grid_for(n), 256, 0, st>>>((const double*)x, net->act[0], batch, net->L[0].cin,
                                                   net->L[0].cs, net->g, net->norm, net->norm + 128);
  else
    k_to_nhwc<float><<<grid_for(n), 256, 0, st>>>((const float*)x, net->act[0], batch, net->L[0].cin, net->L[0].cs,
                                                  net->g, net->norm, net->norm + 128);
  CCUDA(cudaGetLastError());
  return forward_layers(net, batch, y, y_f64, net->norm + 256, net->norm + 384, st);
}

// gradients of the MSE loss of net(x) against t (both standardised, FP32
// NCHW device arrays) into the gradient vector; loss (host) if not NULL
PQG_API int pqg_cnn_backward(pqg_cnn* net, const float* x, const float* t, int batch, float* loss, void* stream) {
  if (!net || !x || !t) return cfail(PQG_ERR_INVALID, "NULL argument");
  if (batch < 1 || batch > net->maxB) return cfail(PQG_ERR_INVALID, "bad batch size");
  cudaStream_t st = (cudaStream_t)stream;
  const size_t npix = (size_t)batch * net->H * net->W;
  const float* ones = net->norm + 512;
  const float* zeros = net->norm + 640;
  k_to_nhwc<float><<<grid_for(npix * net->L[0].cin), 256, 0, st>>>(x, net->act[0], batch, net->L[0].cin,
                                                                   net->L[0].cs, net->g, zeros, ones);
  CCUDA(cudaGetLastError());
  int rc = forward_layers(net, batch, net->out, 0, ones, zeros, st);
  if (rc) return rc;
  CCUDA(cudaMemsetAsync(net->grads, 0, 4 * net->nparams, st));
  CCUDA(cudaMemsetAsync(net->loss, 0, 4, st));
  const int nl = net->nl;
  const int cl = net->L[nl - 1].cout;
  k_mse<<<grid_for(npix * cl), 256, 0, st>>>(net->out, t, net->ga, batch, cl, net->g, net->loss);
  CCUDA(cudaGetLastError());
  bf16* g = net->ga;     // gradient of the current layer's pre-activation output
  bf16* gn = net->gb;
  for (int i = nl - 1; i >= 0; i--) {
    const CnnLayer& l = net->L[i];
    k_bias_grad<<<(int)std::min<size_t>(1024, (npix * l.cout + 255) / 256), 256, 0, st>>>(
        g, batch, l.cout, net->g, net->grads + l.boff);
    CCUDA(cudaGetLastError());
    rc = launch_wgrad(net, l, net->act[i], g, batch, st);
    if (rc) return rc;
    if (i > 0) {
      // gradient of layer i's input, masked by the ReLU of layer i-1's output
      Epi e{};
      e.mode = 2;
      e.cout = l.cin;
      e.out_bf = gn;
      e.mask = net->act[i];
      rc = launch_conv(net, l, true, g, batch, e, st);
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
