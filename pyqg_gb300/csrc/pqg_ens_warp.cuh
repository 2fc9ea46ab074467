// Warp-owned FP32 transforms and the row / column kernels built on them, for
// ensemble groups of FP32 members (included inside pqg_ensemble.cu's
// anonymous namespace, after the pointwise helpers and the layout helpers).
//
// A group of G = n / 8 consecutive lanes owns one length-n sequence at a
// time: lane j holds the eight values x[j + G r] (r = 0..7) in registers.
// The transform is a radix-8 first stage in registers followed by the
// power-of-two Stockham stages of n / 8 (radix 8, then 4, then 2); between
// stages the values pass through a buffer private to the group, with
// __syncwarp and no block barrier.  On exit lane j holds X[j + G q]
// (q = 0..7), the index set it started with, so a forward transform, the
// pointwise physics and an inverse transform chain in registers.
//
// The row kernel gives every group one image row (C2R of the mixed U, V, Q
// planes, the products, R2C of uq, vq); the column kernel gives every group
// one spectral column of one member with all of its layers, so the layer
// inversion and the Adams-Bashforth update run in registers without
// clusters.  Every warp transforms its own rows or columns; block barriers
// only order the twiddle table's copy into shared memory and, in the staged
// row kernel, the CTA's coalesced tile loads and stores around them.

namespace wg {

__host__ __device__ constexpr int wpad(int i) { return i + (i >> 3); }

// Stride between the group buffers of one warp (complex values): the padded
// sequence, rounded so that consecutive groups start G banks (of 8 bytes)
// apart and the lanes of a warp touch distinct banks.
__host__ __device__ constexpr int wstride(int n) { return wpad(n) + ((((n / 8) - wpad(n)) % 16) + 16) % 16; }

// Stockham stages after the first: NS = product of the earlier radices.
// TS: twiddle table step (the table holds exp(-2 pi i m / (TS n))).
template <int N, int NS, bool INV, int TS>
struct WStages {
  static constexpr int G = N / 8;
  static constexpr int R = pow2_radix(ilog2(N / 8), ilog2(NS / 8));
  static constexpr int PER = 8 / R;   // butterflies of this stage per lane
  static __device__ __forceinline__ void run(float2 (&v)[8], float2* buf, int j, const float2* __restrict__ tw) {
    float2 x[PER][R];
#pragma unroll
    for (int i = 0; i < PER; i++) {
      const int b = j + G * i;
#pragma unroll
      for (int r = 0; r < R; r++) x[i][r] = buf[wpad(b + (N / R) * r)];
    }
#pragma unroll
    for (int i = 0; i < PER; i++) {
      const int b = j + G * i, jm = b & (NS - 1);
      const int ts = (N / (NS * R)) * jm;
#pragma unroll
      for (int r = 1; r < R; r++) {
        const float2 w = tw[TS * r * ts];
        x[i][r] = INV ? cmulc(x[i][r], w) : cmul(x[i][r], w);
      }
      Dft<R, INV>::run(x[i]);
    }
    if constexpr (NS * R == N) {
#pragma unroll
      for (int i = 0; i < PER; i++)
#pragma unroll
        for (int r = 0; r < R; r++) v[i + PER * r] = x[i][r];
    } else {
      __syncwarp();
#pragma unroll
      for (int i = 0; i < PER; i++) {
        const int b = j + G * i, jm = b & (NS - 1);
#pragma unroll
        for (int r = 0; r < R; r++) buf[wpad((b - jm) * R + jm + NS * r)] = x[i][r];
      }
      __syncwarp();
      WStages<N, NS * R, INV, TS>::run(v, buf, j, tw);
    }
  }
};

// Unnormalised length-N transform of the group's sequence (forward:
// exp(-2 pi i ...), inverse: exp(+...)); all lanes of the warp call it.
template <int N, bool INV, int TS = 1>
__device__ __forceinline__ void wfft(float2 (&v)[8], float2* buf, int j, const float2* __restrict__ tw) {
  Dft<8, INV>::run(v);
  if constexpr (N > 8) {
    __syncwarp();
#pragma unroll
    for (int r = 0; r < 8; r++) buf[wpad(8 * j + r)] = v[r];
    __syncwarp();
    WStages<N, 8, INV, TS>::run(v, buf, j, tw);
  }
}

// C2R packing of one row (the c2r_pre formula for one index at a time):
// z[r] = Z'[k], k = j + G r, from the half spectrum X (stride sx) and the
// length-2M table tw.
template <int M>
__device__ __forceinline__ void c2r_in(float2 (&z)[8], const float2* X, int sx, int j, const float2* tw) {
  constexpr int G = M / 8;
#pragma unroll
  for (int r = 0; r < 8; r++) {
    const int k = j + G * r;
    const float2 a = X[(size_t)k * sx], bb = X[(size_t)(M - k) * sx];
    if (k == 0) {
      z[r] = mk(sadd(a.x, bb.x), ssub(a.x, bb.x));
    } else {
      const float2 b = mk(bb.x, -bb.y);
      const float2 A = cadd(a, b), B = csub(a, b);
      const float2 D = cmulc(B, tw[k]);
      z[r] = mk(ssub(A.x, D.y), sadd(A.y, D.x));
    }
  }
}

// R2C unpacking of one row (the r2c_post formula for one index at a time):
// Z[q] = FFT_M(x[2m] + i x[2m+1]) at k = j + G q; Z[M - k] comes from lane
// (G - j) mod G of the group by a shuffle.  Writes X[k] (and X[M] for k = 0).
template <int M>
__device__ __forceinline__ void r2c_out(const float2 (&Z)[8], float2* X, int sx, int j, int lane, const float2* tw,
                                        bool store) {
  constexpr int G = M / 8;
  const float half = 0.5f;
  const int src = lane - j + ((G - j) & (G - 1));
#pragma unroll
  for (int q = 0; q < 8; q++) {
    const float2 send = j == 0 ? Z[(8 - q) & 7] : Z[7 - q];
    const float px = __shfl_sync(0xffffffffu, send.x, src);
    const float py = __shfl_sync(0xffffffffu, send.y, src);
    const int k = j + G * q;
    if (!store) continue;
    if (k == 0) {
      const float2 z0 = Z[0];
      X[0] = mk(sadd(z0.x, z0.y), 0.f);
      X[(size_t)M * sx] = mk(ssub(z0.x, z0.y), 0.f);
    } else {
      const float2 a = Z[q], b = mk(px, -py);
      const float2 A = cadd(a, b), B = csub(a, b);
      const float2 C = cmul(B, tw[k]);
      X[(size_t)k * sx] = mk(smul(half, sadd(A.x, C.y)), smul(half, ssub(A.y, C.x)));
    }
  }
}

}  // namespace wg

// ---------------------------------------------------------------------------
// row kernel (the e_row_adv step on warp-owned rows): every group of
// G = M / 8 lanes takes one row of one plane of one member.  Shared: the
// length-2M twiddle table, one buffer per group and, when STAGE, a tile of
// the CTA's RB rows of one mixed plane.
//
// A row's spectral values sit ny apart (the planes are k-major, for the
// column kernel), so with STAGE the CTA moves each plane's tile
// X[0..M][y0 .. y0 + RB) between global and shared memory with consecutive
// threads on consecutive rows (RB x 8 contiguous bytes per k), and the
// groups read and write their own row of the tile.  STAGE needs RB | ny.
// ---------------------------------------------------------------------------
// Register caps: 64 for the staged kernel (spills of 20-52 bytes at
// M = 64, 128; the 1024-member mixed ensemble steps in 0.66
// against 0.68 ms with 85), 128 otherwise;
// both measured faster than the compiler's unbounded choice (up to 125).
template <int LOGM, bool STAGE>
__global__ void __launch_bounds__(256, STAGE ? 4 : 2) e_row_w(EGeo g, EConsts<float> c, float2* scratch, const float* qphys,
                                                  const float2* __restrict__ twx, float scale, float* qout) {
  constexpr int M = 1 << LOGM, G = M / 8, RPW = 32 / G, N = 2 * M, SG = wg::wstride(M);
  extern __shared__ __align__(16) unsigned char esm[];
  float2* tw = reinterpret_cast<float2*>(esm);
  for (int i = threadIdx.x; i < N; i += blockDim.x) tw[i] = twx[i];
  __syncthreads();
  const int lane = threadIdx.x & 31, grp = lane / G, j = lane - grp * G, wib = threadIdx.x >> 5;
  const int W = blockDim.x >> 5, RB = W * RPW;
  float2* buf = tw + N + (size_t)(wib * RPW + grp) * SG;
  const int ny = g.ny, nz = g.nz, nk = g.nk;
  const long long row0 = ((long long)blockIdx.x * W + wib) * RPW;
  const long long nrows = (long long)g.B * nz * ny;
  if (!STAGE && row0 >= nrows) return;   // whole warp (the staged grid is exact)
  long long row = row0 + grp;
  const bool valid = row < nrows;
  if (!valid) row = nrows - 1;   // a copy of the last row: computed, not stored
  const int b = (int)(row / ((long long)nz * ny));
  const int rm = (int)(row - (long long)b * nz * ny), z = rm / ny, y = rm - z * ny;
  const size_t plane = (size_t)ny * nk;
  float2* base = scratch + (size_t)b * g.mstride + (size_t)z * plane + y;   // plane U, row y
  // staged: the tile and the group's row in it
  float2* sT = tw + N + (size_t)W * RPW * SG;
  const int yy = wib * RPW + grp, sts = RB + 1;
  int lrb = 0;
  while ((1 << lrb) < RB) lrb++;
  float2* tb = base - yy;   // plane U at the CTA's first row
  auto stage = [&](const float2* src) {
    for (int i = threadIdx.x; i < (M + 1) * RB; i += blockDim.x) {
      const int k = i >> lrb, r = i & (RB - 1);
      sT[k * sts + r] = src[(size_t)k * ny + r];
    }
  };
  auto unstage = [&](float2* dst) {
    for (int i = threadIdx.x; i < (M + 1) * RB; i += blockDim.x) {
      const int k = i >> lrb, r = i & (RB - 1);
      dst[(size_t)k * ny + r] = sT[k * sts + r];
    }
  };
  const float2* xin = STAGE ? sT + yy : nullptr;
  // q first (both products need it), then each velocity: C2R, product, R2C
  float2 q[8];
  if (qphys) {
    const float2* qr = reinterpret_cast<const float2*>(qphys + (size_t)row * N);
#pragma unroll
    for (int r = 0; r < 8; r++) q[r] = qr[j + G * r];
  } else {
    if constexpr (STAGE) {
      stage(tb + (size_t)2 * nz * plane);
      __syncthreads();
      wg::c2r_in<M>(q, xin, sts, j, tw);
    } else {
      wg::c2r_in<M>(q, base + (size_t)2 * nz * plane, ny, j, tw);
    }
    wg::wfft<M, true, 2>(q, buf, j, tw);
#pragma unroll
    for (int r = 0; r < 8; r++) q[r] = cscale(q[r], scale);
  }
  if (qout && valid) {
    float2* qo = reinterpret_cast<float2*>(qout + (size_t)row * N);
#pragma unroll
    for (int r = 0; r < 8; r++) qo[j + G * r] = q[r];
  }
  const float ub = c.Ubg[b * nz + z];
  float2 w[8];
#pragma unroll
  for (int f = 0; f < 2; f++) {
    float2* pl = base + (size_t)f * nz * plane;
    if constexpr (STAGE) {
      __syncthreads();   // the tile's previous contents are used up
      stage(tb + (size_t)f * nz * plane);
      __syncthreads();
      wg::c2r_in<M>(w, xin, sts, j, tw);
    } else {
      wg::c2r_in<M>(w, pl, ny, j, tw);
    }
    wg::wfft<M, true, 2>(w, buf, j, tw);
#pragma unroll
    for (int r = 0; r < 8; r++) {
      const float2 vv = cscale(w[r], scale);
      w[r] = f == 0 ? mk(smul(sadd(vv.x, ub), q[r].x), smul(sadd(vv.y, ub), q[r].y))
                    : mk(smul(vv.x, q[r].x), smul(vv.y, q[r].y));
    }
    wg::wfft<M, false, 2>(w, buf, j, tw);
    if constexpr (STAGE) {
      wg::r2c_out<M>(w, sT + yy, sts, j, lane, tw, true);
      __syncthreads();
      unstage(tb + (size_t)f * nz * plane);
    } else {
      wg::r2c_out<M>(w, pl, ny, j, lane, tw, valid);
    }
  }
}

// ---------------------------------------------------------------------------
// column kernel (the e_col_fused step on warp-owned columns): every group of
// G = N / 8 lanes takes spectral column k of member b with its NZ layers.
// Lane j holds the rows l = j + G q of every layer, so the inversion
// ph = sum_z' a[z, z'] qh[z'] and the update run in registers.  The new qh
// of a layer is written when its update is done: the inversions that read
// the current qh of every layer have all been formed before the first
// update.
// ---------------------------------------------------------------------------
// Register cap 128 (three layers spill 40-260 bytes): measured faster than
// the unbounded 170-255 registers, which leave 8-16 warps per SM.
template <int LOGN, int NZ>
__global__ void __launch_bounds__(256, 2) e_col_w(EGeo g, EConsts<float> c, float2* scratch, float2* qh,
                                               const float2* dqp, float2* dqpp, const float2* __restrict__ twy,
                                               float c1, float c2, float c3, int forcing) {
  constexpr int N = 1 << LOGN, G = N / 8, UPW = 32 / G, SG = wg::wstride(N);
  extern __shared__ __align__(16) unsigned char esm[];
  float2* tw = reinterpret_cast<float2*>(esm);
  for (int i = threadIdx.x; i < N; i += blockDim.x) tw[i] = twy[i];
  __syncthreads();
  const int lane = threadIdx.x & 31, grp = lane / G, j = lane - grp * G, wib = threadIdx.x >> 5;
  float2* buf = tw + N + (size_t)(wib * UPW + grp) * SG;
  const int nk = g.nk, nz = NZ;
  const long long unit0 = ((long long)blockIdx.x * (blockDim.x >> 5) + wib) * UPW;
  const long long nunits = (long long)g.B * nk;
  if (unit0 >= nunits) return;   // whole warp
  long long unit = unit0 + grp;
  const bool valid = unit < nunits;
  if (!valid) unit = nunits - 1;   // a copy of the last column: computed, not stored
  const int b = (int)(unit / nk), k = (int)(unit - (long long)b * nk);
  const size_t plane = (size_t)N * nk, ck0 = (size_t)k * N;
  float2* mb = scratch + (size_t)b * g.mstride + ck0;   // column k of plane (0, 0)
  // ph of the current qh of every layer (accumulated in z' order)
  float2 ph[NZ][8];
#pragma unroll
  for (int z = 0; z < NZ; z++)
#pragma unroll
    for (int r = 0; r < 8; r++) ph[z][r] = mk(0.f, 0.f);
#pragma unroll
  for (int z1 = 0; z1 < NZ; z1++)
#pragma unroll
    for (int r = 0; r < 8; r++) {
      const int l = j + G * r;
      const float2 qv = qh[sidx(b, z1, l, k, nz, N, nk)];
#pragma unroll
      for (int z = 0; z < NZ; z++) ph[z][r] = g_ph_acc(ph[z][r], c.a[((size_t)z * nz + z1) * plane + ck0 + l], qv);
    }
  const float rek = c.rek[b], kk = c.kk[k];
#pragma unroll
  for (int z = 0; z < NZ; z++) {
    const float2* pU = mb + (size_t)z * plane;
    // the tendency -(ik uqh + il vqh + ikQy ph), accumulated in the order of
    // g_tendency while one transformed field at a time is held: t = k uqh,
    // t += l vqh, then kQy ph
    float2 w[8], t[8];
#pragma unroll
    for (int r = 0; r < 8; r++) w[r] = pU[j + G * r];
    wg::wfft<N, false>(w, buf, j, tw);
#pragma unroll
    for (int r = 0; r < 8; r++) t[r] = mk(smul(kk, w[r].y), smul(kk, w[r].x));
    const float2* pV = pU + (size_t)nz * plane;
#pragma unroll
    for (int r = 0; r < 8; r++) w[r] = pV[j + G * r];
    wg::wfft<N, false>(w, buf, j, tw);
#pragma unroll
    for (int r = 0; r < 8; r++) {
      const float l = c.ll[j + G * r];
      t[r] = mk(sfma(l, w[r].y, t[r].x), sfma(l, w[r].x, t[r].y));
    }
    if (forcing) {
      const float2* pF = pU + (size_t)3 * nz * plane;
#pragma unroll
      for (int r = 0; r < 8; r++) w[r] = pF[j + G * r];
      wg::wfft<N, false>(w, buf, j, tw);
    }
    const float kQy = c.kQy[((size_t)b * nz + z) * nk + k];
    const bool drag = (rek != 0.f) && (z == NZ - 1);
#pragma unroll
    for (int r = 0; r < 8; r++) {
      const int l = j + G * r;
      const size_t ck = ck0 + l, o = sidx(b, z, l, k, nz, N, nk);
      const float2 p = ph[z][r];
      float2 d = mk(sfma(kQy, p.y, t[r].x), -sfma(kQy, p.x, t[r].y));
      if (drag) d = g_friction(d, smul(rek, c.k2l2[ck]), p);
      if (forcing) d = mk(sadd(d.x, w[r].x), sadd(d.y, w[r].y));
      const float2 qn = g_ab(c.filtr[ck], qh[o], d, dqp[o], dqpp[o], c1, c2, c3);
      if (valid) {
        qh[o] = qn;
        dqpp[o] = d;   // the newest tendency takes the oldest one's buffer
      }
      ph[z][r] = qn;   // the layer's ph is no longer needed: keep its new qh
    }
  }
  // mixed U, V of the new streamfunction, then Q = the new qh, per layer
#pragma unroll
  for (int z = 0; z < NZ; z++) {
    float2 p[8], w[8];
#pragma unroll
    for (int r = 0; r < 8; r++) {
      const int l = j + G * r;
      p[r] = mk(0.f, 0.f);
#pragma unroll
      for (int z1 = 0; z1 < NZ; z1++) p[r] = g_ph_acc(p[r], c.a[((size_t)z * nz + z1) * plane + ck0 + l], ph[z1][r]);
      w[r] = g_uh(c.ll[l], p[r]);
    }
    wg::wfft<N, true>(w, buf, j, tw);
    float2* pU = mb + (size_t)z * plane;
    if (valid) {
#pragma unroll
      for (int r = 0; r < 8; r++) pU[j + G * r] = w[r];
    }
#pragma unroll
    for (int r = 0; r < 8; r++) w[r] = g_vh(kk, p[r]);
    wg::wfft<N, true>(w, buf, j, tw);
    if (valid) {
      float2* pV = pU + (size_t)nz * plane;
#pragma unroll
      for (int r = 0; r < 8; r++) pV[j + G * r] = w[r];
    }
  }
#pragma unroll
  for (int z = 0; z < NZ; z++) {
    wg::wfft<N, true>(ph[z], buf, j, tw);
    if (valid) {
      float2* pQ = mb + (size_t)(2 * nz + z) * plane;
#pragma unroll
      for (int r = 0; r < 8; r++) pQ[j + G * r] = ph[z][r];
    }
  }
}
