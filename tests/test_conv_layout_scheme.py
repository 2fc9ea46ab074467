"""The operand addressing of the halo-tile convolution kernel
(``k_conv_halo`` in ``pyqg_gb300/csrc/pqg_cnn.cu``, descriptors from
``pyqg_gb300/csrc/pqg_tc.cuh``), restated in numpy and checked on the CPU
against a direct periodic 5x5 convolution.

What is restated, as the kernel does it:

* the image: NHWC with a periodic halo of 2 pixels on each side;
* the TMA load of a tile: per 8-channel slab a (16 + 4) x (8 SX + 4) pixel
  box, pixel-major, 16 bytes per pixel, slabs one after the other, one
  64-channel unit (or all channels) per halo buffer;
* the weight packing of ``k_pack_taps``: blocks (tap, unit) of N x cu,
  K-major core matrices (``kmajor_off``);
* the MMA operands: the canonical K-major, no-swizzle shared-memory layout
  (element (r, k) at start + (r / 8) SBO + (r % 8) 16 + (k / 8) LBO +
  (k % 8) 2 bytes) with the kernel's descriptors: A of subtile sx and tap
  (dy, dx) starts 8 sx + dy TXH + dx pixels into the halo buffer (LBO = one
  slab, SBO = one halo row), K step kk two slabs further; B of tap t and
  unit h is block t CH + h (LBO = 128, SBO = 16 cu), K step kk 256 bytes
  further;
* the accumulator: row m of subtile sx is output pixel (y0 + m / 8,
  x0 + 8 sx + m % 8).

The GPU kernel is checked against PyTorch in ``tests/test_closure.py``.
"""
import numpy as np
import pytest

PAD, TY, NTAP = 2, 16, 25


def kmajor_off(r, k, kc):
    """Byte offset of element (r, k) in a K-major tile with kc columns."""
    return ((r >> 3) * (kc >> 3) + (k >> 3)) * 128 + (r & 7) * 16 + (k & 7) * 2


def pack_taps(w, N, kpad, nu):
    """k_pack_taps (forward): w[co][tap][ci] -> blocks (tap, unit) of N x cu."""
    cout, _, cin = w.shape
    cu = kpad // nu
    out = np.zeros(NTAP * N * kpad)
    for blk in range(NTAP * nu):
        tap, unit = divmod(blk, nu)
        for n in range(N):
            for cl in range(cu):
                ch = unit * cu + cl
                v = w[n, tap, ch] if (n < cout and ch < cin) else 0.0
                out[blk * N * cu + kmajor_off(n, cl, cu) // 2] = v
    return out


def operand(smem, start, rows, ncols, lbo, sbo):
    """rows x ncols operand read from an element array (2-byte elements)
    with the canonical K-major no-swizzle layout."""
    r = np.arange(rows)[:, None]
    k = np.arange(ncols)[None, :]
    byte = start + (r // 8) * sbo + (r % 8) * 16 + (k // 8) * lbo + (k % 8) * 2
    assert (byte % 2 == 0).all() and byte.min() >= 0 and byte.max() // 2 < smem.size
    return smem[byte // 2]


def conv_halo_emulated(x, w, SX, KUM=4):
    """Forward convolution by the kernel's tiles and operand addressing.
    x: (B, H, W, cin) with cin in {16, 32, 64, 128}; w: (cout, 25, cin)."""
    B, H, W, cin = x.shape
    cout = w.shape[0]
    N = -(-cout // 16) * 16
    KS = cin // 16
    CH = KS // KUM if KS > KUM else 1
    KU = KS // CH
    cu, groups = 16 * KU, 2 * KU
    TXH, TYH = 8 * SX + 2 * PAD, TY + 2 * PAD
    SLAB = TXH * TYH * 16
    hbytes = groups * SLAB
    wbytes = N * cu * 2
    xp = np.pad(x, ((0, 0), (PAD, PAD), (PAD, PAD), (0, 0)), mode="wrap")
    wst = pack_taps(w, N, cin, CH)                      # all 25 x CH blocks resident
    out = np.zeros((B, H, W, cout))
    tiles_x, per_img = W // (8 * SX), (H // TY) * (W // (8 * SX))
    for tile in range(B * per_img):
        b, r = divmod(tile, per_img)
        y0, x0 = (r // tiles_x) * TY, (r % tiles_x) * 8 * SX
        acc = np.zeros((SX, 128, N))
        for h in range(CH):
            # TMA: slab gq holds channels cu h + 8 gq .. + 7 of the padded box
            halo = np.zeros(hbytes // 2)
            for gq in range(groups):
                c0 = cu * h + 8 * gq
                box = xp[b, y0:y0 + TYH, x0:x0 + TXH, c0:c0 + 8]          # (TYH, TXH, 8)
                halo[gq * SLAB // 2:(gq + 1) * SLAB // 2] = box.reshape(-1)
            for sx in range(SX):
                for t in range(NTAP):
                    dy, dx = divmod(t, 5)
                    a_start = (8 * sx + dy * TXH + dx) * 16          # bytes
                    b_start = (t * CH + h) * wbytes
                    for kk in range(KU):
                        A = operand(halo, a_start + kk * 2 * SLAB, 128, 16, SLAB, TXH * 16)
                        Bm = operand(wst, b_start + kk * 256, N, 16, 128, cu * 16)
                        acc[sx] += A @ Bm.T
        for sx in range(SX):
            m = np.arange(128)
            ys, xs = y0 + m // 8, x0 + 8 * sx + m % 8
            out[b, ys, xs, :] = acc[sx][:, :cout]
    return out


def conv_direct(x, w):
    """out[b, y, x, co] = sum_{tap, ci} x[b, y + dy - 2, x + dx - 2, ci] w[co, tap, ci] (periodic)."""
    out = np.zeros(x.shape[:3] + (w.shape[0],))
    for t in range(NTAP):
        dy, dx = divmod(t, 5)
        sh = np.roll(np.roll(x, -(dy - 2), axis=1), -(dx - 2), axis=2)
        out += np.einsum("byxc,oc->byxo", sh, w[:, t, :])
    return out


@pytest.mark.parametrize("cin,cout,SX,H,W", [
    (16, 128, 2, 16, 32),     # the first layer: input zero-padded to 16 channels
    (32, 32, 4, 32, 64),      # 32 -> 32 layers
    (64, 32, 4, 16, 32),      # 64 -> 32
    (128, 64, 4, 16, 32),     # 128 -> 64: two 64-channel units per tile
    (32, 2, 8, 16, 64),       # output layer: N = 16 for 2 channels, eight subtiles
])
def test_halo_kernel_addressing_is_the_convolution(cin, cout, SX, H, W):
    rng = np.random.default_rng(cin * 1000 + cout)
    x = rng.standard_normal((2, H, W, cin))
    w = rng.standard_normal((cout, NTAP, cin))
    got = conv_halo_emulated(x, w, SX)
    want = conv_direct(x, w)
    np.testing.assert_allclose(got, want, rtol=1e-12, atol=1e-10)


def test_kmajor_offsets_tile_the_block():
    """Every (row, column) of an N x KC K-major tile has its own 2-byte slot
    and the slots fill the block."""
    for n, kc in ((16, 16), (128, 64), (64, 128)):
        offs = {kmajor_off(r, k, kc) for r in range(n) for k in range(kc)}
        assert len(offs) == n * kc and min(offs) == 0 and max(offs) == 2 * n * kc - 2
