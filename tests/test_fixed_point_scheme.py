"""The arithmetic of the 64-bit block-fixed-point transform engine
(``pyqg_gb300/csrc/pqg_fixed.cuh``, the single model's default engine on
power-of-two grids), restated in Python integers and checked on the CPU
against exact rational arithmetic and numpy's FFT.

* ``q62``: the 32-bit-limb carry-chain product, word by word as the inline
  PTX forms it (``mul.hi`` / ``mad.lo.cc`` / ``madc.hi`` ...), then the sign
  correction, the rounding add at bit 61 and the funnel shifts, against
  floor((x w + 2^61) / 2^62).
* ``to_fixed`` / ``from_fixed``: the bit-level conversions against
  round-half-away-from-zero of v 2^S and the correctly rounded float of
  f 2^-S.
* ``block_shift``: the headroom rule |v| 2^S < 2^(62 - G).
* A whole transform: Q62 twiddles, the radix 8 / 4 / 2 Stockham stages of
  the library's plan (radix-8 butterfly with its sqrt(2)/2 products) and
  the conversions, against numpy.fft at lengths 8 .. 1024.

The GPU results of the engine are checked against the reference in
``tests/test_gpu_parity.py``.
"""
import struct
from fractions import Fraction

import numpy as np
import pytest

M32 = 0xFFFFFFFF
M64 = (1 << 64) - 1
Q62_ONE = 1 << 62
Q62_H8 = 3260954456333195553          # round(2^62 sqrt(2) / 2)
NAN_SHIFT = -1000000


# --- q62: the carry-chain product -------------------------------------------
def _hi(a, b):
    return (a * b) >> 32


def _lo(a, b):
    return (a * b) & M32


def q62(x, w):
    """round(x w / 2^62) as the device forms it from 32-bit limbs."""
    ux, uw = x & M64, w & M64
    x0, x1, w0, w1 = ux & M32, ux >> 32, uw & M32, uw >> 32
    # mul.hi r1 = hi(x0 w0)
    r1 = _hi(x0, w0)
    # mad.lo.cc r1 += lo(x0 w1)
    t = r1 + _lo(x0, w1); r1, c = t & M32, t >> 32
    # madc.hi r2 = hi(x0 w1) + c
    r2 = (_hi(x0, w1) + c) & M32
    # mad.lo.cc r1 += lo(x1 w0)
    t = r1 + _lo(x1, w0); r1, c = t & M32, t >> 32
    # madc.hi.cc r2 = hi(x1 w0) + r2 + c
    t = _hi(x1, w0) + r2 + c; r2, c = t & M32, t >> 32
    # madc.hi r3 = hi(x1 w1) + c
    r3 = (_hi(x1, w1) + c) & M32
    # mad.lo.cc r2 += lo(x1 w1); addc r3 += c
    t = r2 + _lo(x1, w1); r2, c = t & M32, t >> 32
    r3 = (r3 + c) & M32
    # signed product = unsigned - 2^64 (x < 0 ? w : 0) - 2^64 (w < 0 ? x : 0)
    hi = ((r3 << 32) | r2)
    hi = (hi - (((uw if x < 0 else 0) + (ux if w < 0 else 0)) & M64)) & M64
    lo1, h0, h1 = r1, hi & M32, hi >> 32
    # add.cc lo1 += 2^29 (bit 61 of the product); addc.cc h0; addc h1
    t = lo1 + 0x20000000; lo1, c = t & M32, t >> 32
    t = h0 + c; h0, c = t & M32, t >> 32
    h1 = (h1 + c) & M32
    up = ((h1 << 2) | (h0 >> 30)) & M32        # __funnelshift_l(h0, h1, 2)
    low = ((h0 << 2) | (lo1 >> 30)) & M32      # __funnelshift_l(lo1, h0, 2)
    r = (up << 32) | low
    return r - (1 << 64) if r >> 63 else r


def test_q62_matches_the_rounded_product():
    rng = np.random.default_rng(7)
    edges = [0, 1, -1, Q62_ONE, -Q62_ONE, Q62_ONE - 1, -(Q62_ONE - 1), Q62_H8, -Q62_H8, 1 << 61, -(1 << 61),
             (1 << 32) - 1, -(1 << 32), 3, -3]
    pairs = [(a, b) for a in edges for b in edges]
    for _ in range(20000):
        ex, ew = int(rng.integers(0, 63)), int(rng.integers(0, 63))
        x = int(rng.integers(-(1 << ex), (1 << ex) + 1))
        w = int(rng.integers(-(1 << ew), (1 << ew) + 1))
        pairs.append((x, w))
    for x, w in pairs:
        assert q62(x, w) == (x * w + (1 << 61)) >> 62, (x, w)


# --- conversions ---------------------------------------------------------------
def _bits(v):
    return struct.unpack("<Q", struct.pack("<d", v))[0]


def _float(b):
    return struct.unpack("<d", struct.pack("<Q", b))[0]


def bexp(v):
    return (_bits(v) & 0x7FFFFFFFFFFFFFFF) >> 52


def block_shift(emax, G):
    return NAN_SHIFT if emax >= 2047 else 1084 - G - emax


def to_fixed(v, S):
    b = _bits(v)
    E, m = (b >> 52) & 0x7FF, b & ((1 << 52) - 1)
    if E:
        m |= 1 << 52
    else:
        E = 1
    k = E - 1075 + S
    if k >= 0:
        r = m << min(k, 10)
    else:
        sh = -k
        r = 0 if sh >= 63 else (m + (1 << (sh - 1))) >> sh
    return -r if b >> 63 else r


def from_fixed(f, S):
    if S == NAN_SHIFT:
        return float("nan")
    if f == 0:
        return 0.0
    sign = 1 if f < 0 else 0
    a = -f if f < 0 else f
    lz = 64 - a.bit_length()
    n = (a << lz) & M64
    mant, rem = n >> 11, n & 0x7FF
    if rem > 0x400 or (rem == 0x400 and mant & 1):
        mant += 1
    e = 63 - lz - S
    if mant == 1 << 53:
        mant >>= 1
        e += 1
    E = e + 1023
    if E <= 0:
        return -0.0 if sign else 0.0
    return _float((sign << 63) | (E << 52) | (mant & ((1 << 52) - 1)))


def _round_half_away(q):
    n = abs(q.numerator) * 2 + q.denominator
    r = n // (2 * q.denominator)
    return -r if q < 0 else r


def test_to_fixed_rounds_half_away_from_zero():
    rng = np.random.default_rng(11)
    for _ in range(5000):
        G = int(rng.integers(2, 15))
        v = float(rng.standard_normal() * 10.0 ** rng.integers(-30, 30))
        S = block_shift(bexp(v), G)
        for vv in (v, v * 2.0 ** -int(rng.integers(0, 70))):      # the largest element and smaller ones
            f = to_fixed(vv, S)
            assert f == _round_half_away(Fraction(vv) * Fraction(2) ** S), (vv, S)
            assert abs(f) < 1 << (62 - G)
    # exact halves, both signs
    for S in (0, 3, 20):
        for k in range(1, 40):
            v = (2 * k + 1) / 2.0 ** (S + 1)
            assert to_fixed(v, S) == k + 1 and to_fixed(-v, S) == -(k + 1)


def test_from_fixed_is_correctly_rounded():
    rng = np.random.default_rng(12)
    for _ in range(5000):
        nb = int(rng.integers(1, 63))
        f = int(rng.integers(-(1 << nb), (1 << nb) + 1))
        S = int(rng.integers(-200, 900))
        got = from_fixed(f, S)
        want = float(Fraction(f) / Fraction(2) ** S)
        if want != 0.0 and abs(want) < 2.2250738585072014e-308:
            continue                       # below the normal range: flushed to zero by design
        assert got == want, (f, S)
    # ties go to even
    for S in (0, 10):
        f = (1 << 53) + 1                  # halfway between two doubles after the shift
        assert from_fixed(f, S) == float(Fraction(f) / Fraction(2) ** S)


def test_round_trip_and_nan_marker():
    rng = np.random.default_rng(13)
    for _ in range(2000):
        v = float(rng.standard_normal() * 10.0 ** rng.integers(-20, 20))
        S = block_shift(bexp(v), 4)
        # 58 bits kept for the largest element: the round trip is exact
        assert from_fixed(to_fixed(v, S), S) == v
    assert block_shift(bexp(float("inf")), 4) == NAN_SHIFT
    assert np.isnan(from_fixed(123, NAN_SHIFT))


# --- a whole transform -----------------------------------------------------------
def _pow2_eights(a):
    return a // 3 - 1 if (a % 3 == 1 and a >= 4) else a // 3


def _pow2_fours(a):
    return (2 if a >= 4 else 0) if a % 3 == 1 else (1 if a % 3 == 2 else 0)


def _radix(a, s):
    e, f = _pow2_eights(a), _pow2_fours(a)
    return 8 if s < 3 * e else (4 if s < 3 * e + 2 * f else 2)


def _q62_twiddles(n):
    mp = pytest.importorskip("mpmath")
    mp.mp.prec = 200
    out = []
    for m in range(n):
        ang = 2 * mp.pi * m / n
        out.append((int(mp.nint(mp.cos(ang) * Q62_ONE)), int(mp.nint(-mp.sin(ang) * Q62_ONE))))
    return out


def test_q62_constants_are_correctly_rounded():
    import os
    import re
    src = open(os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))),
                            "pyqg_gb300", "csrc", "pqg_fixed.cuh")).read()
    consts = {k: int(v) for k, v in re.findall(r"constexpr \w+ (kQ62One|kQ62H8|kNanShift) = (-?\d+)", src)}
    assert consts == {"kQ62One": Q62_ONE, "kQ62H8": Q62_H8, "kNanShift": NAN_SHIFT}
    mp = pytest.importorskip("mpmath")
    mp.mp.prec = 200
    assert Q62_H8 == int(mp.nint(mp.sqrt(2) / 2 * Q62_ONE))
    tw = _q62_twiddles(16)
    assert tw[2][0] == Q62_H8 and tw[2][1] == -Q62_H8 and tw[4] == (0, -Q62_ONE)


def _cmul(a, w):
    return (q62(a[0], w[0]) - q62(a[1], w[1]), q62(a[0], w[1]) + q62(a[1], w[0]))


def _cmulc(a, w):
    return (q62(a[0], w[0]) + q62(a[1], w[1]), q62(a[1], w[0]) - q62(a[0], w[1]))


def _add(a, b):
    return (a[0] + b[0], a[1] + b[1])


def _sub(a, b):
    return (a[0] - b[0], a[1] - b[1])


def _rot(a, inv):       # * -i (forward) / +i (inverse)
    return (-a[1], a[0]) if inv else (a[1], -a[0])


def _dft(v, inv):
    if len(v) == 2:
        return [_add(v[0], v[1]), _sub(v[0], v[1])]
    if len(v) == 4:
        a, b = _add(v[0], v[2]), _sub(v[0], v[2])
        c, d = _add(v[1], v[3]), _rot(_sub(v[1], v[3]), inv)
        return [_add(a, c), _add(b, d), _sub(a, c), _sub(b, d)]
    e, o = _dft(v[0::2], inv), _dft(v[1::2], inv)
    t = o[1]
    o[1] = ((q62(t[0] - t[1], Q62_H8), q62(t[0] + t[1], Q62_H8)) if inv
            else (q62(t[0] + t[1], Q62_H8), q62(t[1] - t[0], Q62_H8)))
    o[2] = _rot(o[2], inv)
    t = o[3]
    o[3] = ((q62(-(t[0] + t[1]), Q62_H8), q62(t[0] - t[1], Q62_H8)) if inv
            else (q62(t[1] - t[0], Q62_H8), q62(-(t[0] + t[1]), Q62_H8)))
    return [_add(e[r], o[r]) for r in range(4)] + [_sub(e[r], o[r]) for r in range(4)]


def fixed_fft(x, inv, G):
    """The engine's transform of one complex sequence: block shift, Stockham
    stages of the library's radix plan, conversion back (unnormalised)."""
    n = len(x)
    emax = max(max(bexp(float(v.real)), bexp(float(v.imag))) for v in x)
    S = block_shift(emax, G)
    buf = [(to_fixed(float(v.real), S), to_fixed(float(v.imag), S)) for v in x]
    tw = _q62_twiddles(n)
    a, ns = n.bit_length() - 1, 1
    while ns < n:
        R = _radix(a, ns.bit_length() - 1)
        nb = n // R
        out = [None] * n
        for j in range(nb):
            v = [buf[j + r * nb] for r in range(R)]
            jm = j % ns
            if ns > 1:
                ts = (n // (ns * R)) * jm
                for r in range(1, R):
                    v[r] = _cmulc(v[r], tw[r * ts]) if inv else _cmul(v[r], tw[r * ts])
            v = _dft(v, inv)
            for r in range(R):
                out[(j - jm) * R + jm + r * ns] = v[r]
        buf = out
        ns *= R
    return np.array([complex(from_fixed(p[0], S), from_fixed(p[1], S)) for p in buf])


@pytest.mark.parametrize("n", [8, 16, 32, 64, 128, 256, 1024])
@pytest.mark.parametrize("peak", [1.0, 1e3])
def test_fixed_point_transform_against_numpy(n, peak):
    """Normwise error against numpy.fft within the engine's bound: the
    sequence's largest element sets the quantum 2^-(62 - G) max|x|, and the
    roundings of the stages add up to about sqrt(n) quanta relative to
    ||X|| = sqrt(n) ||x|| (measured 0.4-0.7 of that bound from n = 128 on;
    below it the error is numpy's own, about 1.5e-16)."""
    rng = np.random.default_rng(100 + n)
    x = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    x[3] *= peak                             # a large element sets the block shift
    G = (n.bit_length() - 1) + 2
    bound = max(4e-16, 2.0 * 2.0 ** -(62 - G) * np.sqrt(n) * np.abs(x).max() / np.linalg.norm(x))
    for inv in (False, True):
        got = fixed_fft(x, inv, G)
        want = np.fft.ifft(x) * n if inv else np.fft.fft(x)
        err = np.linalg.norm(got - want) / np.linalg.norm(want)
        assert err < bound, (n, inv, err, bound)
    # the round trip returns the input within twice the bound
    back = fixed_fft(fixed_fft(x, False, G), True, G) / n
    assert np.linalg.norm(back - x) / np.linalg.norm(x) < 2 * bound
