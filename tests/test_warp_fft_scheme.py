"""The index scheme of the warp-owned FP32 ensemble transforms
(``pyqg_gb300/csrc/pqg_ens_warp.cuh``), restated in numpy and checked
against numpy's FFT on the CPU.

A group of G = n / 8 lanes owns a length-n sequence; lane j starts with
x[j + G r] (r < 8), runs a radix-8 stage in registers, then the
power-of-two Stockham stages of n / 8 (radix 8, then 4, then 2) through a
buffer addressed with one pad slot every 8 values, and ends with
X[j + G q] (q < 8).  The real-row packing computes one index at a time
(C2R: Z'[k] from X[k] and X[M - k]; R2C: X[k] from Z[k] and the value
Z[M - k] that the lane (G - j) mod G holds in register 7 - q, or (8 - q)
mod 8 for lane 0).  This is the emulation that was run before the
kernels' first GPU run; the kernels' results are checked on the GPU in
``tests/test_ensemble.py``.
"""
import numpy as np
import pytest


def _pow2_plan(n):
    """Radices of a power-of-two length (radix 8 stages, then 4s, then a
    2), the order of the library's compile-time plans."""
    if n == 1:
        return []
    a = int(np.log2(n))
    eights = a // 3 - 1 if (a % 3 == 1 and a >= 4) else a // 3
    fours = (2 if a >= 4 else 0) if a % 3 == 1 else (1 if a % 3 == 2 else 0)
    st = [8] * eights + [4] * fours
    rem = n // int(np.prod(st)) if st else n
    if rem == 2:
        st.append(2)
    assert int(np.prod(st)) == n
    return st


def _plan(n):
    return [8] + _pow2_plan(n // 8)


def _pad(i):
    return i + (i >> 3)


def _dft(v, inv):
    r = len(v)
    s = 1 if inv else -1
    return [sum(v[q] * np.exp(s * 2j * np.pi * q * p / r) for q in range(r)) for p in range(r)]


def wfft(x, inv):
    n = len(x)
    g = n // 8
    regs = [[x[j + g * r] for r in range(8)] for j in range(g)]
    buf = np.zeros(_pad(n) + 8, complex)
    tw = np.exp(-2j * np.pi * np.arange(n) / n)
    ns = 1
    stages = _plan(n)
    for si, radix in enumerate(stages):
        first, last = si == 0, si == len(stages) - 1
        nb, per = n // radix, 8 // radix
        outs = {}
        for j in range(g):
            for i in range(per):
                b = j + g * i
                v = list(regs[j]) if first else [buf[_pad(b + nb * r)] for r in range(radix)]
                jm = b % ns
                if ns > 1:
                    ts = (n // (ns * radix)) * jm
                    for r in range(1, radix):
                        w = tw[(r * ts) % n]
                        v[r] = v[r] * (np.conj(w) if inv else w)
                outs[(j, i)] = (b, jm, _dft(v, inv))
        for (j, i), (b, jm, o) in outs.items():
            for r in range(radix):
                if last:
                    q = i + per * r
                    assert b + ns * r == j + g * q     # lane j ends with X[j + G q]
                    regs[j][q] = o[r]
                else:
                    buf[_pad((b - jm) * radix + jm + ns * r)] = o[r]
        ns *= radix
    out = np.zeros(n, complex)
    for j in range(g):
        for q in range(8):
            out[j + g * q] = regs[j][q]
    return out


def c2r(X, m):
    """Inverse real transform of length 2m through the m-point warp
    transform (unnormalised)."""
    g, n = m // 8, 2 * m
    tw = np.exp(-2j * np.pi * np.arange(n) / n)
    z = np.zeros(m, complex)
    for j in range(g):
        for r in range(8):
            k = j + g * r
            a, bb = X[k], X[m - k]
            if k == 0:
                z[0] = complex(a.real + bb.real, a.real - bb.real)
            else:
                b = np.conj(bb)
                A, B = a + b, a - b
                D = B * np.conj(tw[k])
                z[k] = complex(A.real - D.imag, A.imag + D.real)
    y = wfft(z, True)
    out = np.zeros(n)
    out[0::2], out[1::2] = y.real, y.imag
    return out


def r2c(x, m):
    g, n = m // 8, 2 * m
    tw = np.exp(-2j * np.pi * np.arange(n) / n)
    Z = wfft(x[0::2] + 1j * x[1::2], False)
    X = np.zeros(m + 1, complex)
    for j in range(g):
        for q in range(8):
            k = j + g * q
            jp = (g - j) % g
            qp = ((8 - q) & 7) if jp == 0 else 7 - q
            if k == 0:
                X[0], X[m] = complex(Z[0].real + Z[0].imag, 0), complex(Z[0].real - Z[0].imag, 0)
            else:
                assert jp + g * qp == m - k            # the shuffled partner value
                a, b = Z[k], np.conj(Z[jp + g * qp])
                A, B = a + b, a - b
                C = B * tw[k]
                X[k] = 0.5 * complex(A.real + C.imag, A.imag - C.real)
    return X


@pytest.mark.parametrize("n", [8, 16, 32, 64, 128, 256])
def test_warp_transform_scheme(n):
    rng = np.random.default_rng(n)
    x = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    np.testing.assert_allclose(wfft(x, False), np.fft.fft(x), atol=1e-12 * n)
    np.testing.assert_allclose(wfft(x, True), np.fft.ifft(x) * n, atol=1e-12 * n)


@pytest.mark.parametrize("m", [8, 16, 32, 64, 128])
def test_row_packing_scheme(m):
    rng = np.random.default_rng(100 + m)
    x = rng.standard_normal(2 * m)
    X = np.fft.rfft(x)
    np.testing.assert_allclose(c2r(X, m), np.fft.irfft(X) * 2 * m, atol=1e-11 * m)
    np.testing.assert_allclose(r2c(x, m), X, atol=1e-12 * m)


def test_group_buffer_stride_spreads_banks():
    """Consecutive lane groups' buffers start G banks (of 8 bytes) apart
    modulo 16, so the lanes of a warp touch distinct banks in the
    transforms' first-stage stores (pqg_ens_warp.cuh: wstride)."""
    for n in (8, 16, 32, 64, 128, 256):
        g = n // 8
        stride = _pad(n) + (((g - _pad(n)) % 16) + 16) % 16
        assert stride >= _pad(n) and stride % 16 == g % 16
        # the 16 lanes of a half-warp (lane = group * G + j), store r = 0
        slots = {(grp * stride + _pad(8 * j)) % 16 for grp in range(max(1, 32 // g)) for j in range(g)
                 if grp * g + j < 16}
        assert len(slots) == 16, (n, sorted(slots))
