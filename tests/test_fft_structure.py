"""Float64 model of the double-float FFT's index structure.

The pulse-compression kernel (ss_waveform.cu, `df_fft_forward` /
`df_fft_inverse`) transforms a row in place without any reordering:
radix-4 decimation in frequency (block length L = 4q, butterfly b -> j =
b mod q, base = (b div q) L + j) takes the natural-order row to a base-4
digit-reversed spectrum, a radix-2 stage of block length 2 ends the
forward transform when log2 N is odd, the pulse spectrum made by the same
transform is in the same order, and the mirrored decimation-in-time
inverse (radix-2 first, then radix-4 with conjugate twiddles) returns
natural order. Twiddles w_L^{jk} sit at entries N - 4q + 3j + k - 1 of an
N-entry table. This model repeats those index computations in NumPy
complex128 and checks that forward, product and inverse give the circular
convolution, and that the forward output is a permutation of the DFT, for
every N from 2 to 2048.
"""

import numpy as np
import pytest


def _twiddles(n, lg):
    tw = np.zeros(n, complex)
    for lq in range(lg - 2, -1, -2):
        q = 1 << lq
        for r in range(3 * q):
            j, k = divmod(r, 3)
            t = j * (k + 1) * (n >> (lq + 2))
            tw[n - 4 * q + r] = np.exp(-2j * np.pi * t / n)
    return tw


def _forward(x, n, lg, tw):
    x = x.copy()
    for lq in range(lg - 2, -1, -2):
        q = 1 << lq
        T = tw[n - 4 * q:]
        b = np.arange(n >> 2)
        j = b & (q - 1)
        base = ((b >> lq) << (lq + 2)) + j
        a0, a1, a2, a3 = (x[base], x[base + q], x[base + 2 * q],
                          x[base + 3 * q])
        b0, b1, b2, b3 = a0 + a2, a0 - a2, a1 + a3, a1 - a3
        mib3 = -1j * b3
        x[base] = b0 + b2
        x[base + q] = (b1 + mib3) * T[3 * j]
        x[base + 2 * q] = (b0 - b2) * T[3 * j + 1]
        x[base + 3 * q] = (b1 - mib3) * T[3 * j + 2]
    if lg & 1:
        a0, a1 = x[0::2].copy(), x[1::2].copy()
        x[0::2], x[1::2] = a0 + a1, a0 - a1
    return x


def _inverse(x, n, lg, tw):
    x = x.copy()
    if lg & 1:
        a0, a1 = x[0::2].copy(), x[1::2].copy()
        x[0::2], x[1::2] = a0 + a1, a0 - a1
    for lq in range(lg & 1, lg - 1, 2):
        q = 1 << lq
        T = tw[n - 4 * q:]
        b = np.arange(n >> 2)
        j = b & (q - 1)
        base = ((b >> lq) << (lq + 2)) + j
        c0 = x[base]
        c1 = x[base + q] * np.conj(T[3 * j])
        c2 = x[base + 2 * q] * np.conj(T[3 * j + 1])
        c3 = x[base + 3 * q] * np.conj(T[3 * j + 2])
        d0, d1, d2, d3 = c0 + c2, c0 - c2, c1 + c3, c1 - c3
        x[base], x[base + 2 * q] = d0 + d2, d0 - d2
        x[base + q], x[base + 3 * q] = d1 + 1j * d3, d1 - 1j * d3
    return x


@pytest.mark.parametrize("lg", range(1, 12))
def test_forward_product_inverse_is_the_circular_convolution(lg):
    n = 1 << lg
    rng = np.random.default_rng(lg)
    x = rng.normal(size=n) + 1j * rng.normal(size=n)
    p = rng.normal(size=n) + 1j * rng.normal(size=n)
    tw = _twiddles(n, lg)
    X = _forward(x, n, lg, tw)
    ref_spec = np.fft.fft(x)
    # the forward output holds the DFT's values in a permuted order
    np.testing.assert_allclose(np.sort_complex(np.round(X, 8)),
                               np.sort_complex(np.round(ref_spec, 8)))
    y = _inverse(X * _forward(p, n, lg, tw), n, lg, tw) / n
    ref = np.fft.ifft(np.fft.fft(x) * np.fft.fft(p))
    assert np.abs(y - ref).max() <= 1e-12 * np.abs(ref).max()
    # every index the stages touch stays inside the row and the table
    for lq in range(lg - 2, -1, -2):
        q = 1 << lq
        b = np.arange(n >> 2)
        base = ((b >> lq) << (lq + 2)) + (b & (q - 1))
        assert base.min() >= 0 and (base + 3 * q).max() < n
        assert n - 4 * q + 3 * ((b & (q - 1)).max()) + 2 < n
