"""Post-kernel pulse compression in float64 (oracle).

Restates soundersim ``waveform.py``: the analytic raised-cosine windowed
sinc (:79-101), the explicit LFM matched filter (:104-123), the 'same'-mode
fast-time convolution (:126-138) and the coherent ``apply_waveform`` branch
(:141-160).
"""

import numpy as np

WINDOW_A = {"none": 1.0, "hann": 0.5, "hamming": 0.54}


def compressed_pulse(bandwidth, pulse_length, dt, window="hann",
                     construction="analytic"):
    """p(m dt), m in [-M, M], M = ceil(T/dt), p[M] = 1 (waveform.py:79-123)."""
    a = WINDOW_A[window]
    m = int(np.ceil(pulse_length / dt))
    if construction == "chirp":
        over = max(1, int(np.ceil(2.0 * bandwidth * dt)))
        dts = dt / over
        n = int(np.ceil(pulse_length / dts)) | 1
        t = (np.arange(n) - (n - 1) / 2) * dts
        s = np.exp(1j * np.pi * (bandwidth / pulse_length) * t * t)
        w = a + (1.0 - a) * np.cos(2.0 * np.pi * t / pulse_length)
        ker = np.conj(s[::-1]) * w
        nfft = 1 << (2 * n - 2).bit_length()
        y = np.fft.ifft(np.fft.fft(s, nfft) * np.fft.fft(ker, nfft))[:2 * n - 1]
        y = y / y[n - 1]
        p = np.zeros(2 * m + 1, np.complex128)
        j = np.arange(-m, m + 1)
        idx = n - 1 + j * over
        ok = (idx >= 0) & (idx < len(y)) & (np.abs(j * dt) <= pulse_length)
        p[ok] = y[idx[ok]]
        p[m] = 1.0
        return p, m
    x = bandwidth * dt * np.arange(-m, m + 1)
    p = (a * np.sinc(x) + 0.5 * (1.0 - a) * (np.sinc(x - 1.0)
                                             + np.sinc(x + 1.0))) / a
    return p, m


def convolve_fast_time(arr, kernel, center):
    """Direct 'same'-mode convolution along axis 1, kernel zero lag at
    ``center`` (waveform.py:126-138 computes it by FFT; this is the same
    linear convolution summed explicitly in complex128)."""
    arr = np.asarray(arr, np.complex128)
    ker = np.asarray(kernel, np.complex128)
    n = arr.shape[1]
    full = np.zeros((arr.shape[0], n + len(ker) - 1) + arr.shape[2:],
                    np.complex128)
    for j, kv in enumerate(ker):
        full[:, j:j + n] += kv * arr
    return full[:, center:center + n]
