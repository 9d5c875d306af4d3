"""Frequency-sampled facet synthesis in float64 (oracle).

Restates soundersim ``compare/multifreq.py``: midpoint band sampling
(:45-49), raised-cosine weights (:52-55) and the per-position synthesis
y(t) = sum_k Wbar_k H(f_k) exp(2j pi (f_k - f0) t) with H(f_k) the LPA facet
sum at wavenumber 2 pi f_k / c, either with full per-frequency amplitudes or
with amplitudes frozen at f0 (:58-98). ``synth_traces`` generalises the
per-position referee to every trace of a track.
"""

import numpy as np

from .lpa import lpa_field
from .waveform import WINDOW_A


def band_frequencies(f0, bandwidth, n_freq):
    return f0 - bandwidth / 2.0 + (np.arange(n_freq) + 0.5) * (bandwidth
                                                               / n_freq)


def window_weights(freqs, f0, bandwidth, window):
    a = WINDOW_A[window]
    return a + (1.0 - a) * np.cos(2.0 * np.pi * (freqs - f0) / bandwidth)


def band_response(p, c, nrm, area, e1, e2, *, gamma, f0, bandwidth, cc,
                  n_freq, freeze_amplitudes=False):
    """H(f_k) for one position (multifreq.py:78-96)."""
    freqs = band_frequencies(f0, bandwidth, n_freq)
    r = np.linalg.norm(p - c, axis=-1)
    H = np.empty(n_freq, np.complex128)
    if freeze_amplitudes:
        k0 = 2.0 * np.pi * f0 / cc
        c0, _ = lpa_field(p, c, nrm, area, e1, e2, k0, gamma)
        amp0 = c0 * np.exp(2j * k0 * r)
    for j, f in enumerate(freqs):
        k = 2.0 * np.pi * f / cc
        if freeze_amplitudes:
            H[j] = np.sum(amp0 * np.exp(-2j * k * r))
        else:
            H[j] = np.sum(lpa_field(p, c, nrm, area, e1, e2, k, gamma)[0])
    return freqs, H


def multifreq_profile(position, centers, normals, areas, e1, e2, *, gamma,
                      f0, bandwidth, c, twtt, window="hann", n_freq=128,
                      freeze_amplitudes=False):
    """Compressed profile at ``twtt`` for one position (multifreq.py:58-98),
    including the alias guard."""
    p = np.asarray(position, np.float64)
    twtt = np.asarray(twtt, np.float64)
    r = np.linalg.norm(p - np.asarray(centers, np.float64), axis=-1)
    tau = 2.0 * r / c
    span = max(twtt.max(), tau.max()) - min(twtt.min(), tau.min())
    if span > n_freq / bandwidth:
        raise ValueError("multifreq referee would alias")
    freqs, H = band_response(p, np.asarray(centers, np.float64),
                             np.asarray(normals, np.float64),
                             np.asarray(areas, np.float64),
                             np.asarray(e1, np.float64),
                             np.asarray(e2, np.float64), gamma=gamma, f0=f0,
                             bandwidth=bandwidth, cc=c, n_freq=n_freq,
                             freeze_amplitudes=freeze_amplitudes)
    w = window_weights(freqs, f0, bandwidth, window)
    wbar = w / w.sum()
    return (wbar * H) @ np.exp(2j * np.pi * np.outer(freqs - f0, twtt))


def synth_frozen(r, amp0, *, f0, bandwidth, c, twtt, n_freq, window="hann"):
    """Frozen-amplitude synthesis from per-facet ranges ``r`` and complex
    amplitudes ``amp0`` (the contribution at f0 with its carrier phase
    removed): y = sum_k Wbar_k sum_n amp0_n exp(-2j k_k r_n)
    exp(2j pi (f_k - f0) twtt) (multifreq.py:82-98 with any amplitude
    model, e.g. the rough-facet field)."""
    freqs = band_frequencies(f0, bandwidth, n_freq)
    w = window_weights(freqs, f0, bandwidth, window)
    wbar = w / w.sum()
    H = np.array([np.sum(amp0 * np.exp(-2j * (2.0 * np.pi * f / c) * r))
                  for f in freqs])
    return (wbar * H) @ np.exp(2j * np.pi * np.outer(freqs - f0,
                                                     np.asarray(twtt)))
