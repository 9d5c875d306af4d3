"""Straight-track time-domain backprojection (focused SAR) in float64
(oracle).

Test infrastructure only: the GPU path never imports this module.

Restates soundersim ``processing.py:262-348`` (``focused_sar``) on plain
arrays: along-track arc length s (``_along_track`` :65-69), the aperture
{j : |s_j - s_i| <= L/2} per output trace, the range-migration delay
dr = sqrt(r0^2 + d^2) - r0 with r0 = c twtt / 2, linear complex
interpolation of trace j at (twtt + 2 dr / c - t0) / dt with samples whose
lower index falls outside [0, nb - 2] dropped, the carrier correction
exp(+2j k dr) and the hann or rectangular aperture weight; plus the lambda/4
Doppler guard (:241-259).
"""

import numpy as np

C_DEFAULT = 299792458.0


def along_track(pos):
    """Cumulative arc length, s[0] = 0 (processing.py:65-69)."""
    pos = np.asarray(pos, np.float64)
    seg = np.linalg.norm(np.diff(pos, axis=0), axis=1)
    return np.concatenate([[0.0], np.cumsum(seg)])


def mean_spacing(pos):
    pos = np.asarray(pos, np.float64)
    if pos.shape[0] < 2:
        return 0.0
    return float(np.linalg.norm(np.diff(pos, axis=0), axis=1).mean())


def doppler_guard(spacing, wavelength, aperture_m, r_ref):
    """True when the spacing exceeds lambda / (4 sin theta_max)
    (processing.py:241-259)."""
    if r_ref <= 0:
        return False
    st = np.sin(np.arctan((aperture_m / 2.0) / r_ref))
    if st <= 0:
        return False
    return spacing > wavelength / (4.0 * st)


def window_weight(window, d, half):
    if window == "hann":
        return 0.5 * (1.0 + np.cos(np.pi * d / half))
    if window in ("none", "rect", None):
        return np.ones_like(d)
    raise ValueError(f"unknown window {window!r} (use 'hann' or 'none')")


def focused_sar(field, twtt, pos, wavelength, aperture_m, window="hann",
                c=C_DEFAULT):
    """(out complex128 (T, nb), power float32) as processing.py:301-340
    computes them."""
    k = 2.0 * np.pi / wavelength
    twtt = np.asarray(twtt, np.float64)
    dt = float(twtt[1] - twtt[0])
    t0 = float(twtt[0])
    nb = twtt.size
    r0 = c * twtt / 2.0
    s = along_track(pos)
    F = np.asarray(field).astype(np.complex128)
    T = F.shape[0]
    half = aperture_m / 2.0
    window_weight(window, np.zeros(1), half)  # validates the name
    out = np.zeros((T, nb), np.complex128)
    for i in range(T):
        d = s - s[i]
        J = np.nonzero(np.abs(d) <= half)[0]
        if J.size == 0:
            continue
        dJ = d[J][:, None]
        dr = np.sqrt(r0[None, :] ** 2 + dJ ** 2) - r0[None, :]
        x = ((twtt[None, :] + 2.0 * dr / c) - t0) / dt
        i0 = np.floor(x).astype(np.int64)
        frac = x - i0
        valid = (i0 >= 0) & (i0 < nb - 1)
        i0c = np.clip(i0, 0, nb - 2)
        rows = J[:, None]
        samp = F[rows, i0c] * (1.0 - frac) + F[rows, i0c + 1] * frac
        samp = np.where(valid, samp, 0.0)
        w = window_weight(window, d[J], half)[:, None]
        out[i] = np.sum(w * samp * np.exp(2j * k * dr), axis=0)
    return out, np.abs(out).astype(np.float32) ** 2
