"""Surface coherent LPA facet sum in float64 (oracle).

Restates soundersim ``kernels/coherent.py``: the per-pair linear-phase-
approximation field (``lpa_contributions`` :107-128), its rough-facet form
(``rough_lpa_contributions`` :131-168), the off-specular taper (:94-104),
the in-kernel antenna weighting (:216-218), binning with drop-not-wrap,
sub-bin interpolation and side split (:219-236), and the host-side culling
and argument conventions of ``coherent_cluttergram`` (:247-362).
"""

import numpy as np

from . import antenna, roughness
from .geometry import culling_plan, twtt_bin

TWO_PI = 2.0 * np.pi


def taper(cos, s_eff):
    """exp(-tan^2(alpha) / (2 s_eff^2)) with cos clamped to [1e-9, 1]
    (coherent.py:94-104)."""
    cc = np.clip(cos, 1e-9, 1.0)
    c2 = cc * cc
    return np.exp(-(1.0 - c2) / (c2 * (2.0 * s_eff * s_eff)))


def _sinc(x):
    """sin(x)/x via the normalised np.sinc, as the reference calls it."""
    return np.sinc(x / np.pi)


def pair_geometry(p, c, nrm):
    """Range, incidence cosine and unit vector facet -> platform."""
    d = p - c
    r = np.sqrt((d[..., 0] * d[..., 0] + d[..., 1] * d[..., 1])
                + d[..., 2] * d[..., 2])
    cos = ((d[..., 0] * nrm[..., 0] + d[..., 1] * nrm[..., 1])
           + d[..., 2] * nrm[..., 2]) / r
    return d, r, cos, d / r[..., None]


def _dot(a, b):
    return (a[..., 0] * b[..., 0] + a[..., 1] * b[..., 1]) + a[..., 2] * b[..., 2]


def lpa_field(p, c, nrm, area, e1, e2, k, gamma, taper_s=None):
    """j (k/2pi) gamma cos A sinc(k rhat.e1) sinc(k rhat.e2) e^{-2jkr} / r^2
    and r (coherent.py:107-128, absolute phase)."""
    _, r, cos, rhat = pair_geometry(p, c, nrm)
    s1 = np.sinc(_dot(rhat, e1) * (k / np.pi))
    s2 = np.sinc(_dot(rhat, e2) * (k / np.pi))
    amp = (k / TWO_PI) * gamma * cos * area * s1 * s2 / (r * r)
    if taper_s is not None:
        amp = amp * taper(cos, taper_s)
    return 1j * amp * np.exp(1j * ((-2.0 * k) * r)), r


def rough_lpa_field(p, c, nrm, area, e1, e2, k, gamma, sigma, l, phasors,
                    n_terms, taper_s=None, area_only=False, acf="gaussian"):
    """Smooth term x exp(-sigma^2 K^2/2) + incoherent sqrt(D_Phi) phi_r term
    with the same non-phase factor (coherent.py:131-168)."""
    _, r, cos, rhat = pair_geometry(p, c, nrm)
    d1 = _dot(rhat, e1)
    d2 = _dot(rhat, e2)
    s1 = np.sinc(d1 * (k / np.pi))
    s2 = np.sinc(d2 * (k / np.pi))
    amp = (k / TWO_PI) * gamma * cos * area * s1 * s2 / (r * r)
    if taper_s is not None:
        amp = amp * taper(cos, taper_s)
    l1 = np.sqrt(_dot(e1, e1))
    l2 = np.sqrt(_dot(e2, e2))
    kk = 2.0 * k * cos
    with np.errstate(invalid="ignore", divide="ignore"):
        dp = roughness.d_phi(sigma, l, kk, 2.0 * k * d1 / l1,
                             2.0 * k * d2 / l2, l1, l2, n_terms=n_terms,
                             area_only=area_only, acf=acf)
        amp_i = np.where(area > 0,
                         (k / TWO_PI) * gamma * cos / (r * r) * np.sqrt(dp),
                         0.0)
    contrib = amp * roughness.mean_attenuation(sigma, kk) + amp_i * phasors
    return 1j * contrib * np.exp(1j * ((-2.0 * k) * r)), r


def _bin_into(hist, drop, t, contrib, twtt, t0, dt, n_samples, interp,
              right):
    """Drop-not-wrap binning of one trace's contributions
    (coherent.py:219-236). Returns the dropped power."""
    b = twtt_bin(twtt, t0, dt)
    if interp:
        w = (twtt - t0) / dt - b.astype(np.float64)
        parts = ((contrib * (1.0 - w), b), (contrib * w, b + 1))
    else:
        parts = ((contrib, b),)
    for part, pb in parts:
        ok = (pb >= 0) & (pb < n_samples)
        seg = pb + (right * n_samples if right is not None else 0)
        np.add.at(hist[t], seg[ok], part[ok])
        drop[t] += float(np.sum(np.abs(part[~ok]) ** 2))


def coherent_cluttergram(positions, u_ct, centers, normals, areas, e1, e2, *,
                         k, gamma, t0, dt, n_samples, c, split_sides=False,
                         interp_bins=False, pattern=None, roughness=None,
                         taper_s=None, d_phi_area=False, block_size=None,
                         window_cull=True):
    """Float64 binned coherent field (coherent.py:247-362 conventions).

    Returns (field complex128 (T, n) or (T, n, 2), dropped float64 (T,)).
    ``roughness`` is ``(sigma, l, phasors, n_terms[, acf])``; sigma and l may
    also be per-facet (N,) arrays (extension used by the roughness configs).
    """
    pos = np.asarray(positions, np.float64)
    uct = np.asarray(u_ct, np.float64)
    n = len(centers)
    order, bs, n_blocks, off, n_win = culling_plan(
        pos, centers, t0=t0, dt=dt, n_samples=n_samples, c=c,
        block_size=block_size, target_pairs=1 << 19, window_cull=window_cull)

    def fq(a):  # float32-quantised facet data, sorted, as float64
        return np.asarray(a, np.float32)[order].astype(np.float64)

    cf, nf, af, f1, f2 = (fq(centers), fq(normals), fq(areas), fq(e1),
                          fq(e2))
    gamma_arr = np.asarray(gamma)
    if gamma_arr.ndim > 0:
        if gamma_arr.shape != (n,):
            raise ValueError(f"per-facet gamma shape {gamma_arr.shape} != "
                             f"({n},)")
        gam = fq(gamma_arr)
    else:
        gam = None
    rough = None
    if roughness is not None:
        sig, lc, ph, n_terms, *rest = roughness
        acf = rest[0] if rest else "gaussian"
        if acf == "exponential" and not d_phi_area:
            raise ValueError("roughness acf='exponential' requires the "
                             "area-only D_Phi (d_phi_area / grazing fix)")
        sig = fq(sig) if np.ndim(sig) else float(sig)
        lc = fq(lc) if np.ndim(lc) else float(lc)
        ph = np.asarray(ph, np.complex64)[order].astype(np.complex128)
        rough = (sig, lc, ph, int(n_terms), acf)
    kind, pv, pa, pb = pattern or ("isotropic", np.zeros((len(pos), 3)), 0.0,
                                   0.0)
    pv = np.asarray(pv, np.float64)
    n_seg = (2 if split_sides else 1) * n_samples
    hist = np.zeros((len(pos), n_seg), np.complex128)
    drop = np.zeros(len(pos), np.float64)
    for t in range(len(pos)):
        sl = slice(int(off[t]) * bs, min((int(off[t]) + n_win) * bs, n))
        p = pos[t]
        g_t = gamma if gam is None else gam[sl]
        if rough is None:
            contrib, r = lpa_field(p, cf[sl], nf[sl], af[sl], f1[sl], f2[sl],
                                   k, g_t, taper_s)
        else:
            sig, lc, ph, n_terms, acf = rough
            contrib, r = rough_lpa_field(
                p, cf[sl], nf[sl], af[sl], f1[sl], f2[sl], k, g_t,
                sig if np.ndim(sig) == 0 else sig[sl],
                lc if np.ndim(lc) == 0 else lc[sl], ph[sl], n_terms,
                taper_s=taper_s, area_only=d_phi_area, acf=acf)
        if kind != "isotropic":
            g = antenna.gain(kind, (cf[sl] - p) / r[:, None], pv[t], pa, pb)
            contrib = contrib * (g * g)
        right = None
        if split_sides:
            right = (_dot(cf[sl] - p, uct[t]) > 0).astype(np.int64)
        _bin_into(hist, drop, t, contrib, 2.0 * r / c, t0, dt, n_samples,
                  interp_bins, right)
    if split_sides:
        hist = hist.reshape(-1, 2, n_samples).transpose(0, 2, 1)
    return hist, drop
