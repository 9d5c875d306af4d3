"""Incoherent (power-summing) facet sum in float32 (oracle).

Test infrastructure only: the GPU path never imports this module.

Restates soundersim ``kernels/incoherent.py``: per pair the power
(A cos)^2 / r^4 (:43), the two-way antenna weighting g^4 from the departure
direction (:44-46), the fast-time bin floor((2r/c - t0)/dt)
(``kernels/geometry.py:18-24``), drop-not-wrap into a per-trace scalar
(:47-53) and the left/right split by the sign of (c - p) . u_ct (:49-51).
Like the reference's traced program every quantity is float32: positions,
facets, t0, dt and c are rounded to float32 first (:86-99) and each
operation rounds to float32, in the reference's order, so the bins are the
reference's bins. Powers are accumulated in float64 here (the reference
sums float32 blocks); the power tolerance of the tests covers that.
"""

import numpy as np

from . import antenna

F32 = np.float32


def pair_terms(p, u, centers, normals, areas):
    """Range, power and side of every facet for one trace, float32.

    r = sqrt((dx^2 + dy^2) + dz^2) and cos = (d . n) / r with d = p - c
    (geometry.py:6-15); power (A cos)^2 / r^4 with r^4 formed as (r^2)^2
    (incoherent.py:43; XLA expands the integer power by squaring);
    right = ((c - p) . u > 0) (incoherent.py:50).
    """
    d = p[None, :] - centers
    r = np.sqrt((d[:, 0] * d[:, 0] + d[:, 1] * d[:, 1]) + d[:, 2] * d[:, 2])
    cos = ((d[:, 0] * normals[:, 0] + d[:, 1] * normals[:, 1])
           + d[:, 2] * normals[:, 2]) / r
    ac = areas * cos
    r2 = r * r
    pwr = (ac * ac) / (r2 * r2)
    a = -d
    right = ((a[:, 0] * u[0] + a[:, 1] * u[1]) + a[:, 2] * u[2]) > 0
    return d, r, pwr, right


def bins(r, t0, dt, c):
    """floor((2r/c - t0)/dt) in float32 (geometry.py:18-24), int64."""
    twtt = (F32(2.0) * r) / c
    return np.floor((twtt - t0) / dt).astype(np.int64)


def incoherent_cluttergram(positions, u_ct, centers, normals, areas, *, t0,
                           dt, n_samples, c, split_sides=False, pattern=None,
                           block_size=65536):
    """(power, dropped) as the reference returns them
    (incoherent.py:64-103): float32 (T, n_samples) or (T, n_samples, 2)
    [left, right], and float32 (T,). ``block_size`` only changes the
    reference's summation grouping, never the result."""
    del block_size
    pos = np.asarray(positions, F32)
    uct = np.asarray(u_ct, F32)
    cen = np.asarray(centers, F32)
    nrm = np.asarray(normals, F32)
    area = np.asarray(areas, F32)
    t0f, dtf, cf = F32(t0), F32(dt), F32(c)
    T = len(pos)
    n_seg = (2 if split_sides else 1) * n_samples
    hist = np.zeros((T, n_seg), np.float64)
    dropped = np.zeros(T, np.float64)
    if pattern is not None:
        kind, pv, pa, pb = pattern
        pv = np.asarray(pv, F32)
        pa = np.asarray(pa, F32)
        pb = np.asarray(pb, F32)
    for t in range(T):
        d, r, pwr, right = pair_terms(pos[t], uct[t], cen, nrm, area)
        pwr = pwr.astype(np.float64)
        if pattern is not None and kind != "isotropic":
            dhat = (-d) / r[:, None]
            g = antenna.gain(kind, dhat, pv[t], pa, pb)
            pwr = pwr * g ** 4
        b = bins(r, t0f, dtf, cf)
        ok = (b >= 0) & (b < n_samples)
        seg = b + (right.astype(np.int64) * n_samples if split_sides else 0)
        np.add.at(hist[t], seg[ok], pwr[ok])
        dropped[t] = pwr[~ok].sum()
    hist = hist.astype(F32)
    if split_sides:
        hist = hist.reshape(T, 2, n_samples).transpose(0, 2, 1)
    return hist, dropped.astype(F32)
