"""One-way antenna field gains evaluated per pair (float64 oracle).

Restates soundersim ``antenna.py:204-258`` (``gain_fn``) for one trace:
``dhat`` (..., 3) departure directions antenna -> facet, ``pv`` that trace's
pattern vector ((3,) or (2, 3) for arrays), ``pa``/``pb`` the kind's
parameters as ``antenna.pattern_args`` packs them.
"""

import numpy as np


def element_field(cos_b, q, enabled):
    """Forward-hemisphere cos^(q/2) element field (antenna.py:138-143)."""
    c = np.clip(cos_b, 0.0, 1.0)
    fwd = np.where(cos_b >= 0.0, c ** (q / 2.0), 0.0)
    return fwd if enabled else np.ones_like(c)


def gain(kind, dhat, pv, pa, pb):
    """g(dhat) for one trace (antenna.py:204-258)."""
    d = np.asarray(dhat, np.float64)
    pv = np.asarray(pv, np.float64)
    if kind == "isotropic":
        return np.ones(d.shape[:-1])
    if kind == "dipole":
        ca = d @ pv
        s = np.sqrt(np.maximum(1.0 - ca * ca, 1e-12))
        return np.cos((np.pi / 2.0) * ca) / s
    if kind == "array":
        n = float(np.asarray(pa))
        pb = np.asarray(pb, np.float64)
        x = np.pi * pb[0] * (d @ pv[0])
        sx = np.sin(x)
        near = np.abs(sx) < 1e-5
        with np.errstate(divide="ignore", invalid="ignore"):
            af = np.where(near, np.cos(n * x) / np.cos(x),
                          np.sin(n * x) / (n * np.where(near, 1.0, sx)))
        ef = element_field(d @ pv[1], pb[2], bool(pb[3]))
        return pb[1] * ef * np.abs(af)
    if kind == "array_tapered":
        pa = np.asarray(pa, np.float64)
        pb = np.asarray(pb, np.float64)
        n = pa.shape[1]
        m = np.arange(n) - (n - 1) / 2.0
        ph = (2.0 * np.pi * pb[0]) * (d @ pv[0])[..., None] * m
        cs, sn = np.cos(ph), np.sin(ph)

        def af(w):
            return np.sqrt((cs @ w) ** 2 + (sn @ w) ** 2) / np.sum(w)

        ef = element_field(d @ pv[1], pb[2], bool(pb[3]))
        return pb[1] * ef * np.sqrt(af(pa[0]) * af(pa[1]))
    if kind == "finite_dipole":
        kh = np.pi * float(np.asarray(pa))
        ca = d @ pv
        s = np.sqrt(np.maximum(1.0 - ca * ca, 1e-12))
        return np.abs(np.cos(kh * ca) - np.cos(kh)) / (s * (1.0 - np.cos(kh)))
    if kind == "tabulated":
        ct = np.clip(d @ pv, -1.0, 1.0)
        return np.interp(np.arccos(ct), np.asarray(pa, np.float64),
                         np.asarray(pb, np.float64))
    raise ValueError(f"unknown pattern kind {kind!r}")
