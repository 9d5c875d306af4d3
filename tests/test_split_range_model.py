"""Float32 model of the surface split kernel's per-trace range difference.

The kernel (ss_coherent_split.cu) forms the range r_c to a trace block's
middle platform p_c once per facet as a double-float, then for a trace at
w = p_t - p_c adds dr = r_t - r_c = N / (2 r_c + dr) with N = 2 q.w + |w|^2
(q = p_c - c): w = lam u + eps along the block's track direction u, q.u a
double-float once per facet, N = 2 (lam q.u + q.eps) + |w|^2 with one
exact product per pair, the quotient in float32 with one correction
against the double-float denominator. Its bin position is then good to ~2e-7 bins, inside the 2e-6
band that sends a pair to the exact re-bin. This model repeats the
kernel's lines in NumPy float32 (exact products emulated in float64, where
a product of two floats is exact) on surface facets of the roughness
configuration, for offsets up to the kernel's 160 m single-reference
limit, and checks dr and the incidence cosine against float64.
"""

import numpy as np
import pytest

F32 = np.float32


def two_prod(a, b):
    p = (a * b).astype(F32)
    e = (a.astype(np.float64) * b.astype(np.float64) - p).astype(F32)
    return p, e


def two_sum(a, b):
    s = (a + b).astype(F32)
    bb = (s - a).astype(F32)
    e = ((a - (s - bb)) + (b - bb)).astype(F32)
    return s, e


def fma(a, b, c):
    return (np.float64(a) * np.float64(b) + np.float64(c)).astype(F32)


@pytest.fixture(scope="module")
def pairs():
    from radar_sounder_simulator_gb300 import scenes
    cfg = scenes.config3(n_cells=256, n_traces=512)
    s = cfg.surface
    c = s.centers.astype(np.float32).astype(np.float64)
    n = s.normals.astype(np.float32).astype(np.float64)
    pc = cfg.pos[len(cfg.pos) // 2]
    rng = np.random.default_rng(7)
    idx = rng.choice(len(c), 20000, replace=False)
    return pc, c[idx], n[idx]


def _model(pc, w, C, Nn):
    q = pc - C
    qh = q.astype(F32)
    ql = (q - qh).astype(F32)
    rc = np.linalg.norm(q, axis=1)
    rch = rc.astype(F32)
    rcl = (rc - rch).astype(F32)
    wh = w.astype(F32)
    wl = (w - wh).astype(F32)
    w2 = float(np.dot(w, w))
    w2h = F32(w2)
    w2l = F32(w2 - float(w2h))
    # w = lam u + eps along the block's track direction u (x here)
    u = np.array([1.0, 0.0, 0.0])
    lam = float(np.dot(w, u))
    eps = (w - lam * u).astype(F32)
    lh = F32(lam)
    ll = F32(lam - float(lh))
    uh = u.astype(F32)
    ul = (u - uh).astype(F32)
    # q.u as a double-float once per facet
    p = [two_prod(qh[:, j], np.full(len(q), uh[j], F32)) for j in range(3)]
    s1, f1 = two_sum(p[0][0], p[1][0])
    s2, f2 = two_sum(s1, p[2][0])
    qul = ((f1 + f2) + (p[0][1] + p[1][1] + p[2][1]) +
           (ql * uh).sum(1, dtype=F32) + (qh * ul).sum(1, dtype=F32))
    quh = (s2 + qul).astype(F32)
    qul = (qul - (quh - s2)).astype(F32)
    # per pair: one exact product, the lo parts and q.eps in float
    pq, eq = two_prod(np.full(len(q), lh, F32), quh)
    lo = (eq + fma(lh, qul, ll * quh) + (qh * eps).sum(1, dtype=F32)
          ).astype(F32)
    Nh, g = two_sum((F32(2) * pq).astype(F32), fma(F32(2), lo, w2h))
    Nl = (g + w2l).astype(F32)
    rr = fma(rch, rch, Nh)
    inv = (F32(1) / np.sqrt(rr)).astype(F32)
    dr0 = (Nh / (rch + rr * inv)).astype(F32)
    Dh, De = two_sum((F32(2) * rch).astype(F32), dr0)
    Dl = fma(F32(2), rcl, De)
    iD = (F32(1) / Dh).astype(F32)
    dr = (Nh * iD).astype(F32)
    drl = ((fma(-dr, Dh, Nh) + fma(-dr, Dl, Nl)) * iD).astype(F32)
    # cosine: exact q.n / r_c once per facet, moved to the trace
    cosc = (np.sum(q * Nn, 1) / rc).astype(F32)
    nw = (Nn.astype(F32) * wh).sum(1, dtype=F32)
    cosv = ((nw - cosc * dr) * inv + cosc).astype(F32)
    return rc, dr.astype(np.float64) + drl.astype(np.float64), cosv


@pytest.mark.parametrize("wx", [6.25, 25.0, 75.0, 160.0])
def test_range_difference_is_exact_to_the_bin_band(pairs, wx):
    """Straight block (eps = 0): dr to 1e-8 m (measured 7e-12 m at 6.25 m,
    2.3e-9 m at 160 m). Bent blocks, eps up to the kernel's 1 m limit:
    q.eps is a float32 product, 1e-7 m at 1 m (2e-6 rad at 450 MHz, 1e-7
    bins: far inside the 2e-6-bin band)."""
    pc, C, Nn = pairs
    for w, bound in ((np.array([wx, 0.0, 0.0]), 1e-8),
                     (np.array([-wx, 0.3, -0.2]), 1e-7),
                     (np.array([wx, 0.7, 0.7]), 2e-7)):
        rc, dr, cosv = _model(pc, w, C, Nn)
        exact = np.linalg.norm(pc + w - C, axis=1)
        err = np.abs(rc + dr - exact)
        assert err.max() <= bound, (w, err.max())
        cos = np.sum((pc + w - C) * Nn, 1) / exact
        assert np.abs(cosv - cos).max() <= 1e-6
        assert np.sqrt(np.mean(((cosv - cos) / cos) ** 2)) <= 1e-7
