"""Refraction-point solvers in float64 (oracle).

Restates the two-point flat-interface Snell solve (soundersim
``refraction.py:78-161`` and its component-form twin
``kernels/multilayer.py:196-266``) and the joint N-interface damped-Newton
solve (``refraction_joint.py``: ``_chain_scan`` :131-140, ``_polyline``
:143-176, ``sequential_chain`` :179-193, ``_plane_basis`` :196-204, ``_inv2``
:207-215, ``_block_thomas`` :218-246, ``joint_crossings`` :249-322).

Arrays carry points as (..., 3); every 3-dot sums as (x + y) + z.
"""

from typing import NamedTuple

import numpy as np

EPS64 = np.finfo(np.float64).eps
TINY = 1e-30


def dot3(a, b):
    return (a[..., 0] * b[..., 0] + a[..., 1] * b[..., 1]) + a[..., 2] * b[..., 2]


class Crossing(NamedTuple):
    x: np.ndarray
    theta1: np.ndarray
    theta2: np.ndarray
    s1: np.ndarray
    s2: np.ndarray
    residual: np.ndarray
    valid: np.ndarray


def snell(p, q, o, nrm, n1, n2, n_iter, *, component=True, tol=1e-9):
    """Two-point refraction crossing on the plane (o, nrm) for p (index n1)
    to q (index n2): safeguarded Newton on sigma = sin(theta_rare) with a
    fixed iteration budget, lengths scaled by a + b + L.

    ``component=True`` follows the multilayer kernel's operation order
    (multilayer.py:196-266: one reciprocal of s, rsqrt products);
    ``component=False`` follows refraction.py:78-161 (divisions), used by the
    joint solver's sequential initialiser."""
    with np.errstate(invalid="ignore", divide="ignore", over="ignore"):
        h1 = dot3(p - o, nrm)
        h2 = dot3(q - o, nrm)
        a, b = np.abs(h1), np.abs(h2)
        fp = p - h1[..., None] * nrm
        fq = q - h2[..., None] * nrm
        w = fq - fp
        L = np.sqrt(dot3(w, w))
        u = w / np.maximum(L, TINY)[..., None]
        s = np.maximum(a + b + L, TINY)
        if component:
            inv_s = 1.0 / s
            ah, bh, Lh = a * inv_s, b * inv_s, L * inv_s
        else:
            ah, bh, Lh = a / s, b / s, L / s
        swap = n1 > n2
        ratio = min(n1, n2) / max(n1, n2)
        ar = np.where(swap, bh, ah)
        bd = np.where(swap, ah, bh)
        hi0 = 1.0 - 8.0 * EPS64
        sig = np.minimum(Lh / np.maximum(np.sqrt(Lh * Lh + (ah + bh) ** 2),
                                         TINY), hi0)
        lo = np.zeros_like(Lh)
        hi = hi0 * np.ones_like(Lh)
        for _ in range(n_iter):
            v = ratio * sig
            c1 = np.maximum((1.0 - sig) * (1.0 + sig), TINY)
            c2 = np.maximum((1.0 - v) * (1.0 + v), TINY)
            if component:
                F = ar * sig * (1.0 / np.sqrt(c1)) + bd * v * (
                    1.0 / np.sqrt(c2)) - Lh
            else:
                F = ar * sig / np.sqrt(c1) + bd * v / np.sqrt(c2) - Lh
            neg = F <= 0
            lo = np.where(neg, sig, lo)
            hi = np.where(neg, hi, sig)
            if component:
                Fp = ar / (c1 * np.sqrt(c1)) + (bd * ratio) / (c2 * np.sqrt(c2))
            else:
                Fp = (ar / (c1 * np.sqrt(c1))
                      + bd * ratio / (c2 * np.sqrt(c2)))
            sn = sig - F / np.maximum(Fp, TINY)
            ok = (sn >= lo) & (sn <= hi) & np.isfinite(sn)
            sig = np.where(ok, sn, 0.5 * (lo + hi))
        c1 = np.maximum((1.0 - sig) * (1.0 + sig), TINY)
        if component:
            tr = ar * sig * (1.0 / np.sqrt(c1))
        else:
            tr = ar * sig / np.sqrt(c1)
        t = np.clip(np.where(swap, Lh - tr, tr), 0.0, Lh)
        d2 = Lh - t
        r1 = np.maximum(np.sqrt(ah * ah + t * t), TINY)
        r2 = np.maximum(np.sqrt(bh * bh + d2 * d2), TINY)
        residual = n1 * t / r1 - n2 * d2 / r2
        x = fp + (s * t)[..., None] * u
        th1 = np.arctan2(t, ah)
        th2 = np.arctan2(d2, bh)
        valid = (h1 * h2 < 0) & (np.abs(residual) <= tol)
    return Crossing(x, th1, th2, s * r1, s * r2, residual, valid)


class Joint(NamedTuple):
    x: np.ndarray         # (N, M, 3)
    theta1: np.ndarray    # (N, M)
    theta2: np.ndarray    # (N, M)
    s: np.ndarray         # (N+1, M)
    residual: np.ndarray  # (M,)
    converged: np.ndarray
    valid: np.ndarray


def chain(p, q, o, nrm, n_media, n_iter):
    """Sequential two-point chain over the interface axis (refraction_joint
    :131-140); o/nrm (N, M, 3), n_media (N+1,). Returns crossings and
    all-valid."""
    cur = np.broadcast_to(p, q.shape)
    xs, ok = [], np.ones(q.shape[:-1], bool)
    for i in range(o.shape[0]):
        r = snell(cur, q, o[i], nrm[i], n_media[i], n_media[i + 1], n_iter,
                  component=False)
        xs.append(r.x)
        ok &= r.valid
        cur = r.x
    return np.stack(xs), ok


def polyline(x, p, q, nrm, n_media, tol, converged=None):
    """Honest geometry of p -> x_0..x_{N-1} -> q (refraction_joint:143-176)."""
    with np.errstate(invalid="ignore", divide="ignore", over="ignore"):
        m = q.shape[:-1]
        P = np.concatenate([np.broadcast_to(p, q.shape)[None], x, q[None]], 0)
        d = P[1:] - P[:-1]
        s = np.sqrt(dot3(d, d))
        dh = d / np.maximum(s, TINY)[..., None]
        din, dout = dh[:-1], dh[1:]
        ct1 = dot3(nrm, din)
        ct2 = dot3(nrm, dout)
        t1 = din - ct1[..., None] * nrm
        t2 = dout - ct2[..., None] * nrm
        st1 = np.sqrt(dot3(t1, t1))
        st2 = np.sqrt(dot3(t2, t2))
        th1 = np.arctan2(st1, np.abs(ct1))
        th2 = np.arctan2(st2, np.abs(ct2))
        nm = np.asarray(n_media, np.float64).reshape((-1,) + (1,) * len(m))
        dG = nm[:-1, ..., None] * din - nm[1:, ..., None] * dout
        rt = dG - dot3(nrm, dG)[..., None] * nrm
        residual = np.max(np.sqrt(dot3(rt, rt)), axis=0)
        hp = dot3(nrm, P[:-2] - x)
        hn = dot3(nrm, P[2:] - x)
        sides = np.all(hp * hn < 0, axis=0)
        evan = np.any(nm[:-1] * st1 > nm[1:] * (1.0 + 64.0 * EPS64), axis=0)
        fin = (np.all(np.isfinite(x), axis=(0, -1)) & np.isfinite(residual)
               & np.all(np.isfinite(s), axis=0))
        if converged is None:
            converged = (residual <= tol) & fin
        valid = converged & sides & ~evan & fin
    return Joint(x, th1, th2, s, residual, converged, valid)


def sequential_chain(p, q, o, nrm, n_media, n_iter=25):
    """refraction_joint.sequential_chain (:179-193)."""
    x, ok = chain(p, q, o, nrm, n_media, n_iter)
    return polyline(x, p, q, nrm, n_media, None, converged=ok)


def plane_basis(nrm):
    """Orthonormal in-plane basis (..., 3, 2) (refraction_joint:196-204)."""
    ref = np.zeros_like(nrm)
    use_z = np.abs(nrm[..., 2]) < 0.9
    ref[..., 2] = np.where(use_z, 1.0, 0.0)
    ref[..., 0] = np.where(use_z, 0.0, 1.0)
    u = np.cross(ref, nrm)
    u = u / np.maximum(np.sqrt(dot3(u, u)), TINY)[..., None]
    return np.stack([u, np.cross(nrm, u)], axis=-1)


def inv2(m):
    """2x2 inverse with |det| clamped to >= 1e-30 (refraction_joint:207-215)."""
    a, b = m[..., 0, 0], m[..., 0, 1]
    c, d = m[..., 1, 0], m[..., 1, 1]
    det = a * d - b * c
    det = np.where(np.abs(det) < TINY, TINY, det)
    out = np.empty_like(m)
    out[..., 0, 0] = d / det
    out[..., 0, 1] = -b / det
    out[..., 1, 0] = -c / det
    out[..., 1, 1] = a / det
    return out


def block_thomas(A, C, rhs):
    """Symmetric block-tridiagonal solve (refraction_joint:218-246): diag
    A_i, upper C_i, lower C_i^T; forward elimination then back
    substitution."""
    n = A.shape[0]
    dinv = np.empty_like(A)
    y = np.empty_like(rhs)
    dinv_prev = np.zeros_like(A[0])
    y_prev = np.zeros_like(rhs[0])
    for i in range(n):
        cp = C[i - 1] if i > 0 else np.zeros_like(A[0])
        cpt = np.swapaxes(cp, -1, -2) @ dinv_prev
        dinv[i] = inv2(A[i] - cpt @ cp)
        y[i] = rhs[i] - np.einsum("...ij,...j->...i", cpt, y_prev)
        dinv_prev, y_prev = dinv[i], y[i]
    out = np.empty_like(rhs)
    d_next = np.zeros_like(rhs[0])
    for i in range(n - 1, -1, -1):
        cn = C[i] if i < n - 1 else np.zeros_like(A[0])
        r = y[i] - np.einsum("...ij,...j->...i", cn, d_next)
        out[i] = np.einsum("...ij,...j->...i", dinv[i], r)
        d_next = out[i]
    return out


def joint_crossings(p, q, o, nrm, n_media, *, n_newton=20, n_backtrack=10,
                    n_iter_init=25, tol=1e-9):
    """Joint stationary path through N local planes
    (refraction_joint:249-322): chain initialiser, scale by |p - q|, 2-D
    in-plane offsets, damped Newton with block-Thomas steps, step halving on
    |F|^2, Levenberg shift eps^0.75."""
    nm = np.asarray(n_media, np.float64)
    q = np.asarray(q, np.float64)
    bshape = q.shape[:-1]
    nmb = nm.reshape((-1,) + (1,) * len(bshape))
    with np.errstate(invalid="ignore", divide="ignore", over="ignore"):
        x0, _ = chain(p, q, o, nrm, nm, n_iter_init)
        pq = np.broadcast_to(p, q.shape) - q
        scale = np.maximum(np.sqrt(dot3(pq, pq)), TINY)
        inv = (1.0 / scale)[..., None]
        ps = np.broadcast_to(p, q.shape) * inv
        qs = q * inv
        os_ = o * inv
        basis = plane_basis(nrm)                      # (N, M, 3, 2)
        ab = np.einsum("...kj,...k->...j", basis, x0 * inv - os_)
        lam = 2.0 ** (-np.arange(n_backtrack, dtype=np.float64))
        mu = EPS64 ** 0.75
        eye2, eye3 = np.eye(2), np.eye(3)

        def geom(ab_):
            x = os_ + np.einsum("...kj,...j->...k", basis, ab_)
            pl = np.concatenate([ps[None], x, qs[None]], 0)
            d = pl[1:] - pl[:-1]
            s = np.maximum(np.sqrt(dot3(d, d)), TINY)
            dh = d / s[..., None]
            g = nmb[..., None] * dh
            f = np.einsum("...kj,...k->...j", basis, g[:-1] - g[1:])
            return x, s, dh, f

        for _ in range(n_newton):
            _, s, dh, f = geom(ab)
            w = (nmb / s)[..., None, None] * (
                eye3 - dh[..., :, None] * dh[..., None, :])
            A = (np.einsum("...ki,...kl,...lj->...ij", basis, w[:-1] + w[1:],
                           basis) + mu * eye2)
            Cm = -np.einsum("...ki,...kl,...lj->...ij", basis[:-1], w[1:-1],
                            basis[1:])
            delta = block_thomas(A, Cm, -f)
            m0 = np.sum(f * f, axis=(0, -1))
            lam_sel = np.zeros(bshape)
            done = np.zeros(bshape, bool)
            for lj in lam:
                mc = np.sum(geom(ab + lj * delta)[3] ** 2, axis=(0, -1))
                take = (~done) & (mc < m0)
                lam_sel = np.where(take, lj, lam_sel)
                done |= take
            ab = ab + lam_sel[None, ..., None] * delta
        x = geom(ab)[0] * scale[..., None]
    return polyline(x, p, q, nrm, nm, tol)
