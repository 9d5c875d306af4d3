"""Refracted multilayer cluttergram in float64 (oracle).

Restates soundersim ``kernels/multilayer.py``: lookup constants
(``_grid_consts`` :269-283, ``_joint_consts`` :286-330), the sequential
chained path (``path`` :352-406), the joint path (``path_joint`` :408-457),
the per-pair radiometry and binning (``one_trace``/``step`` :459-588) and the
host conventions of ``refracted_cluttergram`` (:594-770). Physics helpers:
``fresnel_te`` (physics.py:33-67), spreading (physics.py:109-150).
"""

import numpy as np

from . import antenna
from . import roughness as rough_model
from .geometry import culling_plan, twtt_bin
from .refraction import dot3, joint_crossings, sequential_chain, snell

TWO_PI = 2.0 * np.pi
C_MIN = 1e-9


def fresnel_te_gamma(eps1, eps2, cos1):
    """TE field reflection coefficient (physics.py:33-67)."""
    n1, n2 = np.sqrt(eps1), np.sqrt(eps2)
    sin2_sq = (eps1 / eps2) * (1.0 - cos1 * cos1)
    cos2 = np.sqrt(np.maximum(1.0 - sin2_sq, 0.0))
    return (n1 * cos1 - n2 * cos2) / (n1 * cos1 + n2 * cos2)


def grid_consts(f):
    """(float32 centre grid, float32 normal grid, affine (x, y, 1) -> (row,
    col) least-squares fit, area-weighted mean point, unit mean normal)
    (multilayer.py:269-283)."""
    ny, nx = f.grid_shape
    gc = np.asarray(f.centers).reshape(ny, nx, 3).astype(np.float32)
    gn = np.asarray(f.normals).reshape(ny, nx, 3).astype(np.float32)
    a = np.column_stack([f.centers[:, 0], f.centers[:, 1],
                         np.ones(len(f.centers))])
    coef = np.linalg.lstsq(a, np.asarray(f.cell, np.float64), rcond=None)[0]
    w = (f.areas / f.areas.sum())[:, None]
    mp = (f.centers * w).sum(0)
    mn = (f.normals * w).sum(0)
    return gc, gn, coef, mp, mn / np.linalg.norm(mn)


def joint_consts(crossed, pad_to, z_platform):
    """Stacked lookup constants padded at the top with index-matched no-op
    planes in the air gap (multilayer.py:286-330)."""
    per = [grid_consts(f) for f in crossed]
    k = pad_to - len(crossed)
    if k < 0:
        raise ValueError(f"pad_to={pad_to} < {len(crossed)} crossed "
                         "interfaces")
    ny = max(g[0].shape[0] for g in per)
    nx = max(g[0].shape[1] for g in per)
    gc = np.zeros((pad_to, ny, nx, 3), np.float32)
    gn = np.zeros((pad_to, ny, nx, 3), np.float32)
    gn[..., 2] = 1.0
    coef = np.zeros((pad_to, 3, 2))
    shp = np.ones((pad_to, 2), np.int32)
    mp = np.zeros((pad_to, 3))
    mn = np.zeros((pad_to, 3))
    mn[:, 2] = 1.0
    if k:
        z_surf = float(crossed[0].centers[:, 2].max())
        gap = float(z_platform) - z_surf
        if gap <= 0:
            raise ValueError("joint refraction padding needs the platform "
                             f"above the surface (gap {gap:.1f} m)")
        zs = z_surf + gap * (np.arange(k, 0, -1) / (k + 1.0))
        gc[:k, :, :, 2] = zs[:, None, None]
        mp[:k, 2] = zs
    for i, (c, n, cf, p0, n0) in enumerate(per):
        j = k + i
        gc[j, :c.shape[0], :c.shape[1]] = c
        gn[j, :n.shape[0], :n.shape[1]] = n
        coef[j], shp[j], mp[j], mn[j] = cf, c.shape[:2], p0, n0
    return gc, gn, coef, shp, mp, mn, k


def _lookup(gc, gn, coef, rows_max, cols_max, x):
    """Nearest-facet local plane from an affine index fit: round, clip,
    gather, renormalise (multilayer.py:377-386 / :422-431)."""
    rc0 = x[..., 0] * coef[0, 0] + x[..., 1] * coef[1, 0] + coef[2, 0]
    rc1 = x[..., 0] * coef[0, 1] + x[..., 1] * coef[1, 1] + coef[2, 1]
    row = np.clip(np.round(rc0), 0, rows_max - 1).astype(np.int32)
    col = np.clip(np.round(rc1), 0, cols_max - 1).astype(np.int32)
    pt = gc[row, col].astype(np.float64)
    nr = gn[row, col].astype(np.float64)
    return pt, nr, row, col


def path_sequential(p, q, consts, n_leg, eps_leg, att, k0, sig_c):
    """Chained two-point solves top-down (multilayer.py:352-406)."""
    m = q.shape[0]
    cur = np.broadcast_to(p, q.shape).copy()
    valid = np.ones(m, bool)
    opl = np.zeros(m)
    loss_db, sum_par, sum_perp = np.zeros(m), np.zeros(m), np.zeros(m)
    tau2 = np.ones(m)
    c_first = x_first = c_last = None
    idx = []
    for i, (gc, gn, coef, mp, mn) in enumerate(consts):
        x1 = snell(cur, q, mp, mn, n_leg[i], n_leg[i + 1], 10).x
        pt, nr, row, col = _lookup(gc, gn, coef, gc.shape[0], gc.shape[1],
                                   x1)
        idx.append((row, col))
        nr = nr * (1.0 / np.sqrt(dot3(nr, nr)))[:, None]
        r = snell(cur, q, pt, nr, n_leg[i], n_leg[i + 1], 25)
        valid &= r.valid
        c_inc = np.maximum(np.cos(r.theta1), C_MIN)
        if i == 0:
            c_first, x_first = c_inc, r.x
        g = fresnel_te_gamma(eps_leg[i], eps_leg[i + 1], c_inc)
        tau2 = tau2 * (1.0 - g * g)
        if sig_c is not None:
            kt = k0 * (n_leg[i] * c_inc - n_leg[i + 1] * np.cos(r.theta2))
            tau2 = tau2 * np.exp(-2.0 * (sig_c[i] * kt) ** 2)
        opl = opl + n_leg[i] * r.s1
        loss_db = loss_db + r.s1 * (att[i] / 1000.0)
        sum_perp = sum_perp + r.s1 / n_leg[i]
        sum_par = sum_par + r.s1 / (n_leg[i] * c_inc * c_inc)
        c_last = np.maximum(np.cos(r.theta2), C_MIN)
        cur = r.x
    return (cur, valid, opl, loss_db, sum_par, sum_perp, tau2, c_first,
            c_last, x_first, idx)


def path_joint(p, q, consts, n_leg, eps_leg, att, k0, sig_c, n_newton,
               n_backtrack):
    """Mean-plane chain anchors the facet lookups, then the joint solve on
    the local planes (multilayer.py:408-457)."""
    gc, gn, coef, shp, mp, mn, k_pad = consts
    n_pad = mp.shape[0]
    m = q.shape[0]
    mpb = np.broadcast_to(mp[:, None, :], (n_pad, m, 3))
    mnb = np.broadcast_to(mn[:, None, :], (n_pad, m, 3))
    r1 = sequential_chain(p, q, mpb, mnb, n_leg, n_iter=10)
    pts, nrs, idx = [], [], []
    for i in range(n_pad):
        pt, nr, row, col = _lookup(gc[i], gn[i], coef[i], shp[i][0],
                                   shp[i][1], r1.x[i])
        idx.append((row, col))
        pts.append(pt)
        nrs.append(nr / np.linalg.norm(nr, axis=-1, keepdims=True))
    r2 = joint_crossings(p, q, np.stack(pts), np.stack(nrs), n_leg,
                         n_newton=n_newton, n_backtrack=n_backtrack)
    s_up = r2.s[:-1]
    c_inc = np.maximum(np.cos(r2.theta1), C_MIN)
    c_surf = c_inc[k_pad]
    is_pad = (np.arange(n_pad) < k_pad)[:, None]
    g = fresnel_te_gamma(eps_leg[:-1, None], eps_leg[1:, None], c_inc)
    tau2 = np.prod(1.0 - g * g, axis=0)
    if sig_c is not None:
        kt = k0 * (n_leg[:-1, None] * np.cos(r2.theta1)
                   - n_leg[1:, None] * np.cos(r2.theta2))
        tau2 = tau2 * np.prod(np.exp(-2.0 * (sig_c[:, None] * kt) ** 2),
                              axis=0)
    c_par = np.where(is_pad, c_surf[None], c_inc)
    nl = n_leg[:-1, None]
    opl = np.sum(nl * s_up, axis=0)
    loss_db = np.sum(s_up * (att[:-1, None] / 1000.0), axis=0)
    sum_perp = np.sum(s_up / nl, axis=0)
    sum_par = np.sum(s_up / (nl * c_par * c_par), axis=0)
    c_last = np.maximum(np.cos(r2.theta2[-1]), C_MIN)
    return (r2.x[-1], r2.valid, opl, loss_db, sum_par, sum_perp, tau2,
            c_surf, c_last, r2.x[0], idx)


def refracted_cluttergram(positions, u_ct, target, crossed, eps_leg, att_leg,
                          *, mode, t0, dt, n_samples, c, gamma=0.0, k0=None,
                          split_sides=False, pattern=None, roughness=None,
                          crossed_sigma=None, diffuse=None, taper_s=None,
                          d_phi_area=False, block_size=None,
                          refraction="sequential", pad_to=None,
                          joint_newton=6, joint_backtrack=4, window_cull=True,
                          return_lookups=False):
    """Float64 refracted-path cluttergram (multilayer.py:594-770).

    Returns (out, dropped): complex128 field (coherent) or float64 power
    (incoherent), (T, n) or (T, n, 2); dropped float64 (T,). With
    ``return_lookups`` also returns, per trace, the (row, col) facet indices
    each lookup selected (the indexing decisions checked bit-exactly)."""
    coherent = mode == "coherent"
    joint = refraction == "joint"
    if (roughness is not None or crossed_sigma is not None) and not coherent:
        raise ValueError("roughness requires coherent mode")
    if (taper_s is not None or d_phi_area) and not coherent:
        raise ValueError("the grazing fix requires coherent mode")
    gamma_arr = np.asarray(gamma, np.float64)
    gamma_facet = gamma_arr.ndim > 0
    if gamma_facet and not coherent:
        raise ValueError("per-facet gamma requires coherent mode")
    eps = np.asarray(eps_leg, np.float64)
    n_leg = np.sqrt(eps)
    att = np.asarray(att_leg, np.float64)
    pos = np.asarray(positions, np.float64)
    uct = np.asarray(u_ct, np.float64)
    sig_c = (None if crossed_sigma is None
             else np.asarray(crossed_sigma, np.float64))
    if joint:
        consts = joint_consts(crossed, pad_to or len(crossed),
                              pos[:, 2].min())
        kp = consts[-1]
        n_leg = np.concatenate([np.full(kp, n_leg[0]), n_leg])
        eps = np.concatenate([np.full(kp, eps[0]), eps])
        att = np.concatenate([np.full(kp, att[0]), att])
        if sig_c is not None:
            sig_c = np.concatenate([np.zeros(kp), sig_c])
    else:
        consts = [grid_consts(f) for f in crossed]
    n = target.centers.shape[0]
    order, bs, n_blocks, off, n_win = culling_plan(
        pos, target.centers, t0=t0, dt=dt, n_samples=n_samples, c=c,
        block_size=block_size or (4096 if joint else None),
        target_pairs=1 << 18, window_cull=window_cull)

    def fq(a):
        return np.asarray(a, np.float32)[order].astype(np.float64)

    cf, nf, af, f1, f2 = (fq(target.centers), fq(target.normals),
                          fq(target.areas), fq(target.e1), fq(target.e2))
    rough = None
    if roughness is not None:
        sig_t, l_t, ph, n_terms, *rest = roughness
        acf = rest[0] if rest else "gaussian"
        if acf == "exponential" and not d_phi_area:
            raise ValueError("roughness acf='exponential' requires the "
                             "area-only D_Phi (d_phi_area / grazing fix)")
        sig_t = fq(sig_t) if np.ndim(sig_t) else float(sig_t)
        l_t = fq(l_t) if np.ndim(l_t) else float(l_t)
        rough = (sig_t, l_t, np.asarray(ph, np.complex64)[order].astype(
            np.complex128), int(n_terms), acf)
    dif = None
    if diffuse is not None:
        if not coherent:
            raise ValueError("diffuse channel requires coherent mode")
        d_amp, d_ph, n_exp = diffuse
        d_amp = np.asarray(d_amp, np.float64)
        if d_amp.shape != (n,):
            raise ValueError(f"diffuse amp shape {d_amp.shape} != ({n},)")
        dif = (d_amp[order], np.asarray(d_ph, np.complex64)[order].astype(
            np.complex128), float(n_exp))
    if gamma_facet:
        if gamma_arr.shape != (n,):
            raise ValueError(f"per-facet gamma shape {gamma_arr.shape} != "
                             f"({n},)")
        gam_all = gamma_arr[order]
    kind, pv, pa, pb = pattern or ("isotropic", np.zeros((len(pos), 3)), 0.0,
                                   0.0)
    pv = np.asarray(pv, np.float64)
    n_seg = (2 if split_sides else 1) * n_samples
    out = np.zeros((len(pos), n_seg),
                   np.complex128 if coherent else np.float64)
    drop = np.zeros(len(pos))
    lookups = []
    k0 = 0.0 if k0 is None else float(k0)
    for t in range(len(pos)):
        lo_i = int(off[t]) * bs
        sl = slice(lo_i, min((int(off[t]) + n_win) * bs, n))
        p = pos[t]
        q = cf[sl]
        with np.errstate(invalid="ignore", divide="ignore", over="ignore"):
            if joint:
                res = path_joint(p, q, consts, n_leg, eps, att, k0, sig_c,
                                 joint_newton, joint_backtrack)
            else:
                res = path_sequential(p, q, consts, n_leg, eps, att, k0,
                                      sig_c)
            (cur, valid, opl, loss_db, sum_par, sum_perp, tau2, c0, c_last,
             x_first, idx) = res
            lookups.append(idx)
            d = cur - q
            s_j = np.sqrt(dot3(d, d))
            rhat = d * (1.0 / np.maximum(s_j, 1e-30))[:, None]
            nj = n_leg[-1]
            opl = opl + nj * s_j
            loss_db = loss_db + s_j * (att[-1] / 1000.0)
            sum_perp = sum_perp + s_j / nj
            sum_par = sum_par + s_j / (nj * c_last * c_last)
            l_perp = n_leg[0] * sum_perp
            l_par = n_leg[0] * c0 * c0 * sum_par
            flux = (n_leg[0] * c0) / (nj * c_last)
            att_f = 10.0 ** (-loss_db / 10.0)
            cos_t = dot3(rhat, nf[sl])
            spread = tau2 * flux / (l_par * l_perp)
            if kind != "isotropic":
                d0 = x_first - p
                dm = np.maximum(np.sqrt(dot3(d0, d0)), 1e-30)
                g = antenna.gain(kind, d0 / dm[:, None], pv[t], pa, pb)
                spread = spread * (g * g)
            fa = af[sl]
            if coherent:
                gam = gam_all[sl] if gamma_facet else float(gamma_arr)
                kj = k0 * nj
                d1 = dot3(rhat, f1[sl])
                d2 = dot3(rhat, f2[sl])
                s1 = np.sinc(d1 * (kj / np.pi))
                s2 = np.sinc(d2 * (kj / np.pi))
                amp = ((kj / TWO_PI) * gam * cos_t * fa * s1 * s2 * spread
                       * att_f)
                if taper_s is not None:
                    ct2 = np.clip(cos_t, C_MIN, 1.0) ** 2
                    amp = amp * np.exp(-(1.0 - ct2)
                                       / (ct2 * (2.0 * taper_s * taper_s)))
                if rough is not None:
                    sg, lc, ph, n_terms, acf = rough
                    sg = sg if np.ndim(sg) == 0 else sg[sl]
                    lc = lc if np.ndim(lc) == 0 else lc[sl]
                    l1 = np.sqrt(dot3(f1[sl], f1[sl]))
                    l2 = np.sqrt(dot3(f2[sl], f2[sl]))
                    kk = 2.0 * kj * cos_t
                    dp = rough_model.d_phi(sg, lc, kk, 2.0 * kj * d1 / l1,
                                         2.0 * kj * d2 / l2, l1, l2,
                                         n_terms=n_terms,
                                         area_only=d_phi_area, acf=acf)
                    amp = (amp * rough_model.mean_attenuation(sg, kk)
                           + np.where(fa > 0, (kj / TWO_PI) * gam * cos_t
                                      * spread * att_f * np.sqrt(dp)
                                      * ph[sl], 0.0))
                if dif is not None:
                    d_amp, d_ph, n_exp = dif
                    ct = np.maximum(cos_t, 0.0)
                    a_d = (np.sqrt(np.maximum(fa, 0.0) / TWO_PI) * d_amp[sl]
                           * ct * ct ** (0.5 * n_exp) * spread * att_f)
                    amp = amp + np.where(fa > 0, a_d * d_ph[sl], 0.0)
                contrib = 1j * amp * np.exp(-2j * k0 * opl)
                pwr = np.abs(contrib) ** 2
            else:
                a = fa * cos_t * spread
                contrib = a * a * att_f * att_f
                pwr = contrib
            b = twtt_bin(2.0 * opl / c, t0, dt)
            ok = valid & (b >= 0) & (b < n_samples)
            if split_sides:
                right = (dot3(q - p, uct[t]) > 0).astype(np.int32)
                b = b + right * n_samples
            np.add.at(out[t], b[ok], contrib[ok])
            drop[t] += float(np.sum(pwr[~ok]))
    if split_sides:
        out = out.reshape(-1, 2, n_samples).transpose(0, 2, 1)
    if return_lookups:
        return out, drop, lookups
    return out, drop
