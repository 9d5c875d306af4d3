"""Drop-in ``refracted_cluttergram`` on GB300.

Mirrors soundersim ``kernels/multilayer.py:594-770``: same arguments, the
same host preparation (per-interface lookup tables and mean planes,
``_grid_consts`` :269-283; joint no-op padding, ``_joint_consts`` :286-330;
leg arrays; culling; float32 facet quantisation) and the same ``ValueError``
texts. The device program is ``ss_refracted_fwd``; there is no CPU path.

``prepare_refracted`` stages everything on the device once and returns a
plan whose ``run()`` only launches the kernel (the form the batched and
benchmark paths use); ``refracted_cluttergram`` is prepare + run + copy back.
"""

import ctypes as C

import numpy as np
import torch

from . import _lib
from .coherent import (_dev, _field_to_host, pattern_struct, permuted,
                       rough_struct, stage_facets, to_host)
from .geometry import cull_plan, group_within_blocks


def _affine_fit(cen, rc):
    """Least-squares (x, y, 1) -> (row, col) fit, the problem
    multilayer.py:277-278 hands to lstsq, solved through the 2x2 normal
    equations of the centred coordinates (equal to the SVD solution to
    float64 rounding for a frame centred near the scene). The moments come
    from two matrix products over the (N, 3) centres, so the fit costs about
    one pass over the data. ``rc`` (N, 2). Returns coef (3, 2): rows x, y,
    1."""
    n = len(cen)
    G = cen.T @ cen                       # raw second moments
    m = (np.ones(n) @ cen) / n            # means
    S = G[:2, :2] - n * np.outer(m[:2], m[:2])
    det = S[0, 0] * S[1, 1] - S[0, 1] * S[1, 0]
    if not det > 1e-12 * max(S[0, 0] * S[1, 1], 1e-300):
        a = np.column_stack([cen[:, :2], np.ones(n)])
        return np.linalg.lstsq(a, rc, rcond=None)[0]
    mr = (np.ones(n) @ rc) / n
    B = (cen.T @ rc)[:2] - n * np.outer(m[:2], mr)
    cx = (S[1, 1] * B[0] - S[0, 1] * B[1]) / det
    cy = (S[0, 0] * B[1] - S[0, 1] * B[0]) / det
    return np.vstack([cx, cy, mr - cx * m[0] - cy * m[1]])


def grid_consts_device(f, device):
    """Lookup table (ny, nx, 6) float32 [centre, normal], affine (x, y, 1) ->
    (row, col) least-squares fit, area-weighted mean point and unit normal
    (multilayer.py:269-283). The per-facet work runs on the device: one
    float64 upload of centres, normals, areas and cells, the float32 table
    and the moments of the fit and the mean plane formed there, 27 numbers
    back. Returns (table tensor on ``device``, coef (3, 2), mean point, unit
    mean normal)."""
    ny, nx = f.grid_shape
    cen = torch.from_numpy(np.ascontiguousarray(f.centers, np.float64)).to(
        device)
    nrm = torch.from_numpy(np.ascontiguousarray(f.normals, np.float64)).to(
        device)
    area = torch.from_numpy(np.ascontiguousarray(f.areas, np.float64)).to(
        device)
    rc = torch.from_numpy(np.ascontiguousarray(f.cell)).to(device).to(
        torch.float64)
    tab = torch.cat([cen, nrm], 1).to(torch.float32).reshape(ny, nx, 6)
    n = cen.shape[0]
    # moments as elementwise products and tree reductions (a (3 x N) (N x 3)
    # float64 GEMM is a poor shape for the tensor-core DGEMM: ~1 ms each)
    small = torch.cat([(cen[:, :, None] * cen[:, None, :]).sum(0).reshape(-1),
                       cen.sum(0), rc.sum(0),
                       (cen[:, :, None] * rc[:, None, :]).sum(0).reshape(-1),
                       area.sum().reshape(1), (area[:, None] * cen).sum(0),
                       (area[:, None] * nrm).sum(0)]).cpu().numpy()
    G = small[0:9].reshape(3, 3)
    m = small[9:12] / n
    mr = small[12:14] / n
    CR = small[14:20].reshape(3, 2)
    sa = small[20]
    mp = small[21:24] / sa
    mn = small[24:27]
    S = G[:2, :2] - n * np.outer(m[:2], m[:2])
    det = S[0, 0] * S[1, 1] - S[0, 1] * S[1, 0]
    if not det > 1e-12 * max(S[0, 0] * S[1, 1], 1e-300):
        coef = _affine_fit(np.asarray(f.centers, np.float64),
                           np.asarray(f.cell, np.float64))
    else:
        B = CR[:2] - n * np.outer(m[:2], mr)
        cx = (S[1, 1] * B[0] - S[0, 1] * B[1]) / det
        cy = (S[0, 0] * B[1] - S[0, 1] * B[0]) / det
        coef = np.vstack([cx, cy, mr - cx * m[0] - cy * m[1]])
    return tab, coef, mp, mn / np.linalg.norm(mn)


def pad_planes(crossed, pad_to, z_platform):
    """No-op air planes stacked above the surface (multilayer.py:311-321):
    returns their heights top-down."""
    k = pad_to - len(crossed)
    if k < 0:
        raise ValueError(f"pad_to={pad_to} < {len(crossed)} crossed "
                         "interfaces")
    if k == 0:
        return np.zeros(0)
    z_surf = float(np.asarray(crossed[0].centers)[:, 2].max())
    gap = float(z_platform) - z_surf
    if gap <= 0:
        raise ValueError("joint refraction padding needs the platform above "
                         f"the surface (gap {gap:.1f} m)")
    return z_surf + gap * (np.arange(k, 0, -1) / (k + 1.0))


class RefractedPlan:
    """Device-resident inputs of one refracted_cluttergram call."""

    def __init__(self, **kw):
        self.__dict__.update(kw)

    def run(self, precision=None, out=None):
        """Launch the kernel on the current stream; returns device tensors
        (field (T, n_seg, 2) float64 re/im, dropped (T,) float64)."""
        prec = _lib.PREC[precision or self.precision]
        self.opts.precision = prec
        L = _lib.lib()
        nbytes = L.ss_refracted_scratch_bytes(C.byref(self.opts), self.T,
                                              self.N)
        if nbytes == 0:
            raise ValueError("unsupported sizes for the refracted kernel")
        if self.scratch is None or self.scratch.numel() < nbytes:
            self.scratch = torch.empty(nbytes, dtype=torch.uint8,
                                       device=self.device)
        if out is None:
            field = torch.empty((self.T, self.n_seg, 2), dtype=torch.float64,
                                device=self.device)
            dropped = torch.empty(self.T, dtype=torch.float64,
                                  device=self.device)
        else:
            field, dropped = out
        o = _lib.Output(field.data_ptr(), None, dropped.data_ptr())
        stream = torch.cuda.current_stream(self.device).cuda_stream
        st = L.ss_refracted_fwd(C.byref(self.opts), C.byref(self.fst),
                                C.byref(self.tr), C.byref(self.pst),
                                C.byref(self.rst), C.byref(o),
                                C.c_void_p(self.scratch.data_ptr()), nbytes,
                                C.c_void_p(stream))
        _lib.check(st, "ss_refracted_fwd")
        return field, dropped

    def kernel_launches(self, precision=None):
        """Library kernels one ``run()`` launches: main pass and chunk
        reduce, plus the split form's fix-up pass."""
        return 2 if (precision or self.precision) == "fp64" else 3

    def to_numpy(self, field, dropped, out_dtype=None):
        if self.coherent:
            res = _field_to_host(field, out_dtype or np.complex64)
        else:
            res = field[..., 0].to(torch.float32 if (out_dtype or np.float32)
                                   == np.float32 else torch.float64)
            res = to_host(res).astype(out_dtype or np.float32, copy=False)
        if self.split:
            res = res.reshape(self.T, self.n_samples, 2)
        return res, to_host(dropped.to(torch.float32))


def prepare_refracted(positions, u_ct, target, crossed, eps_leg, att_leg, *,
                      mode, t0, dt, n_samples, c, gamma=0.0, k0=None,
                      split_sides=False, pattern=None, roughness=None,
                      crossed_sigma=None, diffuse=None, taper_s=None,
                      d_phi_area=False, block_size=None,
                      refraction="sequential", pad_to=None, joint_newton=6,
                      joint_backtrack=4, window_cull=True, precision="fp64",
                      device=None):
    """Validate, build the host-side constants and stage all inputs."""
    device = torch.device(device or "cuda")
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
    if precision not in _lib.PREC:
        raise ValueError(f"unknown precision {precision!r}")
    # the remaining argument errors also come before any device work
    n = np.asarray(target.centers).shape[0]
    rst, s_arr, l_arr, phasors = rough_struct(roughness, d_phi_area)
    if diffuse is not None:
        if not coherent:
            raise ValueError("diffuse channel requires coherent mode")
        d_amp = np.asarray(diffuse[0], np.float64)
        if d_amp.shape != (n,):
            raise ValueError(f"diffuse amp shape {d_amp.shape} != ({n},)")
    if gamma_facet and gamma_arr.shape != (n,):
        raise ValueError(f"per-facet gamma shape {gamma_arr.shape} != "
                         f"({n},)")
    if pattern is not None and pattern[0] not in _lib.PATTERN:
        raise ValueError(f"unknown pattern kind {pattern[0]!r}")
    eps = np.asarray(eps_leg, np.float64)
    n_leg = np.sqrt(eps)
    att = np.asarray(att_leg, np.float64)
    pos = np.asarray(positions, np.float64)
    T = len(pos)
    sig_c = (None if crossed_sigma is None
             else np.asarray(crossed_sigma, np.float64))
    ifaces, keep = [], []
    k_pad = 0
    if joint:
        zs = pad_planes(crossed, pad_to or len(crossed), pos[:, 2].min())
        k_pad = len(zs)
        for z in zs:
            tab = np.array([[[0.0, 0.0, z, 0.0, 0.0, 1.0]]], np.float32)
            ifaces.append((tab, np.zeros((3, 2)), np.array([0.0, 0.0, z]),
                           np.array([0.0, 0.0, 1.0])))
        n_leg = np.concatenate([np.full(k_pad, n_leg[0]), n_leg])
        eps = np.concatenate([np.full(k_pad, eps[0]), eps])
        att = np.concatenate([np.full(k_pad, att[0]), att])
        if sig_c is not None:
            sig_c = np.concatenate([np.zeros(k_pad), sig_c])
    ni = k_pad + len(crossed)
    if not 1 <= ni <= 40:
        raise ValueError(f"{ni} crossed interfaces; the kernel takes 1..40")
    if len(n_leg) < ni + 1 or (joint and len(n_leg) != ni + 1):
        raise ValueError("eps_leg/att_leg need len(crossed) + 1 entries")
    ifaces += [grid_consts_device(f, device) for f in crossed]
    arr = (_lib.Interface * ni)()
    for j, (tab, coef, mp, mn) in enumerate(ifaces):
        t = (tab if isinstance(tab, torch.Tensor)
             else _dev(tab, np.float32, device))
        keep.append(t)
        arr[j].table = t.data_ptr()
        arr[j].ny, arr[j].nx = tab.shape[0], tab.shape[1]
        arr[j].coef[:] = list(np.asarray(coef, np.float64).ravel())
        arr[j].mean_point[:] = list(np.asarray(mp, np.float64))
        arr[j].mean_normal[:] = list(np.asarray(mn, np.float64))
    legs = [np.ascontiguousarray(v, np.float64) for v in (n_leg, eps, att)]
    sig_arr = (np.ascontiguousarray(sig_c, np.float64) if sig_c is not None
               else None)

    centers = np.asarray(target.centers)
    bs_req = block_size or (4096 if joint else None)
    plan = cull_plan(pos, centers, t0=t0, dt=dt, n_samples=n_samples, c=c,
                     block_size=bs_req, target_pairs=1 << 18,
                     window_cull=window_cull, device=device)
    if s_arr is not None:     # per-facet rms heights: similar series lengths
        plan = group_within_blocks(plan, s_arr)   # share a warp
    fac = stage_facets(centers, target.normals, target.areas, target.e1,
                       target.e2, plan.order, device, sigma=s_arr,
                       corr=l_arr, phasors=phasors)
    n_exp = 0.0
    if diffuse is not None:
        _, d_ph, n_exp = diffuse
        fac.extras["diffuse_amp"] = permuted(d_amp, np.float64, plan.order,
                                             device)
        fac.extras["diffuse_phasor"] = permuted(
            np.ascontiguousarray(d_ph, np.complex64).view(
                np.float32).reshape(n, 2), np.float32, plan.order,
            device).reshape(-1)
    if gamma_facet:
        fac.extras["gamma_f64"] = permuted(gamma_arr, np.float64,
                                           plan.order, device)
    pst, pv_t, pv_len, pkeep = pattern_struct(pattern, T, device)
    pos_t = _dev(pos, np.float64, device)
    uct_t = _dev(np.asarray(u_ct, np.float64).reshape(T, 3), np.float64,
                 device)
    off_t = _dev(plan.off, np.int32, device)
    tr = _lib.Traces(pos_t.data_ptr(), uct_t.data_ptr(),
                     pv_t.data_ptr() if pv_t is not None else None,
                     off_t.data_ptr(), T, pv_len)
    opts = _lib.RefractedOpts()
    opts.n_crossed = ni
    opts.k_pad = k_pad
    opts.n_legs = len(n_leg)
    opts.crossed = C.cast(arr, C.POINTER(_lib.Interface))
    opts.n_leg = legs[0].ctypes.data_as(C.POINTER(C.c_double))
    opts.eps_leg = legs[1].ctypes.data_as(C.POINTER(C.c_double))
    opts.att_leg = legs[2].ctypes.data_as(C.POINTER(C.c_double))
    opts.sigma_crossed = (sig_arr.ctypes.data_as(C.POINTER(C.c_double))
                          if sig_arr is not None else None)
    opts.k0 = 0.0 if k0 is None else float(k0)
    opts.gamma = 0.0 if gamma_facet else float(gamma_arr)
    opts.t0, opts.dt, opts.c = float(t0), float(dt), float(c)
    opts.taper_s = float(taper_s or 0.0)
    opts.diffuse_exp = float(n_exp)
    opts.n_samples = int(n_samples)
    opts.block_size = plan.block_size
    opts.n_win = plan.n_win
    opts.split_sides = int(bool(split_sides))
    opts.coherent = int(coherent)
    opts.joint = int(joint)
    opts.joint_newton = int(joint_newton)
    opts.joint_backtrack = int(joint_backtrack)
    opts.taper = int(taper_s is not None)
    opts.precision = _lib.PREC[precision]
    return RefractedPlan(
        opts=opts, fst=fac.struct(), tr=tr, pst=pst, rst=rst,
        keep=[fac, keep, pkeep, pos_t, uct_t, off_t, pv_t, arr, legs,
              sig_arr],
        T=T, N=n, n_samples=int(n_samples),
        n_seg=int(n_samples) * (2 if split_sides else 1),
        split=bool(split_sides), coherent=coherent, device=device,
        precision=precision, scratch=None, cull=plan, fac=fac, legs=legs,
        ifaces=arr)


def refracted_cluttergram(positions, u_ct, target, crossed, eps_leg, att_leg,
                          *, mode, t0, dt, n_samples, c, gamma=0.0, k0=None,
                          split_sides=False, pattern=None, roughness=None,
                          crossed_sigma=None, diffuse=None, taper_s=None,
                          d_phi_area=False, block_size=None,
                          refraction="sequential", pad_to=None,
                          joint_newton=6, joint_backtrack=4, window_cull=True,
                          precision="fp64", out_dtype=None, device=None):
    """Binned refracted-path contributions from one target interface
    (multilayer.py:594-770). Returns ``(out, dropped)``: complex64 field
    (coherent) or float32 power (incoherent), (T, n) or (T, n, 2); dropped
    (T,) float32 (out-of-window and invalid-path power)."""
    plan = prepare_refracted(
        positions, u_ct, target, crossed, eps_leg, att_leg, mode=mode, t0=t0,
        dt=dt, n_samples=n_samples, c=c, gamma=gamma, k0=k0,
        split_sides=split_sides, pattern=pattern, roughness=roughness,
        crossed_sigma=crossed_sigma, diffuse=diffuse, taper_s=taper_s,
        d_phi_area=d_phi_area, block_size=block_size, refraction=refraction,
        pad_to=pad_to, joint_newton=joint_newton,
        joint_backtrack=joint_backtrack, window_cull=window_cull,
        precision=precision, device=device)
    field, dropped = plan.run()
    return plan.to_numpy(field, dropped, out_dtype)
