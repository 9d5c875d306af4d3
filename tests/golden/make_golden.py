"""Freeze the reference's own outputs as golden fixtures (run here, once).

    SOUNDERSIM_REF=/path/to/reference PYTHONPATH=. \
        python tests/golden/make_golden.py [--only a,b]
    PYTHONPATH=. python tests/golden/make_golden.py [--only a,b] /path/to/reference

Runs the UNMODIFIED soundersim source (``refload`` + ``jaxshim``: NumPy in
place of JAX) on small seeded scenes and writes ``tests/golden/*.npz``.
The GPU host never runs this; it only reads the committed ``.npz`` files.
Every case stores its inputs next to the reference outputs so the tests are
self-contained.
"""

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
if __package__ in (None, ""):
    sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
    from tests.golden import refload, xrshim  # noqa: E402
else:
    from . import refload, xrshim

C = 299792458.0


def grid_scene(Facets, n, d, z0, amp, seed, slope=(0.0, 0.0)):
    """Vertex grid -> mean-plane facets (the build_facets corner rule,
    scene.py:156-166) on a planar frame; seeded white relief."""
    rng = np.random.default_rng(seed)
    ax = (np.arange(n + 1) - n / 2) * d
    X, Y = np.meshgrid(ax, ax)
    Z = z0 + amp * rng.standard_normal(X.shape) + slope[0] * X + slope[1] * Y
    V = np.stack([X, Y, Z], -1)
    v00, v01, v10, v11 = V[:-1, :-1], V[:-1, 1:], V[1:, :-1], V[1:, 1:]
    e1 = ((v01 + v11) - (v00 + v10)) / 2.0
    e2 = ((v10 + v11) - (v00 + v01)) / 2.0
    c = ((v00 + v01 + v10 + v11) / 4.0).reshape(-1, 3)
    raw = np.cross(e1, e2).reshape(-1, 3)
    a = np.linalg.norm(raw, axis=1)
    nr = raw / a[:, None]
    nr *= np.where(nr[:, 2] < 0, -1.0, 1.0)[:, None]
    ci, cj = np.meshgrid(np.arange(n), np.arange(n), indexing="ij")
    return Facets(c, nr, a, e1.reshape(-1, 3), e2.reshape(-1, 3),
                  np.stack([ci.ravel(), cj.ravel()], 1), (n, n))


def facet_dict(prefix, f):
    return {f"{prefix}_centers": f.centers, f"{prefix}_normals": f.normals,
            f"{prefix}_areas": f.areas, f"{prefix}_e1": f.e1,
            f"{prefix}_e2": f.e2, f"{prefix}_cell": f.cell,
            f"{prefix}_grid": np.asarray(f.grid_shape)}


def track(n, z, dx, y=0.0, x0=None):
    x0 = -(n - 1) * dx / 2 if x0 is None else x0
    p = np.column_stack([x0 + dx * np.arange(n), np.full(n, y),
                         np.full(n, z) + 0.37 * np.sin(np.arange(n))])
    u = np.tile([0.0, -1.0, 0.0], (n, 1))
    return p, u


def make_primitives(ns):
    out = {}
    rng = np.random.default_rng(11)
    # Faddeeva on the closed upper half plane
    z = rng.uniform(-30, 30, 200) + 1j * rng.uniform(0, 40, 200)
    out["fad_z"] = z
    out["fad_w"] = np.asarray(ns.roughness.faddeeva(z))
    # d_phi, all three forms, float64 (roughness.py:127-186)
    m = 64
    K = rng.uniform(0.5, 20.0, m)
    A0 = rng.uniform(-3, 3, m)
    B0 = rng.uniform(-3, 3, m)
    Lx = rng.uniform(5, 60, m)
    Ly = rng.uniform(5, 60, m)
    out.update(dp_K=K, dp_A0=A0, dp_B0=B0, dp_Lx=Lx, dp_Ly=Ly)
    for tag, kw in (("full", dict()), ("area", dict(area_only=True)),
                    ("exp", dict(area_only=True, acf="exponential"))):
        out[f"dp_{tag}"] = np.asarray(ns.roughness.d_phi(
            0.31, 4.0, K, A0, B0, Lx, Ly, n_terms=120, **kw))
    xs = np.array([0.0, 0.01, 1.0, 37.5, 250.0, 1e4])
    out["nterms_x"] = xs
    out["nterms"] = np.array([ns.roughness.n_terms_for(x) for x in xs])
    out["phasors_0_0"] = ns.roughness.speckle_phasors(64, (0, 0))
    out["phasors_7_3"] = ns.roughness.speckle_phasors(64, (7, 3))
    # two-point Snell and joint solves, float64
    p = np.array([120.0, -40.0, 2000.0])
    q = np.column_stack([rng.uniform(-900, 900, 32), rng.uniform(-900, 900, 32),
                         rng.uniform(-1500, -100, 32)])
    o = np.zeros(3)
    nrm = np.array([0.05, -0.02, 1.0])
    nrm /= np.linalg.norm(nrm)
    sc = ns.refraction.snell_crossing(p, q, o, nrm, 1.0, 1.78, xp=np)
    out.update(sn_p=p, sn_q=q, sn_o=o, sn_n=nrm, sn_x=sc.x, sn_th1=sc.theta1,
               sn_th2=sc.theta2, sn_s1=sc.s1, sn_s2=sc.s2,
               sn_valid=sc.valid)
    planes_o = np.array([[0, 0, 0.0], [0, 0, -60.0], [0, 0, -400.0]])
    planes_n = np.array([[0.03, 0.0, 1.0], [0.0, 0.04, 1.0], [0.0, 0.0, 1.0]])
    planes_n /= np.linalg.norm(planes_n, axis=1, keepdims=True)
    n_media = np.array([1.0, 1.35, 1.77, 1.78])
    qj = q.copy()
    qj[:, 2] = rng.uniform(-1500, -500, 32)
    jo = np.broadcast_to(planes_o[:, None, :], (3, 32, 3))
    jn = np.broadcast_to(planes_n[:, None, :], (3, 32, 3))
    jc = ns.refraction_joint.joint_crossings(p, qj, jo, jn, n_media)
    ch = ns.refraction_joint.sequential_chain(p, qj, jo, jn, n_media)
    out.update(jt_q=qj, jt_o=planes_o, jt_n=planes_n, jt_media=n_media,
               jt_x=np.asarray(jc.x), jt_s=np.asarray(jc.s),
               jt_th1=np.asarray(jc.theta1), jt_valid=np.asarray(jc.valid),
               ch_x=np.asarray(ch.x), ch_valid=np.asarray(ch.valid))
    return out


def make_antenna(ns):
    cfg = refload.importlib.import_module("soundersim.config")
    rng = np.random.default_rng(5)
    d = rng.normal(size=(80, 3))
    d[:, 2] = -np.abs(d[:, 2]) * 3
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    u_at = np.array([[1.0, 0.0, 0.0]])
    u_ct = np.array([[0.0, -1.0, 0.0]])
    ants = {
        "dipole": cfg.AntennaConfig(kind="dipole"),
        "dipole_ct": cfg.AntennaConfig(kind="dipole", axis="cross_track"),
        "array": cfg.AntennaConfig(kind="array", n_elements=6,
                                   spacing_lam=0.5),
        "array_el": cfg.AntennaConfig(kind="array", n_elements=4,
                                      spacing_lam=0.45,
                                      element_directivity_db=6.0),
        "array_tapered": cfg.AntennaConfig(kind="array_tapered",
                                           tx_weights=[0.5, 1, 1, 0.5],
                                           rx_weights=[1, 1, 1, 1],
                                           spacing_lam=0.5),
        "finite_dipole": cfg.AntennaConfig(kind="finite_dipole",
                                           length_lam=0.8),
        "tabulated": cfg.AntennaConfig(kind="tabulated",
                                       theta_deg=[0, 10, 25, 45, 90],
                                       gain=[1.0, 0.9, 0.5, 0.1, 0.01]),
    }
    out = {"ant_dhat": d}
    for name, a in ants.items():
        kind, pv, pa, pb = ns.antenna.pattern_args(a, u_at, u_ct)
        g = ns.antenna.gain_fn(kind)(d, pv[0], np.asarray(pa),
                                     np.asarray(pb))
        out[f"ant_{name}_pv"] = pv[0]
        out[f"ant_{name}_pa"] = np.asarray(pa, np.float64)
        out[f"ant_{name}_pb"] = np.asarray(pb, np.float64)
        out[f"ant_{name}_g"] = np.asarray(g)
        out[f"ant_{name}_kind"] = np.array(kind)
    return out


def make_coherent(ns):
    out = {}
    F = ns.Facets
    surf = grid_scene(F, 32, 25.0, 0.0, 1.5, seed=1, slope=(0.02, -0.01))
    out.update(facet_dict("surf", surf))
    p, u = track(12, 1500.0, 40.0)
    out.update(pos=p, uct=u)
    lam = 5.0
    k = 2 * np.pi / lam
    r = np.linalg.norm(p[:, None, :] - surf.centers[None], axis=-1)
    t0 = 2 * (r.min() - 20.0) / C
    dt = 2.0e-8
    n_s = 160
    base = dict(k=k, gamma=-0.279, t0=t0, dt=dt, n_samples=n_s, c=C)
    out.update(k=k, gamma=-0.279, t0=t0, dt=dt, n_samples=n_s)
    # per-pair float64 formulas (coherent.py:107-168 with xp=np)
    f64 = {a: getattr(surf, a) for a in ("centers", "normals", "areas", "e1",
                                          "e2")}
    cp, rp = ns.coherent.lpa_contributions(p[3], f64["centers"],
                                           f64["normals"], f64["areas"],
                                           f64["e1"], f64["e2"], k, -0.279,
                                           xp=np)
    out.update(pair_contrib=cp, pair_r=rp)
    cpt, _ = ns.coherent.lpa_contributions(p[3], f64["centers"],
                                           f64["normals"], f64["areas"],
                                           f64["e1"], f64["e2"], k, -0.279,
                                           xp=np, taper_s=0.05)
    out["pair_contrib_taper"] = cpt
    ph = ns.roughness.speckle_phasors(len(surf.centers), (0, 0))
    out["phasors"] = ph
    for tag, kw in (("full", {}), ("area", dict(area_only=True)),
                    ("exp", dict(area_only=True, acf="exponential"))):
        cr, _ = ns.coherent.rough_lpa_contributions(
            p[3], f64["centers"], f64["normals"], f64["areas"], f64["e1"],
            f64["e2"], k, -0.279, 0.3, 4.0, ph.astype(np.complex128), 40,
            taper_s=0.05 if tag != "full" else None, **kw)
        out[f"pair_rough_{tag}"] = np.asarray(cr)
    # culling (geometry.py) at a block size that makes windows bite
    order, s_t, s_sorted = ns.geometry.along_track_order(p, surf.centers)
    reach = ns.geometry.window_reach_m(t0, dt, n_s, C)
    off, n_win = ns.geometry.block_windows(s_sorted, s_t, reach * 0.35, 64,
                                           -(-len(order) // 64))
    out.update(cull_order=order, cull_off=off, cull_nwin=np.array(n_win),
               cull_reach=np.array(reach),
               auto_bs=np.array([ns.geometry.auto_block_size(t, 1 << 19)
                                 for t in (1, 12, 256, 1024, 5000)]))
    # full reference kernel (float32 by design)
    gam_f = np.random.default_rng(3).uniform(-0.4, -0.1, len(surf.centers))
    cfg = ns_cfg = refload.importlib.import_module("soundersim.config")
    kind, pv, pa, pb = ns.antenna.pattern_args(
        ns_cfg.AntennaConfig(kind="array", n_elements=4, spacing_lam=0.5),
        np.tile([1.0, 0, 0], (len(p), 1)), u)
    out.update(ant_pv=pv, ant_pa=np.asarray(pa, np.float64),
               ant_pb=np.asarray(pb, np.float64), gamma_facet=gam_f)
    del cfg
    cases = {
        "smooth": dict(),
        "split": dict(split_sides=True),
        "interp": dict(interp_bins=True),
        "blocks": dict(block_size=96),
        "gammaf": dict(gamma=gam_f),
        "array": dict(pattern=(kind, pv, pa, pb)),
        "rough": dict(roughness=(0.3, 4.0, ph, 40)),
        "rough_exp": dict(roughness=(0.3, 4.0, ph, 40, "exponential"),
                          taper_s=0.05, d_phi_area=True),
    }
    for name, kw in cases.items():
        fld, drp = ns.coherent.coherent_cluttergram(
            p, u, surf.centers, surf.normals, surf.areas, surf.e1, surf.e2,
            **{**base, **kw})
        out[f"co_{name}_field"] = fld
        out[f"co_{name}_dropped"] = drp
    return out


def make_refracted(ns):
    out = {}
    F = ns.Facets
    surf = grid_scene(F, 20, 40.0, 0.0, 2.0, seed=21)
    h1 = grid_scene(F, 20, 40.0, -150.0, 1.0, seed=22)
    bed = grid_scene(F, 20, 40.0, -450.0, 4.0, seed=23, slope=(0.01, 0.0))
    for tag, f in (("surf", surf), ("h1", h1), ("bed", bed)):
        out.update(facet_dict(tag, f))
    p, u = track(6, 1200.0, 50.0)
    out.update(pos=p, uct=u)
    k0 = 2 * np.pi / 5.0
    eps = [1.0, 3.15, 3.16]
    att = [0.0, 10.0, 12.0]
    opl_min = 1200 - 5 + 1.775 * 430
    t0 = 2 * opl_min / C
    base = dict(t0=t0, dt=1.5e-8, n_samples=256, c=C)
    out.update(k0=k0, eps=np.array(eps), att=np.array(att), t0=t0, dt=1.5e-8,
               n_samples=256)
    rng = np.random.default_rng(31)
    gam_f = rng.uniform(0.03, 0.3, len(bed.centers))
    ph = ns.roughness.speckle_phasors(len(bed.centers), (0, 2))
    dph = ns.roughness.speckle_phasors(len(bed.centers), (0, 1002))
    damp = rng.uniform(0.0, 0.05, len(bed.centers))
    cfg = refload.importlib.import_module("soundersim.config")
    kind, pv, pa, pb = ns.antenna.pattern_args(
        cfg.AntennaConfig(kind="dipole", axis="cross_track"),
        np.tile([1.0, 0, 0], (len(p), 1)), u)
    out.update(gamma_facet=gam_f, phasors=ph, dif_phasors=dph, dif_amp=damp,
               ant_pv=pv)
    two = [surf, h1]
    cases = {
        "seq1": (bed, [surf], eps[:2] + [3.2], att[:2] + [5.0],
                 dict(mode="coherent", gamma=0.2, k0=k0)),
        "seq2": (bed, two, eps, att, dict(mode="coherent", gamma=0.2, k0=k0)),
        "joint2": (bed, two, eps, att, dict(mode="coherent", gamma=0.2, k0=k0,
                                            refraction="joint")),
        "joint_pad": (bed, two, eps, att,
                      dict(mode="coherent", gamma=0.2, k0=k0,
                           refraction="joint", pad_to=4)),
        "incoh": (bed, two, eps, att, dict(mode="incoherent")),
        "full": (bed, two, eps, att,
                 dict(mode="coherent", gamma=gam_f, k0=k0,
                      roughness=(0.2, 3.0, ph, 30, "exponential"),
                      crossed_sigma=[0.1, 0.02], taper_s=0.05,
                      d_phi_area=True, diffuse=(damp, dph, 1.5),
                      pattern=(kind, pv, pa, pb), split_sides=True)),
        "full_joint": (bed, two, eps, att,
                       dict(mode="coherent", gamma=gam_f, k0=k0,
                            roughness=(0.2, 3.0, ph, 30),
                            crossed_sigma=[0.1, 0.02], refraction="joint",
                            pattern=(kind, pv, pa, pb))),
    }
    for name, (tgt, crossed, e, a, kw) in cases.items():
        o, d = ns.multilayer.refracted_cluttergram(
            p, u, tgt, crossed, e, a, **{**base, **kw})
        out[f"re_{name}_out"] = o
        out[f"re_{name}_dropped"] = d
    return out


def make_waveform(ns):
    out = {}
    for w in ("none", "hann", "hamming"):
        pl, m = ns.waveform.compressed_pulse(15e6, 20e-6, 1.0 / 30e6, w)
        out[f"pulse_{w}"] = pl
        out[f"pulse_{w}_m"] = np.array(m)
    pc, mc = ns.waveform.compressed_pulse(15e6, 8e-6, 1.0 / 30e6, "hann",
                                          "chirp")
    out["pulse_chirp"], out["pulse_chirp_m"] = pc, np.array(mc)
    rng = np.random.default_rng(8)
    arr = (rng.normal(size=(3, 300)) + 1j * rng.normal(size=(3, 300)))
    out["conv_in"] = arr
    out["conv_out"] = ns.waveform.convolve_fast_time(arr, out["pulse_hann"],
                                                     int(out["pulse_hann_m"]))
    # multi-frequency synthesis referee (compare/multifreq.py)
    F = ns.Facets
    s = grid_scene(F, 10, 20.0, 0.0, 0.5, seed=41)
    pos = np.array([10.0, -5.0, 800.0])
    r = np.linalg.norm(pos - s.centers, axis=1)
    tw = 2 * r.min() / C + np.arange(64) * (1.0 / 30e6)
    for frz in (False, True):
        y = ns.multifreq.multifreq_profile(
            pos, s.centers, s.normals, s.areas, s.e1, s.e2, gamma=-0.28,
            f0=60e6, bandwidth=15e6, c=C, twtt=tw, n_freq=64,
            freeze_amplitudes=frz)
        out[f"mf_{'frozen' if frz else 'full'}"] = y
    out.update(facet_dict("mf", s))
    out.update(mf_pos=pos, mf_twtt=tw)
    return out


def make_incoherent(ns):
    """incoherent_cluttergram (kernels/incoherent.py:58-103), float32 by
    design: isotropic, split sides, dipole pattern, small blocks."""
    out = {}
    F = ns.Facets
    surf = grid_scene(F, 32, 25.0, 0.0, 1.5, seed=31, slope=(0.01, 0.02))
    out.update(facet_dict("surf", surf))
    p, u = track(9, 1200.0, 35.0)
    out.update(pos=p, uct=u)
    r = np.linalg.norm(p[:, None, :] - surf.centers[None], axis=-1)
    # the window starts after the nearest facets and ends before the
    # farthest, so both ends drop power
    t0 = 2 * (r.min() + 4.0) / C
    dt, n_s = 2.5e-8, 40
    out.update(t0=t0, dt=dt, n_samples=n_s)
    inc = refload.importlib.import_module("soundersim.kernels.incoherent")
    # per-pair float32 bins through the reference's own geometry helpers
    # (the calls incoherent.py:42 and :47 make)
    f32 = np.float32
    b = [ns.geometry.twtt_bin(
        f32(2.0) * ns.geometry.ranges_and_cos(
            p[t].astype(f32), surf.centers.astype(f32),
            surf.normals.astype(f32))[0] / f32(C), f32(t0), f32(dt))
        for t in range(len(p))]
    out["inc_pair_bins"] = np.stack(b).astype(np.int32)
    ns_cfg = refload.importlib.import_module("soundersim.config")
    kind, pv, pa, pb = ns.antenna.pattern_args(
        ns_cfg.AntennaConfig(kind="dipole", axis="cross_track"),
        np.tile([1.0, 0, 0], (len(p), 1)), u)
    out.update(ant_kind=np.array(kind), ant_pv=pv,
               ant_pa=np.asarray(pa, np.float64),
               ant_pb=np.asarray(pb, np.float64))
    base = dict(t0=t0, dt=dt, n_samples=n_s, c=C)
    cases = {"iso": dict(), "split": dict(split_sides=True),
             "dipole": dict(pattern=(kind, pv, pa, pb)),
             "blocks": dict(block_size=100)}
    for name, kw in cases.items():
        pw, drp = inc.incoherent_cluttergram(p, u, surf.centers, surf.normals,
                                             surf.areas, **{**base, **kw})
        out[f"inc_{name}_power"] = np.asarray(pw)
        out[f"inc_{name}_dropped"] = np.asarray(drp)
    return out


def focus_scene(T, nb, spacing, z, lam, dt, seed):
    """Coherent field of three point targets seen from a jittered straight
    track: per trace a sinc range response at each target's two-way delay
    with carrier phase exp(-2jkR), plus complex noise."""
    rng = np.random.default_rng(seed)
    x = spacing * np.arange(T) + rng.uniform(-0.2, 0.2, T) * spacing
    pos = np.column_stack([x, 0.3 * np.sin(np.arange(T) / 5.0),
                           z + 0.5 * np.cos(np.arange(T) / 7.0)])
    k = 2 * np.pi / lam
    t0 = 2 * (z - 60.0) / C
    twtt = t0 + np.arange(nb) * dt
    targets = np.array([[x[T // 2], 0.0, 0.0], [x[T // 3], 15.0, -20.0],
                        [x[(3 * T) // 4], -10.0, 12.0]])
    F = 0.05 * (rng.standard_normal((T, nb)) +
                1j * rng.standard_normal((T, nb)))
    for tgt, amp in zip(targets, (1.0, 0.6, 0.8)):
        R = np.linalg.norm(pos - tgt, axis=1)
        u = (twtt[None, :] - 2 * R[:, None] / C) / dt
        F += amp * np.sinc(u) * np.exp(-2j * k * R)[:, None]
    return pos, twtt, F.astype(np.complex64)


def make_focus(ns):
    """processing.focused_sar (processing.py:262-348) on a small Dataset,
    through a minimal xarray stand-in; hann and rectangular windows, an
    aperture of about a dozen traces, a non-uniform along-track spacing."""
    xr = xrshim.install()
    proc = refload.importlib.import_module("soundersim.processing")
    T, nb, lam, dt = 64, 96, 5.0, 1.0 / 30e6
    pos, twtt, F = focus_scene(T, nb, 8.0, 800.0, lam, dt, seed=41)
    out = dict(pos=pos, twtt=twtt, field=F, wavelength=lam)

    def dataset():
        return xr.Dataset(
            {"field": (("slow_time", "twtt"), F.copy(), {"units": "V"}),
             "power": (("slow_time", "twtt"), np.abs(F) ** 2, {})},
            coords={"slow_time": ("slow_time", np.arange(T) * 0.1),
                    "twtt": ("twtt", twtt.copy()),
                    "x": ("slow_time", pos[:, 0]),
                    "y": ("slow_time", pos[:, 1]),
                    "z": ("slow_time", pos[:, 2])},
            attrs={"mode": "coherent", "wavelength": lam,
                   "config": '{"radar": {"c": %r}}' % C})
    for name, ap, win in (("hann", 96.0, "hann"), ("rect", 96.0, "none"),
                          ("wide", 250.0, "hann")):
        res = proc.focused_sar(dataset(), ap, window=win)
        out[f"focus_{name}_aperture"] = ap
        out[f"focus_{name}_field"] = np.asarray(res.field.values)
        out[f"focus_{name}_power"] = np.asarray(res.power.values)
    return out


class _AffineLike:
    """Stand-in for affine.Affine (absent here): the attributes and the
    point mapping build_facets uses, (x a + y b + c, x d + y e + f)."""

    def __init__(self, a, b, c, d, e, f):
        self.a, self.b, self.c, self.d, self.e, self.f = a, b, c, d, e, f

    def __mul__(self, xy):
        x, y = xy
        return (x * self.a + y * self.b + self.c,
                x * self.d + y * self.e + self.f)


class _ShiftFrame:
    """LocalFrame stand-in: ECEF -> local is a shift (identity rotation)."""

    def __init__(self, origin):
        self.origin = np.asarray(origin, np.float64)

    def ecef_to_local(self, xyz):
        return np.atleast_2d(xyz) - self.origin


def _pyproj_identity():
    """pyproj stand-in whose transforms are the identity, so build_facets'
    DEM -> projected -> 'ECEF' chain reduces to its own arithmetic."""
    import types
    mod = types.ModuleType("pyproj")

    class Transformer:
        @staticmethod
        def from_crs(*_a, **_k):
            return Transformer()

        def transform(self, x, y, z=None):
            return (x, y) if z is None else (x, y, z)
    mod.Transformer = Transformer
    mod.Proj = None
    sys.modules["pyproj"] = mod


def make_scene(ns):
    """Keyed speckle phasors (roughness.py:207-233) and build_facets
    (scene.py:126-176) through an identity pyproj stand-in and a shift
    frame: lattice, bilinear resampling, affine mapping and corner rule."""
    out = {}
    r, c = np.meshgrid(np.arange(-40, 260, 3), np.arange(700, 980, 7),
                       indexing="ij")
    keys = np.column_stack([r.ravel(), c.ravel()]).astype(np.int64)
    keys = np.concatenate([keys, [[0, 0], [2**40, -5], [-2**45, 2**33]]])
    out["keys"] = keys
    for name, seed in (("s31", (3, 1)), ("s7", 7), ("s11_1002", (11, 1002))):
        out[f"phasors_{name}"] = ns.roughness.speckle_phasors_for_keys(
            keys, seed)
    _pyproj_identity()
    scene = refload.importlib.import_module("soundersim.scene")
    rng = np.random.default_rng(51)
    dem = (800.0 + np.cumsum(rng.normal(0, 2.0, (22, 20)), axis=1)
           + 3.0 * rng.standard_normal((22, 20)))
    tr = (25.0, 0.0, 1000.0, 0.0, -25.0, 5000.0)
    origin = np.array([1400.0, 4500.0, 790.0])
    out.update(dem=dem, transform=np.array(tr), origin=origin)
    for name, sp, go in (("native", None, (0, 0)), ("stride", 50.0, (0, 0)),
                         ("fine", 10.0, (0, 0)),
                         ("crop", 50.0, (3, 5))):
        f = scene.build_facets(dem, _AffineLike(*tr), "EPSG:3413",
                               _ShiftFrame(origin), spacing=sp,
                               grid_origin=go)
        out[f"bf_{name}_spacing"] = np.nan if sp is None else sp
        out[f"bf_{name}_origin"] = np.array(go)
        for k in ("centers", "normals", "areas", "e1", "e2", "cell",
                  "phase_keys"):
            out[f"bf_{name}_{k}"] = getattr(f, k)
        out[f"bf_{name}_grid"] = np.array(f.grid_shape)
    return out


def make_output(ns):
    """output.build_dataset (output.py:47-146) through the xarray stand-in:
    the per-trace products it computes over every facet -- nadir twtt from
    the horizontally nearest facet, first in-window arrival -- with an
    identity frame so first_return_lat/lon name the facet's x, y."""
    import types
    xrshim.install()
    sys.modules["soundersim"].__version__ = "reference"
    out_mod = refload.importlib.import_module("soundersim.output")
    surf = grid_scene(ns.Facets, 40, 25.0, 0.0, 1.5, seed=61,
                      slope=(0.02, -0.03))
    pos, _ = track(12, 900.0, 30.0)
    pos = np.vstack([pos, [[60000.0, 0.0, 900.0]]])   # nothing in window
    T = len(pos)
    r = np.linalg.norm(pos[:12, None, :] - surf.centers[None], axis=-1)
    t0 = 2 * (r.min() + 3.0) / C
    dt, n_s = 1.0 / 60e6, 64
    radar = types.SimpleNamespace(
        c=C, t0=t0, dt=dt, f0=60e6, wavelength=C / 60e6,
        waveform=types.SimpleNamespace(kind="delta"))
    cfg = types.SimpleNamespace(radar=radar, mode="incoherent",
                                model_dump_json=lambda: "{}")
    scene = types.SimpleNamespace(nav_llh=pos, name="golden", crs="local",
                                  params={})
    frame = types.SimpleNamespace(lat0=0.0, lon0=0.0, h0=0.0,
                                  local_to_llh=lambda enu: np.asarray(enu))
    ds = out_mod.build_dataset(
        np.zeros((T, n_s), np.float32), np.zeros(T, np.float32),
        scene=scene, frame=frame, facets=surf,
        track=types.SimpleNamespace(positions=pos), sim_config=cfg)
    out = facet_dict("surf", surf)
    out.update(pos=pos, t0=t0, dt=dt, n_samples=n_s)
    for k in ("nadir_twtt", "first_return_twtt", "first_return_lat",
              "first_return_lon"):
        out[k] = np.asarray(ds[k].values)
    return out


def main():
    only = None
    args = [a for a in sys.argv[1:]]
    if args and args[0] == "--only":
        only = set(args[1].split(","))
        args = args[2:]
    if args:
        os.environ["SOUNDERSIM_REF"] = args[0]
    ns = refload.load()
    for name, fn in (("primitives", make_primitives), ("antenna", make_antenna),
                     ("coherent", make_coherent),
                     ("refracted", make_refracted),
                     ("waveform", make_waveform),
                     ("incoherent", make_incoherent),
                     ("focus", make_focus),
                     ("scene", make_scene),
                     ("output", make_output)):
        if only is not None and name not in only:
            continue
        data = fn(ns)
        path = os.path.join(HERE, f"{name}.npz")
        np.savez_compressed(path, **data)
        print(f"wrote {path} ({os.path.getsize(path) / 1024:.0f} KB)")


if __name__ == "__main__":
    main()
