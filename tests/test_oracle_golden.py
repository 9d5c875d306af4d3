"""Pin the float64 oracle to the reference's own outputs (golden fixtures
written by tests/golden/make_golden.py from the unmodified reference source).

Tolerances: float64 formula fixtures agree to ~1e-12; the reference's surface
cluttergram runs in float32 by design (kernels/coherent.py:298-307), so the
oracle is checked against it at the reference's own f32-vs-f64 gate
(tests/test_coherent_kernel.py:195-199: 5e-4 of peak); the refracted
reference is float64 with complex64 accumulation (multilayer.py:566-569).
"""

import numpy as np
import pytest

from oracle import antenna, geometry, lpa, multifreq, refracted, refraction
from oracle import roughness, waveform
from tests.util import facets_from

C = 299792458.0


def test_faddeeva_and_dphi(golden):
    g = golden("primitives")
    np.testing.assert_allclose(roughness.faddeeva(g["fad_z"]), g["fad_w"],
                               rtol=1e-13, atol=0)
    for tag, kw in (("full", {}), ("area", dict(area_only=True)),
                    ("exp", dict(area_only=True, acf="exponential"))):
        got = roughness.d_phi(0.31, 4.0, g["dp_K"], g["dp_A0"], g["dp_B0"],
                              g["dp_Lx"], g["dp_Ly"], n_terms=120, **kw)
        np.testing.assert_allclose(got, g[f"dp_{tag}"], rtol=1e-11,
                                   atol=1e-12 * np.abs(g[f"dp_{tag}"]).max())
    assert [roughness.n_terms_for(x) for x in g["nterms_x"]] == list(
        g["nterms"])
    np.testing.assert_array_equal(roughness.speckle_phasors(64, (0, 0)),
                                  g["phasors_0_0"])
    np.testing.assert_array_equal(roughness.speckle_phasors(64, (7, 3)),
                                  g["phasors_7_3"])


def test_snell_and_joint(golden):
    g = golden("primitives")
    r = refraction.snell(g["sn_p"], g["sn_q"], g["sn_o"], g["sn_n"], 1.0,
                         1.78, 25, component=False)
    np.testing.assert_allclose(r.x, g["sn_x"], rtol=0, atol=1e-9)
    np.testing.assert_allclose(r.s1, g["sn_s1"], rtol=1e-13)
    np.testing.assert_array_equal(r.valid, g["sn_valid"])
    q = g["jt_q"]
    o = np.broadcast_to(g["jt_o"][:, None, :], (3, len(q), 3))
    n = np.broadcast_to(g["jt_n"][:, None, :], (3, len(q), 3))
    j = refraction.joint_crossings(g["sn_p"], q, o, n, g["jt_media"])
    np.testing.assert_allclose(j.x, g["jt_x"], rtol=0, atol=1e-8)
    np.testing.assert_allclose(j.s, g["jt_s"], rtol=1e-12)
    np.testing.assert_array_equal(j.valid, g["jt_valid"])
    ch = refraction.sequential_chain(g["sn_p"], q, o, n, g["jt_media"])
    np.testing.assert_allclose(ch.x, g["ch_x"], rtol=0, atol=1e-9)
    np.testing.assert_array_equal(ch.valid, g["ch_valid"])


@pytest.mark.parametrize("name", ["dipole", "dipole_ct", "array", "array_el",
                                  "array_tapered", "finite_dipole",
                                  "tabulated"])
def test_antenna_gains(golden, name):
    g = golden("antenna")
    got = antenna.gain(str(g[f"ant_{name}_kind"]), g["ant_dhat"],
                       g[f"ant_{name}_pv"], g[f"ant_{name}_pa"],
                       g[f"ant_{name}_pb"])
    np.testing.assert_allclose(got, g[f"ant_{name}_g"], rtol=1e-12,
                               atol=1e-14)


def test_pair_formulas(golden):
    g = golden("coherent")
    f = facets_from(g, "surf")
    p = g["pos"][3]
    c, r = lpa.lpa_field(p, f.centers, f.normals, f.areas, f.e1, f.e2,
                         float(g["k"]), -0.279)
    np.testing.assert_allclose(r, g["pair_r"], rtol=1e-15)
    np.testing.assert_allclose(c, g["pair_contrib"], rtol=1e-10,
                               atol=1e-12 * np.abs(c).max())
    ct, _ = lpa.lpa_field(p, f.centers, f.normals, f.areas, f.e1, f.e2,
                          float(g["k"]), -0.279, taper_s=0.05)
    np.testing.assert_allclose(ct, g["pair_contrib_taper"], rtol=1e-10,
                               atol=1e-12 * np.abs(ct).max())
    ph = g["phasors"].astype(np.complex128)
    for tag, kw in (("full", {}), ("area", dict(area_only=True)),
                    ("exp", dict(area_only=True, acf="exponential"))):
        cr, _ = lpa.rough_lpa_field(
            p, f.centers, f.normals, f.areas, f.e1, f.e2, float(g["k"]),
            -0.279, 0.3, 4.0, ph, 40,
            taper_s=0.05 if tag != "full" else None, **kw)
        ref = g[f"pair_rough_{tag}"]
        np.testing.assert_allclose(cr, ref, rtol=1e-9,
                                   atol=1e-12 * np.abs(ref).max())


def test_culling_bit_exact(golden):
    g = golden("coherent")
    f = facets_from(g, "surf")
    order, s_t, s_sorted = geometry.along_track_order(g["pos"], f.centers)
    np.testing.assert_array_equal(order, g["cull_order"])
    reach = geometry.window_reach_m(float(g["t0"]), float(g["dt"]),
                                    int(g["n_samples"]), C)
    assert reach == float(g["cull_reach"])
    off, n_win = geometry.block_windows(s_sorted, s_t, reach * 0.35, 64,
                                        -(-len(order) // 64))
    np.testing.assert_array_equal(off, g["cull_off"])
    assert n_win == int(g["cull_nwin"])
    assert [geometry.auto_block_size(t, 1 << 19)
            for t in (1, 12, 256, 1024, 5000)] == list(g["auto_bs"])


CO_CASES = ["smooth", "split", "interp", "blocks", "gammaf", "array", "rough",
            "rough_exp"]


@pytest.mark.parametrize("case", CO_CASES)
def test_coherent_vs_reference_f32(golden, case):
    g = golden("coherent")
    f = facets_from(g, "surf")
    kw = dict(k=float(g["k"]), gamma=-0.279, t0=float(g["t0"]),
              dt=float(g["dt"]), n_samples=int(g["n_samples"]), c=C)
    ph = g["phasors"]
    extra = {
        "smooth": {}, "split": dict(split_sides=True),
        "interp": dict(interp_bins=True), "blocks": dict(block_size=96),
        "gammaf": dict(gamma=g["gamma_facet"]),
        "array": dict(pattern=("array", g["ant_pv"], g["ant_pa"],
                               g["ant_pb"])),
        "rough": dict(roughness=(0.3, 4.0, ph, 40)),
        "rough_exp": dict(roughness=(0.3, 4.0, ph, 40, "exponential"),
                          taper_s=0.05, d_phi_area=True),
    }[case]
    fld, drp = lpa.coherent_cluttergram(g["pos"], g["uct"], f.centers,
                                        f.normals, f.areas, f.e1, f.e2,
                                        **{**kw, **extra})
    ref = g[f"co_{case}_field"]
    assert fld.shape == ref.shape
    # the reference kernel is float32 (its own gate: 5e-4 of peak)
    assert np.abs(fld - ref).max() / np.abs(ref).max() < 5e-4
    np.testing.assert_allclose(drp, g[f"co_{case}_dropped"], rtol=2e-3,
                               atol=1e-6 * np.abs(ref).max() ** 2)


RE_CASES = ["seq1", "seq2", "joint2", "joint_pad", "incoh", "full",
            "full_joint"]


def refracted_case(g, case):
    surf, h1, bed = (facets_from(g, t) for t in ("surf", "h1", "bed"))
    eps = list(g["eps"])
    att = list(g["att"])
    k0 = float(g["k0"])
    pat = ("dipole", g["ant_pv"], np.float64(0.0), np.float64(0.0))
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
                 dict(mode="coherent", gamma=g["gamma_facet"], k0=k0,
                      roughness=(0.2, 3.0, g["phasors"], 30, "exponential"),
                      crossed_sigma=[0.1, 0.02], taper_s=0.05,
                      d_phi_area=True,
                      diffuse=(g["dif_amp"], g["dif_phasors"], 1.5),
                      pattern=pat, split_sides=True)),
        "full_joint": (bed, two, eps, att,
                       dict(mode="coherent", gamma=g["gamma_facet"], k0=k0,
                            roughness=(0.2, 3.0, g["phasors"], 30),
                            crossed_sigma=[0.1, 0.02], refraction="joint",
                            pattern=pat)),
    }
    tgt, crossed, e, a, kw = cases[case]
    base = dict(t0=float(g["t0"]), dt=float(g["dt"]),
                n_samples=int(g["n_samples"]), c=C)
    return g["pos"], g["uct"], tgt, crossed, e, a, {**base, **kw}


@pytest.mark.parametrize("case", RE_CASES)
def test_refracted_vs_reference(golden, case):
    g = golden("refracted")
    pos, uct, tgt, crossed, e, a, kw = refracted_case(g, case)
    out, drp = refracted.refracted_cluttergram(pos, uct, tgt, crossed, e, a,
                                               **kw)
    ref = g[f"re_{case}_out"]
    assert out.shape == ref.shape
    scale = np.abs(ref).max()
    assert scale > 0
    # reference: float64 path, complex64/float32 accumulation
    assert np.abs(out - ref).max() / scale < 2e-6
    np.testing.assert_allclose(drp, g[f"re_{case}_dropped"], rtol=1e-5,
                               atol=1e-7 * scale ** (2 if kw["mode"] ==
                                                     "coherent" else 1))


def test_waveform_and_multifreq(golden):
    g = golden("waveform")
    for w in ("none", "hann", "hamming"):
        p, m = waveform.compressed_pulse(15e6, 20e-6, 1.0 / 30e6, w)
        assert m == int(g[f"pulse_{w}_m"])
        np.testing.assert_allclose(p, g[f"pulse_{w}"], rtol=1e-13,
                                   atol=1e-15)
    pc, mc = waveform.compressed_pulse(15e6, 8e-6, 1.0 / 30e6, "hann",
                                       "chirp")
    assert mc == int(g["pulse_chirp_m"])
    np.testing.assert_allclose(pc, g["pulse_chirp"], rtol=0, atol=1e-9)
    y = waveform.convolve_fast_time(g["conv_in"], g["pulse_hann"],
                                    int(g["pulse_hann_m"]))
    np.testing.assert_allclose(y, g["conv_out"], rtol=0,
                               atol=1e-11 * np.abs(g["conv_out"]).max())
    f = facets_from(g, "mf")
    for tag, frz in (("full", False), ("frozen", True)):
        yy = multifreq.multifreq_profile(
            g["mf_pos"], f.centers, f.normals, f.areas, f.e1, f.e2,
            gamma=-0.28, f0=60e6, bandwidth=15e6, c=C, twtt=g["mf_twtt"],
            n_freq=64, freeze_amplitudes=frz)
        ref = g[f"mf_{tag}"]
        np.testing.assert_allclose(yy, ref, rtol=0,
                                   atol=1e-10 * np.abs(ref).max())
