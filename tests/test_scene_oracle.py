"""Scene-assembly oracle against the reference's own outputs
(tests/golden/scene.npz, made through an identity pyproj stand-in):
keyed speckle phasors and build_facets (lattice, bilinear resampling,
affine map, corner rule, cells, phase keys) bit for bit; and the WGS84 /
polar stereographic formulas, which have no reference run here, by round
trips and closed-form properties."""

import numpy as np
import pytest

from oracle import scene as osc

SEEDS = {"s31": (3, 1), "s7": 7, "s11_1002": (11, 1002)}
CASES = ("native", "stride", "fine", "crop")
FIELDS = ("centers", "normals", "areas", "e1", "e2", "cell", "phase_keys")


@pytest.mark.parametrize("name", sorted(SEEDS))
def test_keyed_phasors_bit_exact(golden, name):
    g = golden("scene")
    ph = osc.speckle_phasors_for_keys(g["keys"], SEEDS[name])
    np.testing.assert_array_equal(ph, g[f"phasors_{name}"])


def test_keyed_phasors_reject_bad_keys():
    with pytest.raises(ValueError):
        osc.speckle_phasors_for_keys(np.zeros((4, 3), np.int64), 1)


@pytest.mark.parametrize("name", CASES)
def test_build_facets_bit_exact(golden, name):
    g = golden("scene")
    sp = float(g[f"bf_{name}_spacing"])
    f = osc.build_facets(
        g["dem"], tuple(g["transform"]), lambda E, N, h: (E, N, h),
        lambda x: np.atleast_2d(x) - g["origin"],
        spacing=None if np.isnan(sp) else sp,
        grid_origin=tuple(g[f"bf_{name}_origin"]))
    for k in FIELDS:
        np.testing.assert_array_equal(f[k], g[f"bf_{name}_{k}"], err_msg=k)
    assert tuple(f["grid_shape"]) == tuple(g[f"bf_{name}_grid"])


@pytest.mark.parametrize("crs", ["EPSG:3413", "EPSG:3031"])
def test_polar_stereographic_round_trip(crs):
    rng = np.random.default_rng(1)
    lat0 = 75.0 if crs == "EPSG:3413" else -78.0
    lat = lat0 + rng.uniform(-8, 8, 500)
    lon = rng.uniform(-180, 180, 500)
    x, y = osc.polar_stereo_forward(lon, lat, crs)
    lo, la = osc.polar_stereo_inverse(x, y, crs)
    assert np.abs(la - lat).max() < 1e-10
    dlon = (lo - lon + 180.0) % 360.0 - 180.0
    assert np.abs(dlon).max() < 1e-9
    # the pole is the projection origin; the scale is 1 on the standard
    # parallel (projected length of 1e-6 rad of longitude there)
    px, py = osc.polar_stereo_forward(0.0, 90.0 if lat0 > 0 else -90.0, crs)
    assert abs(px) < 1e-6 and abs(py) < 1e-6
    lat_c = osc.POLAR[crs][0]
    xa, ya = osc.polar_stereo_forward(10.0, lat_c, crs)
    xb, yb = osc.polar_stereo_forward(10.0 + np.degrees(1e-6), lat_c, crs)
    phi = np.radians(lat_c)
    n = osc.WGS84_A / np.sqrt(1 - osc.WGS84_E2 * np.sin(phi) ** 2)
    assert np.hypot(xb - xa, yb - ya) == pytest.approx(
        n * np.cos(phi) * 1e-6, rel=1e-6)


def test_geodetic_round_trip_and_frame():
    rng = np.random.default_rng(2)
    lat = rng.uniform(-89, 89, 200)
    lon = rng.uniform(-180, 180, 200)
    h = rng.uniform(-500, 9000, 200)
    x, y, z = osc.geodetic_to_ecef(lat, lon, h)
    la, lo, hh = osc.ecef_to_geodetic(x, y, z)
    assert np.abs(la - lat).max() < 1e-10
    assert np.abs(hh - h).max() < 1e-6
    fr = osc.LocalFrame(75.0, -40.0, 100.0)
    assert np.abs(fr.ecef_to_local(fr.origin_ecef)).max() < 1e-9
    np.testing.assert_allclose(fr.up_at(np.zeros((1, 3)))[0], [0, 0, 1],
                               atol=1e-12)


def test_offset_moves_along_ellipsoidal_up():
    fr = osc.LocalFrame(75.0, -40.0, 0.0)
    rng = np.random.default_rng(3)
    enu = np.column_stack([rng.uniform(-2e4, 2e4, 50),
                           rng.uniform(-2e4, 2e4, 50), np.zeros(50)])
    moved = osc.offset_centers(enu, fr, -300.0)
    x0 = fr.local_to_ecef(enu)
    x1 = fr.local_to_ecef(moved)
    h0 = osc.ecef_to_geodetic(x0[:, 0], x0[:, 1], x0[:, 2])[2]
    h1 = osc.ecef_to_geodetic(x1[:, 0], x1[:, 1], x1[:, 2])[2]
    np.testing.assert_allclose(h1 - h0, -300.0, atol=1e-6)
