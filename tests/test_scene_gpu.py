"""Scene assembly on the GPU (ss_scene_vertices, ss_facets_from_vertices,
ss_speckle_phasors_keyed, ss_offset_centers through the drop-in functions)
against the reference's outputs and the oracle.

Tolerances: the lattice, bilinear weights, affine map, corner rule and hash
follow the reference's float64 chain with round-to-nearest operations, so
facets equal the golden ones bit for bit. Keyed phasors use CUDA's float64
log/sin/cos (within an ulp of the C library's); after rounding to complex64
they equal the reference's except, rarely, by one float32 ulp. The polar
stereographic and WGS84 chain is compared with the float64 oracle to 1 mm
(positions 10^6 m from the origin of ECEF: ~1e-10 relative)."""

import types

import numpy as np
import pytest

from oracle import scene as osc
from radar_sounder_simulator_gb300 import scene as gsc

pytestmark = pytest.mark.gpu
SEEDS = {"s31": (3, 1), "s7": 7, "s11_1002": (11, 1002)}
FIELDS = ("centers", "normals", "areas", "e1", "e2", "cell", "phase_keys")


@pytest.mark.parametrize("name", sorted(SEEDS))
def test_keyed_phasors_match_reference(golden, name):
    g = golden("scene")
    ph = gsc.speckle_phasors_for_keys(g["keys"], SEEDS[name])
    ref = g[f"phasors_{name}"]
    assert ph.dtype == np.complex64 and ph.shape == ref.shape
    diff = ph != ref
    assert diff.sum() <= max(1, len(ref) // 10000)
    if diff.any():
        assert np.abs(ph - ref).max() <= 2.5e-7 * np.abs(ref).max()


def test_keyed_phasors_crop_and_order_invariant():
    """The reference's property (tests/test_roughness.py:168-179): a
    subset in any order gets the same phasors."""
    r, c = np.meshgrid(np.arange(100, 300), np.arange(400, 500),
                       indexing="ij")
    keys = np.column_stack([r.ravel(), c.ravel()])
    ph = gsc.speckle_phasors_for_keys(keys, (3, 1))
    take = np.random.default_rng(4).permutation(len(keys))[:3000]
    np.testing.assert_array_equal(ph[take], gsc.speckle_phasors_for_keys(
        keys[take], (3, 1)))
    assert not np.array_equal(ph[take], gsc.speckle_phasors_for_keys(
        keys[take], (3, 2)))
    assert np.mean(np.abs(ph) ** 2) == pytest.approx(1.0, abs=0.03)
    with pytest.raises(ValueError):
        gsc.speckle_phasors_for_keys(keys[:, :1], 1)


@pytest.mark.parametrize("name", ["native", "stride", "fine", "crop"])
def test_build_facets_bit_exact(golden, name):
    g = golden("scene")
    sp = float(g[f"bf_{name}_spacing"])
    frame = types.SimpleNamespace(origin_ecef=g["origin"], R=np.eye(3))
    f = gsc.build_facets(g["dem"], tuple(g["transform"]), None, frame,
                         spacing=None if np.isnan(sp) else sp,
                         grid_origin=tuple(g[f"bf_{name}_origin"]))
    for k in FIELDS:
        np.testing.assert_array_equal(getattr(f, k), g[f"bf_{name}_{k}"],
                                      err_msg=k)
    assert f.grid_shape == tuple(g[f"bf_{name}_grid"])


@pytest.mark.parametrize("crs,lat0,lon0", [("EPSG:3413", 75.0, -40.0),
                                           ("EPSG:3031", -78.0, 110.0)])
def test_polar_dem_to_local_facets(crs, lat0, lon0):
    """A DEM on a polar stereographic grid around (lat0, lon0) through the
    whole chain, against the oracle's projection and frame."""
    rng = np.random.default_rng(8)
    cx, cy = osc.polar_stereo_forward(lon0, lat0, crs)
    posting = 50.0
    ny, nx = 60, 50
    tr = (posting, 0.0, cx - nx * posting / 2, 0.0, -posting,
          cy + ny * posting / 2)
    dem = 700.0 + 30.0 * rng.standard_normal((ny, nx))
    frame = gsc.LocalFrame(lat0, lon0, 0.0)
    ofr = osc.LocalFrame(lat0, lon0, 0.0)

    def to_ecef(E, N, h):
        lo, la = osc.polar_stereo_inverse(E, N, crs)
        return osc.geodetic_to_ecef(la, lo, h)
    ref = osc.build_facets(dem, tr, to_ecef, ofr.ecef_to_local,
                           spacing=100.0)
    f = gsc.build_facets(dem, tr, crs, frame, spacing=100.0)
    assert np.abs(f.centers - ref["centers"]).max() < 1e-3
    assert np.abs(f.normals - ref["normals"]).max() < 1e-9
    np.testing.assert_allclose(f.areas, ref["areas"], rtol=1e-9)
    np.testing.assert_array_equal(f.phase_keys, ref["phase_keys"])
    # facets sit near the frame's tangent plane and face up
    assert np.abs(f.centers[:, 2]).max() < 2000.0
    assert (f.normals[:, 2] > 0.0).all()


def test_offset_facets_along_up():
    frame = gsc.LocalFrame(75.0, -40.0, 0.0)
    ofr = osc.LocalFrame(75.0, -40.0, 0.0)
    rng = np.random.default_rng(9)
    n = 4000
    cen = np.column_stack([rng.uniform(-3e4, 3e4, n),
                           rng.uniform(-3e4, 3e4, n), rng.normal(0, 50, n)])
    f = gsc.Facets(cen, np.tile([0, 0, 1.0], (n, 1)), np.ones(n),
                   np.zeros((n, 3)), np.zeros((n, 3)),
                   np.zeros((n, 2), np.int64), (1, n), None)
    g = gsc.offset_facets(f, frame, -250.0)
    ref = osc.offset_centers(cen, ofr, -250.0)
    assert np.abs(g.centers - ref).max() < 1e-6
    np.testing.assert_array_equal(g.normals, f.normals)


def test_unknown_crs_is_refused():
    frame = types.SimpleNamespace(origin_ecef=np.zeros(3), R=np.eye(3))
    with pytest.raises(ValueError):
        gsc.build_facets(np.zeros((4, 4)), (1, 0, 0, 0, -1, 0), "EPSG:32633",
                         frame)
