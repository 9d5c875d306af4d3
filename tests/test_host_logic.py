"""Host-side logic of the drop-in modules, checked without a GPU: the
regrouping of facets inside culling blocks, the focused-SAR track helpers
and Doppler guard, and the scene lattice and transform handling -- each
against the oracle or the reference's fixtures."""

import warnings

import numpy as np
import pytest

from oracle import processing as oproc
from oracle import scene as oscene
from radar_sounder_simulator_gb300 import processing as gproc
from radar_sounder_simulator_gb300 import scene as gscene
from radar_sounder_simulator_gb300.geometry import (cull_plan,
                                                    group_within_blocks)

C = 299792458.0


def test_regrouping_keeps_blocks_and_sorts_inside(golden):
    g = golden("coherent")
    plan = cull_plan(g["pos"], g["surf_centers"], t0=2 * 1400.0 / C,
                     dt=1e-8, n_samples=64, c=C, block_size=64,
                     target_pairs=1 << 12)
    key = np.random.default_rng(1).lognormal(0, 1, len(g["surf_centers"]))
    new = group_within_blocks(plan, key)
    assert sorted(new.order) == sorted(plan.order)
    np.testing.assert_array_equal(new.off, plan.off)
    for b in range(0, len(plan.order), 64):
        blk = new.order[b:b + 64]
        assert set(blk) == set(plan.order[b:b + 64])
        assert np.all(np.diff(key[blk]) >= 0)


def test_focus_track_helpers_match_oracle(golden):
    g = golden("focus")
    np.testing.assert_array_equal(gproc.along_track(g["pos"]),
                                  oproc.along_track(g["pos"]))
    assert gproc.mean_spacing(g["pos"]) == oproc.mean_spacing(g["pos"])
    sp = gproc.mean_spacing(g["pos"])
    r = C * g["twtt"].min() / 2
    with warnings.catch_warnings(record=True) as w:
        warnings.simplefilter("always")
        gproc.doppler_guard(sp, float(g["wavelength"]), 250.0, r, "x")
        gproc.doppler_guard(sp, float(g["wavelength"]), 96.0, r, "x")
    assert len(w) == 1 and "alias in Doppler" in str(w[0].message)


def test_scene_lattice_and_transform_helpers():
    for n, step, origin in ((40, 1.0, 0.0), (40, 2.0, 3.0), (22, 0.4, 5.0)):
        a, ka = gscene.lattice_axis(n, step, origin)
        b, kb = oscene.lattice_axis(n, step, origin)
        np.testing.assert_array_equal(a, b)
        np.testing.assert_array_equal(ka, kb)
    with pytest.raises(ValueError):
        gscene.lattice_axis(2, 5.0, 0.0)

    class Aff:
        a, b, c, d, e, f = 25.0, 0.0, 1000.0, 0.0, -25.0, 5000.0
    assert gscene._transform6(Aff()) == (25.0, 0.0, 1000.0, 0.0, -25.0,
                                         5000.0)
    with pytest.raises(ValueError):
        gscene._transform6((1.0, 2.0))


def test_local_frame_matches_oracle():
    fr = gscene.LocalFrame(75.0, -40.0, 120.0)
    of = oscene.LocalFrame(75.0, -40.0, 120.0)
    np.testing.assert_allclose(fr.origin_ecef, of.origin_ecef, rtol=0,
                               atol=1e-9)
    np.testing.assert_allclose(fr.R, of.R, atol=1e-15)
    x = np.array([[1000.0, -2000.0, 50.0]])
    np.testing.assert_allclose(fr.local_to_ecef(x), of.local_to_ecef(x),
                               atol=1e-8)


def test_series_length_matches_reference(golden):
    """The series length the benchmark scenes pick follows the reference's
    n_terms_for (roughness.py:189-196), checked against its outputs."""
    from radar_sounder_simulator_gb300 import scenes
    g = golden("primitives")
    assert [scenes.n_terms_for(x) for x in g["nterms_x"]] == list(
        g["nterms"])
