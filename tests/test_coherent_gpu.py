"""GPU parity of the surface coherent kernel against the float64 oracle.

FP64 form: within 1e-9 of the oracle per bin (float64 rounding only; the
binning chain is round-to-nearest, so bins are identical). Split form: the
path tolerances -- relative L2 <= 1e-4, phase <= 1e-3 rad and power
<= 0.01 dB for bins above -60 dB of the peak.
"""

import numpy as np
import pytest

from oracle import lpa
from tests.util import facets_from, field_errors

pytestmark = pytest.mark.gpu
C = 299792458.0

CASES = ["smooth", "split", "interp", "blocks", "gammaf", "array", "rough",
         "rough_exp", "rough_area", "taper"]


def case_kwargs(g, case):
    ph = g["phasors"]
    return {
        "smooth": {}, "split": dict(split_sides=True),
        "interp": dict(interp_bins=True), "blocks": dict(block_size=96),
        "gammaf": dict(gamma=g["gamma_facet"]),
        "array": dict(pattern=("array", g["ant_pv"], g["ant_pa"],
                               g["ant_pb"])),
        "rough": dict(roughness=(0.3, 4.0, ph, 40)),
        "rough_exp": dict(roughness=(0.3, 4.0, ph, 40, "exponential"),
                          taper_s=0.05, d_phi_area=True),
        "rough_area": dict(roughness=(0.3, 4.0, ph, 40), d_phi_area=True),
        "taper": dict(taper_s=0.05),
    }[case]


@pytest.fixture(scope="module")
def scene(golden):
    g = golden("coherent")
    f = facets_from(g, "surf")
    base = dict(k=float(g["k"]), gamma=-0.279, t0=float(g["t0"]),
                dt=float(g["dt"]), n_samples=int(g["n_samples"]), c=C)
    return g, f, base


@pytest.mark.parametrize("case", CASES)
def test_coherent_fp64_and_split_vs_oracle(scene, case):
    from radar_sounder_simulator_gb300.coherent import coherent_cluttergram
    g, f, base = scene
    kw = {**base, **case_kwargs(g, case)}
    args = (g["pos"], g["uct"], f.centers, f.normals, f.areas, f.e1, f.e2)
    ref, ref_drop = lpa.coherent_cluttergram(*args, **kw)
    got, drop = coherent_cluttergram(*args, **kw, precision="fp64",
                                     out_dtype=np.complex128)
    assert got.shape == ref.shape
    scale = np.abs(ref).max()
    assert np.abs(got - ref).max() <= 1e-9 * scale
    # identical occupancy: every oracle bin above 1e-12 of peak is filled
    occ = np.abs(ref) > 1e-12 * scale
    assert np.all(np.abs(got[occ]) > 0)
    np.testing.assert_allclose(drop, ref_drop, rtol=1e-5,
                               atol=1e-9 * scale ** 2)
    sp, sdrop = coherent_cluttergram(*args, **kw, precision="split",
                                     out_dtype=np.complex128)
    err = field_errors(sp, ref)
    assert err["rel_l2"] <= 1e-4, err
    assert err["phase_rad"] <= 1e-3, err
    assert err["power_db"] <= 0.01, err
    np.testing.assert_allclose(sdrop, ref_drop, rtol=1e-3,
                               atol=1e-6 * scale ** 2)


def test_default_dtypes_match_reference(scene):
    from radar_sounder_simulator_gb300.coherent import coherent_cluttergram
    g, f, base = scene
    fld, drp = coherent_cluttergram(g["pos"], g["uct"], f.centers, f.normals,
                                    f.areas, f.e1, f.e2, **base)
    assert fld.dtype == np.complex64 and drp.dtype == np.float32
    assert fld.shape == (len(g["pos"]), int(g["n_samples"]))


def test_split_is_deterministic_in_bins(scene):
    """The chunk reduction is ordered; rerunning gives the same bins."""
    from radar_sounder_simulator_gb300.coherent import coherent_cluttergram
    g, f, base = scene
    args = (g["pos"], g["uct"], f.centers, f.normals, f.areas, f.e1, f.e2)
    a, _ = coherent_cluttergram(*args, **base, precision="split")
    b, _ = coherent_cluttergram(*args, **base, precision="split")
    np.testing.assert_array_equal(a != 0, b != 0)
    np.testing.assert_allclose(a, b, rtol=0, atol=1e-6 * np.abs(a).max())
