"""GPU parity of the refracted multilayer kernel against the float64 oracle
on the reference's own golden cases (sequential / joint / padded joint /
incoherent / full feature set), both precisions.

FP64 form: <= 1e-9 of the oracle's peak per bin (float64 rounding only; the
facet lookups and bins are the same integer decisions). Split form: relative
L2 <= 1e-4, phase <= 1e-3 rad, power <= 0.01 dB above -60 dB of the peak.
"""

import numpy as np
import pytest

from oracle import refracted as oref
from tests.test_oracle_golden import RE_CASES, refracted_case
from tests.util import field_errors

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("case", RE_CASES)
def test_refracted_fp64_vs_oracle(golden, case):
    from radar_sounder_simulator_gb300.multilayer import refracted_cluttergram
    g = golden("refracted")
    pos, uct, tgt, crossed, e, a, kw = refracted_case(g, case)
    ref, ref_drop = oref.refracted_cluttergram(pos, uct, tgt, crossed, e, a,
                                               **kw)
    odt = np.complex128 if kw["mode"] == "coherent" else np.float64
    got, drop = refracted_cluttergram(pos, uct, tgt, crossed, e, a, **kw,
                                      precision="fp64", out_dtype=odt)
    assert got.shape == ref.shape
    scale = np.abs(ref).max()
    assert scale > 0
    assert np.abs(got - ref).max() <= 1e-9 * scale
    pw = scale ** 2 if kw["mode"] == "coherent" else scale
    np.testing.assert_allclose(drop, ref_drop, rtol=1e-5, atol=1e-9 * pw)


@pytest.mark.parametrize("case", RE_CASES)
def test_refracted_split_vs_oracle(golden, case):
    from radar_sounder_simulator_gb300.multilayer import refracted_cluttergram
    g = golden("refracted")
    pos, uct, tgt, crossed, e, a, kw = refracted_case(g, case)
    ref, ref_drop = oref.refracted_cluttergram(pos, uct, tgt, crossed, e, a,
                                               **kw)
    odt = np.complex128 if kw["mode"] == "coherent" else np.float64
    got, drop = refracted_cluttergram(pos, uct, tgt, crossed, e, a, **kw,
                                      precision="split", out_dtype=odt)
    if kw["mode"] == "coherent":
        err = field_errors(got, ref)
        assert err["rel_l2"] <= 1e-4, err
        assert err["phase_rad"] <= 1e-3, err
        assert err["power_db"] <= 0.01, err
        pw = np.abs(ref).max() ** 2
    else:
        keep = ref > ref.max() * 1e-6
        db = np.abs(10 * np.log10(got[keep] / ref[keep]))
        assert db.max() <= 0.01
        pw = ref.max()
    np.testing.assert_allclose(drop, ref_drop, rtol=1e-3, atol=1e-6 * pw)
