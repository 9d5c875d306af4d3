"""The multi-core C++ float64 restatement (the timed CPU baseline) against
the NumPy oracle and the reference's own golden outputs.

Per pair it restates the oracle's formulas; both are float64, so the fields
agree to float64 rounding (<= 1e-10 of the peak; the joint solve's 2x2
products are summed in a different order) and the occupied bins are the
same. Against the reference's fixtures (float64 path, complex64
accumulation) the bound is the fixtures' own 2e-6 of the peak.
"""

import numpy as np
import pytest

from oracle import cpu_ref, lpa
from oracle import refracted as oref
from tests.test_oracle_golden import refracted_case
from tests.util import facets_from

C = 299792458.0

CASES = ["seq1", "seq2", "joint2", "joint_pad"]


@pytest.fixture(scope="module", autouse=True)
def built():
    cpu_ref.build()


@pytest.mark.parametrize("case", CASES)
def test_refracted_vs_oracle_and_reference(golden, case):
    g = golden("refracted")
    pos, uct, tgt, crossed, e, a, kw = refracted_case(g, case)
    want, want_drop = oref.refracted_cluttergram(pos, uct, tgt, crossed, e, a,
                                                 **kw)
    got, drop = cpu_ref.refracted_cluttergram(pos, uct, tgt, crossed, e, a,
                                              **kw)
    scale = np.abs(want).max()
    assert scale > 0
    assert np.array_equal(got != 0, want != 0)
    assert np.abs(got - want).max() <= 1e-10 * scale
    np.testing.assert_allclose(drop, want_drop, rtol=1e-9,
                               atol=1e-12 * scale ** 2)
    ref = g[f"re_{case}_out"]
    assert np.abs(got - ref).max() <= 2e-6 * np.abs(ref).max()


def test_coherent_vs_oracle(golden):
    g = golden("coherent")
    f = facets_from(g, "surf")
    kw = dict(k=float(g["k"]), gamma=-0.279, t0=float(g["t0"]),
              dt=float(g["dt"]), n_samples=int(g["n_samples"]), c=C)
    args = (g["pos"], g["uct"], f.centers, f.normals, f.areas, f.e1, f.e2)
    want, want_drop = lpa.coherent_cluttergram(*args, **kw)
    got, drop = cpu_ref.coherent_cluttergram(*args, **kw)
    scale = np.abs(want).max()
    assert np.array_equal(got != 0, want != 0)
    assert np.abs(got - want).max() <= 1e-12 * scale
    np.testing.assert_allclose(drop, want_drop, rtol=1e-9,
                               atol=1e-14 * scale ** 2)


def test_per_facet_gamma(golden):
    g = golden("coherent")
    f = facets_from(g, "surf")
    kw = dict(k=float(g["k"]), gamma=g["gamma_facet"], t0=float(g["t0"]),
              dt=float(g["dt"]), n_samples=int(g["n_samples"]), c=C)
    args = (g["pos"], g["uct"], f.centers, f.normals, f.areas, f.e1, f.e2)
    want, _ = lpa.coherent_cluttergram(*args, **kw)
    got, _ = cpu_ref.coherent_cluttergram(*args, **kw)
    assert np.abs(got - want).max() <= 1e-12 * np.abs(want).max()


def test_refuses_unrestated_options(golden):
    g = golden("refracted")
    pos, uct, tgt, crossed, e, a, kw = refracted_case(g, "full")
    with pytest.raises(NotImplementedError):
        cpu_ref.refracted_cluttergram(pos, uct, tgt, crossed, e, a, **kw)


def test_thread_count_does_not_change_results(golden):
    """Each trace's row is summed in facet order by one thread, so one
    thread and all of them give the same bits."""
    g = golden("refracted")
    pos, uct, tgt, crossed, e, a, kw = refracted_case(g, "joint2")
    n = cpu_ref.threads()
    try:
        cpu_ref.set_threads(1)
        one, d1 = cpu_ref.refracted_cluttergram(pos, uct, tgt, crossed, e, a,
                                                **kw)
    finally:
        cpu_ref.set_threads(n)
    many, dn = cpu_ref.refracted_cluttergram(pos, uct, tgt, crossed, e, a,
                                             **kw)
    np.testing.assert_array_equal(one, many)
    np.testing.assert_array_equal(d1, dn)
