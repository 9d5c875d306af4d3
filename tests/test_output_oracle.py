"""Per-trace output products of the oracle against the reference's own
build_dataset (tests/golden/output.npz, through the xarray stand-in and an
identity frame): nadir twtt, first-return twtt and the first-return facet,
bit for bit, including a trace with no facet in the window (+inf)."""

import numpy as np

from oracle import output as oo

C = 299792458.0


def test_products_match_reference(golden):
    g = golden("output")
    nt, ni, ft, fi = oo.trace_products(g["surf_centers"], g["pos"],
                                       float(g["t0"]), float(g["dt"]),
                                       int(g["n_samples"]), C)
    np.testing.assert_array_equal(nt, g["nadir_twtt"])
    np.testing.assert_array_equal(ft, g["first_return_twtt"])
    c = g["surf_centers"]
    np.testing.assert_array_equal(c[fi, 0], g["first_return_lat"])
    np.testing.assert_array_equal(c[fi, 1], g["first_return_lon"])
    assert np.isinf(ft[-1]) and fi[-1] == 0
    assert np.isfinite(ft[:-1]).all()
