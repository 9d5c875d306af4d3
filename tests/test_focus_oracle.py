"""The focused-SAR oracle (float64 restatement of processing.py:262-348)
against the reference's own outputs (tests/golden/focus.npz, made by
tests/golden/make_golden.py from the reference source through a minimal
xarray stand-in): bit-identical on all three cases."""

import numpy as np
import pytest

from oracle import processing as op


@pytest.mark.parametrize("name,window", [("hann", "hann"), ("rect", "none"),
                                         ("wide", "hann")])
def test_oracle_matches_reference(golden, name, window):
    g = golden("focus")
    out, pw = op.focused_sar(g["field"], g["twtt"], g["pos"],
                             float(g["wavelength"]),
                             float(g[f"focus_{name}_aperture"]), window)
    np.testing.assert_array_equal(out.astype(np.complex64),
                                  g[f"focus_{name}_field"])
    np.testing.assert_array_equal(pw, g[f"focus_{name}_power"])


def test_point_target_focuses_at_its_trace(golden):
    """The strongest target (amplitude 1 under trace T/2) focuses to a peak
    well above its unfocused single-trace amplitude."""
    g = golden("focus")
    f = g["focus_hann_field"]
    t, b = np.unravel_index(np.abs(f).argmax(), f.shape)
    assert abs(t - 32) <= 1
    assert np.abs(f).max() > 4 * np.abs(g["field"]).max() / 1.5


def test_doppler_guard_fires_for_the_wide_aperture(golden):
    g = golden("focus")
    sp = op.mean_spacing(g["pos"])
    r = 299792458.0 * g["twtt"].min() / 2
    assert op.doppler_guard(sp, float(g["wavelength"]), 250.0, r)
    assert not op.doppler_guard(sp, float(g["wavelength"]), 96.0, r)
