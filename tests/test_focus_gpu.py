"""GPU focused SAR (ss_focused_sar through the drop-in focused_sar /
focus_field) against the reference's outputs and the float64 oracle.

Tolerances: the FP64 form follows the reference's float64 chain operation
by operation (round-to-nearest, same interpolation, phase and summation
order), so it matches the golden complex64 field to within one complex64
rounding (relative 1e-6 of the peak) and the oracle to 1e-12 relative L2.
The split form computes in float32 (dr without cancellation, phase reduced
modulo 2 pi): relative L2 <= 1e-4 (the path's float bound) and the
power of samples above -60 dB within 0.01 dB."""

import json

import numpy as np
import pytest

from oracle import processing as op
from radar_sounder_simulator_gb300 import processing as gp

pytestmark = pytest.mark.gpu
CASES = [("hann", "hann"), ("rect", "none"), ("wide", "hann")]


def _rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


def _db(a, b):
    p = np.abs(b) ** 2
    keep = p > 1e-6 * p.max()
    return np.abs(10 * np.log10(np.abs(a[keep]) ** 2 / p[keep])).max()


@pytest.mark.parametrize("name,window", CASES)
def test_fp64_matches_reference_golden(golden, name, window):
    g = golden("focus")
    ap = float(g[f"focus_{name}_aperture"])
    out, pw = gp.focus_field(g["field"], g["twtt"], g["pos"],
                             wavelength=float(g["wavelength"]),
                             aperture_m=ap, window=window)
    ref = g[f"focus_{name}_field"]
    assert out.dtype == np.complex64 and pw.dtype == np.float32
    peak = np.abs(ref).max()
    assert np.abs(out - ref).max() <= 1e-6 * peak
    np.testing.assert_allclose(pw, g[f"focus_{name}_power"], rtol=1e-5,
                               atol=1e-6 * peak ** 2)
    o64, _ = op.focused_sar(g["field"], g["twtt"], g["pos"],
                            float(g["wavelength"]), ap, window)
    assert _rel(out.astype(np.complex128), o64) <= 1e-6


@pytest.mark.parametrize("name,window", CASES)
def test_split_within_float_bounds(golden, name, window):
    g = golden("focus")
    ap = float(g[f"focus_{name}_aperture"])
    out, _ = gp.focus_field(g["field"], g["twtt"], g["pos"],
                            wavelength=float(g["wavelength"]), aperture_m=ap,
                            window=window, precision="split")
    o64, _ = op.focused_sar(g["field"], g["twtt"], g["pos"],
                            float(g["wavelength"]), ap, window)
    assert _rel(out, o64) <= 1e-4
    assert _db(out, o64) <= 0.01


def test_fp64_device_output_matches_oracle_tightly(golden):
    """complex128 output of the FP64 form against the float64 oracle."""
    import torch
    g = golden("focus")
    ft = torch.as_tensor(g["field"], device="cuda")
    tw = torch.as_tensor(g["twtt"], device="cuda")
    s = torch.as_tensor(gp.along_track(g["pos"]), device="cuda")
    out, _ = gp.focus_tensor(ft, tw, s, wavelength=float(g["wavelength"]),
                             aperture_m=96.0, out_dtype=torch.complex128)
    o64, _ = op.focused_sar(g["field"], g["twtt"], g["pos"],
                            float(g["wavelength"]), 96.0, "hann")
    assert _rel(out.cpu().numpy(), o64) <= 1e-12


@pytest.mark.parametrize("precision", ["fp64", "split"])
def test_longer_track_ragged_and_complex128_input(precision):
    """A track longer than one 256-trace aperture chunk, bins not a multiple
    of the CTA, complex128 input, 450 MHz (large phase corrections)."""
    rng = np.random.default_rng(44)
    T, nb, lam = 300, 333, 299792458.0 / 450e6
    x = np.cumsum(rng.uniform(0.1, 0.25, T))
    pos = np.column_stack([x, np.zeros(T), np.full(T, 500.0)])
    dt = 1.0 / 60e6
    twtt = 2 * 440.0 / 299792458.0 + np.arange(nb) * dt
    F = rng.standard_normal((T, nb)) + 1j * rng.standard_normal((T, nb))
    out, _ = gp.focus_field(F, twtt, pos, wavelength=lam, aperture_m=40.0,
                            precision=precision)
    o64, _ = op.focused_sar(F, twtt, pos, lam, 40.0, "hann")
    tol = 1e-6 if precision == "fp64" else 1e-4
    assert _rel(out, o64) <= tol


@pytest.mark.parametrize("precision", ["fp64", "split"])
def test_tiny_and_empty_apertures(precision):
    """An aperture below the trace spacing keeps only the trace itself; a
    negative one keeps nothing (zeros), as the reference's predicate
    does."""
    g = np.random.default_rng(3)
    T, nb = 10, 40
    pos = np.column_stack([np.arange(T) * 5.0, np.zeros(T), np.full(T, 300.)])
    twtt = 2 * 290.0 / 299792458.0 + np.arange(nb) * 1e-8
    F = (g.standard_normal((T, nb)) + 1j * g.standard_normal((T, nb))
         ).astype(np.complex64)
    for ap in (1.0, -1.0):
        out, _ = gp.focus_field(F, twtt, pos, wavelength=2.0, aperture_m=ap,
                                precision=precision)
        o64, _ = op.focused_sar(F, twtt, pos, 2.0, ap, "hann")
        if ap < 0:
            assert not np.any(out) and not np.any(o64)
        else:
            assert np.abs(out - o64).max() <= 1e-5 * np.abs(o64).max()


def test_dataset_front_end_matches_reference(golden):
    """focused_sar(ds, ...) through a Dataset-like object: checks, warning,
    provenance record and outputs."""
    from tests.golden import xrshim
    g = golden("focus")
    F = g["field"]
    T = F.shape[0]
    ds = xrshim.Dataset(
        {"field": (("slow_time", "twtt"), F, {}),
         "power": (("slow_time", "twtt"), np.abs(F) ** 2, {})},
        coords={"twtt": ("twtt", g["twtt"]),
                "x": ("slow_time", g["pos"][:, 0]),
                "y": ("slow_time", g["pos"][:, 1]),
                "z": ("slow_time", g["pos"][:, 2]),
                "slow_time": ("slow_time", np.arange(T) * 0.1)},
        attrs={"mode": "coherent", "wavelength": float(g["wavelength"]),
               "config": json.dumps({"radar": {"c": 299792458.0}})})
    with pytest.warns(UserWarning, match="alias in Doppler"):
        res = gp.focused_sar(ds, 250.0)
    peak = np.abs(g["focus_wide_field"]).max()
    assert np.abs(res.field.values - g["focus_wide_field"]).max() <= \
        1e-6 * peak
    steps = json.loads(res.attrs["processing"])
    assert steps[-1]["op"] == "focused_sar" and steps[-1]["aperture_m"] == 250
    with pytest.raises(ValueError, match="unknown window"):
        gp.focused_sar(ds, 96.0, window="kaiser")
    ds.attrs["mode"] = "incoherent"
    with pytest.raises(ValueError, match="coherent-mode"):
        gp.focused_sar(ds, 96.0)
