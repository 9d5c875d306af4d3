"""Pulse compression (waveform.py:79-160): host pulse construction against
the reference's own pulses, and the GPU fast-time convolution against the
reference's FFT convolution (golden) and the float64 oracle.

Tolerances: the GPU convolves the float32-rounded input (the reference
convolves the kernels' complex64 output) with compensated float32 sums and
writes complex64, so each output sample is within a few float32 roundings
of the float64 result: absolute error <= 3e-7 of the row peak against the
oracle on the same (rounded) input, and the path's bound -- power within
0.01 dB -- for every sample above -60 dB of the peak.
"""

import types

import numpy as np
import pytest

from oracle import waveform as owf
from radar_sounder_simulator_gb300 import waveform as wf


def _radar(kind="chirp", construction="analytic", envelope=False,
           pulse_length=10e-6, dt=1.0 / 30e6):
    w = types.SimpleNamespace(kind=kind, bandwidth=15e6,
                              pulse_length=pulse_length, window="hann",
                              construction=construction,
                              incoherent_envelope=envelope)
    return types.SimpleNamespace(dt=dt, waveform=w)


def _check(y, ref):
    ref = np.asarray(ref)
    peak = np.abs(ref).max()
    assert np.abs(y - ref).max() <= 3e-7 * peak
    keep = np.abs(ref) ** 2 > 1e-6 * peak ** 2
    db = np.abs(10 * np.log10(np.abs(y[keep]) ** 2 / np.abs(ref[keep]) ** 2))
    assert db.max() <= 0.01


def test_pulses_match_reference(golden):
    g = golden("waveform")
    for w in ("none", "hann", "hamming"):
        p, m = wf.compressed_pulse(15e6, 20e-6, 1.0 / 30e6, w)
        assert m == int(g[f"pulse_{w}_m"])
        np.testing.assert_allclose(p, g[f"pulse_{w}"], rtol=1e-13,
                                   atol=1e-15)
    pc, mc = wf.compressed_pulse(15e6, 8e-6, 1.0 / 30e6, "hann", "chirp")
    assert mc == int(g["pulse_chirp_m"])
    np.testing.assert_allclose(pc, g["pulse_chirp"], rtol=0, atol=1e-9)


def test_delta_and_envelope_off_are_identity():
    x = np.arange(12, dtype=np.complex64).reshape(2, 6)
    assert wf.apply_waveform(x, _radar(kind="delta"), "coherent") is x
    p = np.ones((2, 6), np.float32)
    assert wf.apply_waveform(p, _radar(envelope=False), "incoherent") is p


@pytest.mark.gpu
def test_convolution_matches_reference_fft(golden):
    g = golden("waveform")
    m = int(g["pulse_hann_m"])              # 1201 taps: three tap chunks
    y = wf.convolve_fast_time(g["conv_in"], g["pulse_hann"], m)
    assert y.dtype == np.complex128 and y.shape == g["conv_out"].shape
    peak = np.abs(g["conv_out"]).max()
    assert np.abs(y - g["conv_out"]).max() <= 1e-6 * peak
    x32 = g["conv_in"].astype(np.complex64)
    _check(y, owf.convolve_fast_time(x32, g["pulse_hann"], m))


@pytest.mark.gpu
@pytest.mark.parametrize("construction", ["analytic", "chirp"])
def test_apply_waveform_coherent_split_sides(construction):
    rng = np.random.default_rng(3)
    T, B = 5, 700                           # B not a multiple of the tile
    x = (rng.normal(size=(T, B, 2)) + 1j * rng.normal(size=(T, B, 2)))
    x[:, ::7] *= 1e3                        # strong targets, weak sidelobes
    x = x.astype(np.complex64)
    radar = _radar(construction=construction, pulse_length=8e-6)
    y = wf.apply_waveform(x, radar, "coherent")
    assert y.dtype == np.complex64 and y.shape == x.shape
    p, m = owf.compressed_pulse(15e6, 8e-6, radar.dt, "hann", construction)
    for lane in range(2):
        _check(y[..., lane], owf.convolve_fast_time(x[..., lane], p, m))


@pytest.mark.gpu
def test_apply_waveform_incoherent_envelope():
    rng = np.random.default_rng(4)
    x = rng.exponential(size=(3, 513)).astype(np.float32)
    radar = _radar(envelope=True, pulse_length=5e-6)
    y = wf.apply_waveform(x, radar, "incoherent")
    assert y.dtype == np.float32 and y.shape == x.shape
    p, m = owf.compressed_pulse(15e6, 5e-6, radar.dt, "hann")
    ref = np.maximum(owf.convolve_fast_time(x, np.abs(p) ** 2, m).real, 0.0)
    assert np.abs(y - ref).max() <= 3e-7 * np.abs(ref).max()
    assert (y >= 0).all()


@pytest.mark.gpu
def test_single_tap_is_identity_and_bad_center_raises():
    import torch
    x = np.random.default_rng(5).normal(size=(2, 300)).astype(np.complex64)
    # the FFT path (the reference's method) leaves float64 round-off, the
    # direct sum reproduces the input exactly
    y = wf.convolve_fast_time(x, np.array([1.0]), 0)
    assert np.abs(y - x).max() <= 1e-12 * np.abs(x).max()
    yd = wf.compress_tensor(torch.as_tensor(x, device="cuda"), np.array([1.0]),
                            0, method="direct").cpu().numpy()
    np.testing.assert_array_equal(yd, x)
    xt = torch.zeros((2, 300, 2), dtype=torch.float32, device="cuda")
    with pytest.raises(ValueError):
        wf.compress_tensor(xt, np.ones(3), 3)


@pytest.mark.gpu
@pytest.mark.parametrize("method", ["fft", "direct"])
def test_both_methods_match_the_oracle(method):
    """FFT (float64, the reference's method) and the compensated direct sum,
    complex and power-envelope forms, against the float64 oracle."""
    import torch
    rng = np.random.default_rng(6)
    T, B = 3, 900
    x = (rng.normal(size=(T, B)) + 1j * rng.normal(size=(T, B)))
    x[:, ::11] *= 1e3
    x = x.astype(np.complex64)
    p, m = owf.compressed_pulse(15e6, 8e-6, 1.0 / 30e6, "hann", "chirp")
    xt = torch.as_tensor(x, device="cuda")
    y = wf.compress_tensor(xt, p, m, method=method).cpu().numpy()
    _check(y, owf.convolve_fast_time(x, p, m))
    pw = (np.abs(x) ** 2).astype(np.float32)
    yp = wf.compress_tensor(torch.as_tensor(pw, device="cuda"),
                            np.abs(p) ** 2, m, power=True,
                            method=method).cpu().numpy()
    ref = np.maximum(owf.convolve_fast_time(pw, np.abs(p) ** 2, m).real, 0)
    assert np.abs(yp - ref).max() <= 3e-7 * np.abs(ref).max()


@pytest.mark.gpu
def test_long_rows_fall_back_to_the_direct_sum():
    import torch
    rng = np.random.default_rng(7)
    x = (rng.normal(size=(2, 8000)) +
         1j * rng.normal(size=(2, 8000))).astype(np.complex64)
    p, m = owf.compressed_pulse(15e6, 20e-6, 1.0 / 30e6, "hann")
    xt = torch.as_tensor(x, device="cuda")
    with pytest.raises(ValueError):
        wf.compress_tensor(xt, p, m, method="fft")
    y = wf.compress_tensor(xt, p, m).cpu().numpy()
    _check(y, owf.convolve_fast_time(x, p, m))


def _rows(seed, T, B, lanes=None):
    rng = np.random.default_rng(seed)
    shape = (T, B) if lanes is None else (T, B, lanes)
    x = rng.normal(size=shape) + 1j * rng.normal(size=shape)
    x[:, ::13] *= 1e3                       # strong targets, weak sidelobes
    return x


@pytest.mark.gpu
@pytest.mark.parametrize("B,pulse_us", [(2048, 20e-6), (500, 8e-6),
                                        (700, 8e-6), (300, 2e-6),
                                        (5000, 30e-6)])
def test_split_fft_matches_the_float64_fft(B, pulse_us):
    """The double-float transforms against the float64 ones on the same
    float32-rounded rows: each complex64 output within one float32 rounding
    of the float64 result (plus 1e-12 of the peak), and both within the
    oracle bounds. Sizes give N = 4096 and 1024 (radix-4 stages only), 2048,
    512 and 8192 (odd log2: with the radix-2 stage; 8192 is the largest
    plan)."""
    import torch
    x = _rows(8, 6, B).astype(np.complex64)
    p, m = owf.compressed_pulse(15e6, pulse_us, 1.0 / 30e6, "hann", "chirp")
    xt = torch.as_tensor(x, device="cuda")
    y64 = wf.compress_tensor(xt, p, m, method="fft",
                             precision="fp64").cpu().numpy()
    ys = wf.compress_tensor(xt, p, m, method="fft",
                            precision="split").cpu().numpy()
    peak = np.abs(y64).max()
    assert np.all(np.abs(ys - y64) <= 2.0 ** -23 * np.abs(y64) + 1e-12 * peak)
    ref = owf.convolve_fast_time(x, p, m)
    _check(ys, ref)
    _check(y64, ref)


@pytest.mark.gpu
def test_split_fft_power_envelope_and_float64_input():
    import torch
    rng = np.random.default_rng(9)
    pw = rng.exponential(size=(4, 1500))
    pw[:, ::17] *= 1e4
    p, m = owf.compressed_pulse(15e6, 10e-6, 1.0 / 30e6, "hann")
    taps = np.abs(p) ** 2
    # float64 input is rounded to float32 first, as the reference convolves
    # the kernels' float32 output
    y = wf.compress_tensor(torch.as_tensor(pw, device="cuda"), taps, m,
                           power=True, precision="split").cpu().numpy()
    ref = np.maximum(owf.convolve_fast_time(pw.astype(np.float32), taps,
                                            m).real, 0.0)
    assert y.dtype == np.float32 and (y >= 0).all()
    assert np.abs(y - ref).max() <= 3e-7 * np.abs(ref).max()
    xc = _rows(10, 3, 1500, lanes=2)        # complex128, split sides
    yc = wf.compress_tensor(torch.as_tensor(xc, device="cuda"), p, m,
                            precision="split").cpu().numpy()
    for lane in range(2):
        _check(yc[..., lane], owf.convolve_fast_time(
            xc[..., lane].astype(np.complex64), p, m))


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp64", "split"])
def test_range_compressor_reuses_one_plan(precision):
    """One plan applied to arrays of different trace and lane counts gives
    the one-call results bit for bit; a row length other than the plan's
    is refused."""
    import torch
    p, m = owf.compressed_pulse(15e6, 8e-6, 1.0 / 30e6, "hann", "chirp")
    rc = wf.RangeCompressor(p, m, 900, precision=precision, device="cuda")
    for seed, lanes in ((11, None), (12, 2)):
        xt = torch.as_tensor(_rows(seed, 5, 900, lanes).astype(np.complex64),
                             device="cuda")
        a = rc.run(xt).cpu().numpy()
        b = wf.compress_tensor(xt, p, m, precision=precision).cpu().numpy()
        np.testing.assert_array_equal(a, b)
    with pytest.raises(ValueError):
        rc.run(torch.zeros((2, 901), dtype=torch.complex64, device="cuda"))
    with pytest.raises(ValueError):
        wf.RangeCompressor(p, m, 8000, precision=precision, device="cuda")


@pytest.mark.gpu
def test_split_single_tap_is_identity():
    x = np.random.default_rng(5).normal(size=(2, 300)).astype(np.complex64)
    y = wf.convolve_fast_time(x, np.array([1.0]), 0, precision="split")
    assert np.abs(y - x).max() <= 1e-12 * np.abs(x).max()
