"""Frequency-sampled synthesis (compare/multifreq.py:45-98) on the GPU.

Against the reference's own outputs (golden, float64 facets) and the
float64 oracle on the same float32-quantised facets the kernels read:
FP64 form within 1e-9 of the profile peak (oracle) / 1e-6 (golden, which
differs by the float32 facet quantisation); split form within the
path bounds -- relative L2 <= 1e-4, phase <= 1e-3 rad, power within
0.01 dB for samples above -60 dB of the peak.
"""

import numpy as np
import pytest

from oracle import lpa
from oracle import multifreq as omf
from radar_sounder_simulator_gb300 import multifreq as mf
from tests.util import facets_from, field_errors

pytestmark = pytest.mark.gpu
C = 299792458.0


def q32(f):
    """The facet arrays as the kernels read them (float32-quantised)."""
    return [np.asarray(getattr(f, a), np.float32).astype(np.float64)
            for a in ("centers", "normals", "areas", "e1", "e2")]


def split_ok(y, ref):
    e = field_errors(y, ref)
    assert e["rel_l2"] <= 1e-4, e
    assert e["phase_rad"] <= 1e-3, e
    assert e["power_db"] <= 0.01, e


@pytest.mark.parametrize("frozen", [False, True])
def test_profile_matches_reference(golden, frozen):
    g = golden("waveform")
    f = facets_from(g, "mf")
    kw = dict(gamma=-0.28, f0=60e6, bandwidth=15e6, c=C, twtt=g["mf_twtt"],
              n_freq=64, freeze_amplitudes=frozen)
    ref = g["mf_frozen" if frozen else "mf_full"]
    y64 = mf.multifreq_profile(g["mf_pos"], f.centers, f.normals, f.areas,
                               f.e1, f.e2, precision="fp64", **kw)
    peak = np.abs(ref).max()
    assert y64.shape == ref.shape and y64.dtype == np.complex128
    assert np.abs(y64 - ref).max() <= 1e-6 * peak
    orc = omf.multifreq_profile(g["mf_pos"], *q32(f), **kw)
    assert np.abs(y64 - orc).max() <= 1e-9 * np.abs(orc).max()
    ysp = mf.multifreq_profile(g["mf_pos"], f.centers, f.normals, f.areas,
                               f.e1, f.e2, precision="split", **kw)
    split_ok(ysp, orc)


def _scene(n=24, d=25.0, seed=7):
    rng = np.random.default_rng(seed)
    ax = (np.arange(n + 1) - n / 2) * d
    X, Y = np.meshgrid(ax, ax)
    Z = 3.0 * rng.standard_normal(X.shape)
    V = np.stack([X, Y, Z], -1)
    v00, v01, v10, v11 = V[:-1, :-1], V[:-1, 1:], V[1:, :-1], V[1:, 1:]
    e1 = (((v01 + v11) - (v00 + v10)) / 2.0).reshape(-1, 3)
    e2 = (((v10 + v11) - (v00 + v01)) / 2.0).reshape(-1, 3)
    c = ((v00 + v01 + v10 + v11) / 4.0).reshape(-1, 3)
    raw = np.cross(e1, e2)
    a = np.linalg.norm(raw, axis=1)
    nr = raw / a[:, None]
    return c, nr, a, e1, e2


@pytest.mark.parametrize("precision", ["fp64", "split"])
@pytest.mark.parametrize("n_freq", [256, 1500])
def test_track_matches_per_position_oracle(precision, n_freq):
    c, nr, a, e1, e2 = _scene()
    T = 5
    pos = np.column_stack([np.linspace(-60, 60, T), np.full(T, 7.0),
                           np.full(T, 900.0)])
    r0 = np.linalg.norm(pos[0] - c, axis=1).min()
    tw = 2 * r0 / C - 2e-7 + np.arange(96) * (1.0 / 30e6)
    kw = dict(gamma=-0.3, f0=60e6, bandwidth=15e6, c=C, twtt=tw,
              n_freq=n_freq)
    for frozen in (False, True):
        y = mf.multifreq_traces(pos, c, nr, a, e1, e2, precision=precision,
                                freeze_amplitudes=frozen, **kw)
        assert y.shape == (T, len(tw))
        ref = np.array([omf.multifreq_profile(p, *[np.asarray(v, np.float32)
                                                   .astype(np.float64)
                                                   for v in (c, nr, a, e1,
                                                             e2)],
                                              freeze_amplitudes=frozen, **kw)
                        for p in pos])
        if precision == "fp64":
            assert np.abs(y - ref).max() <= 1e-9 * np.abs(ref).max()
        else:
            split_ok(y, ref)


def test_per_facet_gamma_taper_and_rough_frozen():
    c, nr, a, e1, e2 = _scene(n=16, seed=9)
    rng = np.random.default_rng(2)
    n = len(c)
    gam = rng.uniform(-0.5, 0.5, n)
    ph = np.exp(2j * np.pi * rng.random(n)).astype(np.complex64)
    pos = np.array([[5.0, -3.0, 700.0], [15.0, -3.0, 700.0]])
    tw = 2 * 690.0 / C + np.arange(80) * (1.0 / 30e6)
    f0, bw, K = 60e6, 15e6, 512
    k0 = 2 * np.pi * f0 / C
    q = [np.asarray(v, np.float32).astype(np.float64)
         for v in (c, nr, a, e1, e2)]
    g32 = np.asarray(gam, np.float32).astype(np.float64)
    for rough in (None, (0.2, 3.0, ph, 40, "exponential")):
        y = mf.multifreq_traces(pos, c, nr, a, e1, e2, gamma=gam, f0=f0,
                                bandwidth=bw, c=C, twtt=tw, n_freq=K,
                                freeze_amplitudes=True, taper_s=0.05,
                                roughness=rough, d_phi_area=True,
                                precision="split")
        ref = []
        for p in pos:
            if rough is None:
                c0, r = lpa.lpa_field(p, *q, k0, g32, taper_s=0.05)
            else:
                c0, r = lpa.rough_lpa_field(p, *q, k0, g32, 0.2, 3.0,
                                            ph.astype(np.complex128), 40,
                                            taper_s=0.05, area_only=True,
                                            acf="exponential")
            amp0 = c0 * np.exp(2j * k0 * r)
            ref.append(omf.synth_frozen(r, amp0, f0=f0, bandwidth=bw, c=C,
                                        twtt=tw, n_freq=K))
        split_ok(y, np.array(ref))


def test_alias_guard_and_argument_errors():
    c, nr, a, e1, e2 = _scene(n=8)
    pos = np.array([0.0, 0.0, 900.0])
    tw = 2 * 900.0 / C + np.arange(64) * (1.0 / 30e6)
    with pytest.raises(ValueError, match="alias"):
        mf.multifreq_profile(pos, c, nr, a, e1, e2, gamma=-0.3, f0=60e6,
                             bandwidth=15e6, c=C, twtt=tw * 3.0, n_freq=16)
    with pytest.raises(ValueError):
        mf.multifreq_traces(pos[None], c, nr, a, e1, e2, gamma=-0.3,
                            f0=60e6, bandwidth=15e6, c=C, twtt=tw,
                            n_freq=64, roughness=(0.1, 2.0,
                                                  np.ones(len(c)), 10))
