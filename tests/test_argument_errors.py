"""Argument errors of the drop-in entry points, on the host.

The reference raises ``ValueError`` for bad option combinations and shapes
before any kernel work (kernels/coherent.py:325-327, :341-343;
kernels/multilayer.py:314-318, :654-661, :710-712, :719-725, :729-731;
compare/multifreq.py:69-76). The GPU entry points keep the same texts and
raise them before any device allocation or copy: on a host without a GPU a
call that reached device work would fail with a CUDA error instead, so a
``ValueError`` here shows the check came first.
"""

import numpy as np
import pytest

from radar_sounder_simulator_gb300.coherent import coherent_cluttergram
from radar_sounder_simulator_gb300.incoherent import incoherent_cluttergram
from radar_sounder_simulator_gb300.multifreq import multifreq_traces
from radar_sounder_simulator_gb300.multilayer import refracted_cluttergram
from radar_sounder_simulator_gb300.scenes import facets_from_vertices

C = 299792458.0
K0 = 2 * np.pi * 60e6 / C
POS = np.array([[0.0, 0.0, 500.0], [10.0, 0.0, 500.0]])
UCT = np.tile([0.0, -1.0, 0.0], (2, 1))


def _grid(z0, n=4, d=10.0):
    ax = np.arange(n + 1) * d - n * d / 2
    X, Y = np.meshgrid(ax, ax)
    return facets_from_vertices(X, Y, z0 + 0.0 * X)


SURF, BED = _grid(0.0), _grid(-50.0)
N = len(BED.centers)
PH = np.ones(N, np.complex64)


def _coherent(**kw):
    args = dict(k=K0, gamma=-0.3, t0=0.0, dt=1e-8, n_samples=64, c=C)
    args.update(kw)
    return coherent_cluttergram(POS, UCT, BED.centers, BED.normals,
                                BED.areas, BED.e1, BED.e2, **args)


def _refracted(crossed=(SURF,), eps=(1.0, 3.15), **kw):
    args = dict(mode="coherent", t0=0.0, dt=1e-8, n_samples=64, c=C,
                gamma=-0.1, k0=K0)
    args.update(kw)
    return refracted_cluttergram(POS, UCT, BED, list(crossed), list(eps),
                                 [0.0] * len(eps), **args)


@pytest.mark.parametrize("kw,match", [
    (dict(roughness=(0.1, 5.0, PH, 20, "exponential")), "area-only D_Phi"),
    (dict(gamma=np.full(N + 1, -0.3)), "per-facet gamma shape"),
    (dict(pattern=("horn", np.zeros((2, 3)), 0.0, 0.0)),
     "unknown pattern kind"),
    (dict(roughness=(0.1, 5.0, PH, 20, "fractal"), d_phi_area=True),
     "unknown roughness acf"),
    (dict(precision="fp16"), "unknown precision"),
])
def test_coherent_argument_errors(kw, match):
    with pytest.raises(ValueError, match=match):
        _coherent(**kw)


@pytest.mark.parametrize("kw,match", [
    (dict(mode="incoherent", roughness=(0.1, 5.0, PH, 20)),
     "roughness requires coherent mode"),
    (dict(mode="incoherent", crossed_sigma=[0.1]),
     "roughness requires coherent mode"),
    (dict(mode="incoherent", taper_s=0.05), "grazing fix requires coherent"),
    (dict(mode="incoherent", d_phi_area=True),
     "grazing fix requires coherent"),
    (dict(mode="incoherent", gamma=np.zeros(N)),
     "per-facet gamma requires coherent mode"),
    (dict(mode="incoherent", diffuse=(np.ones(N), PH, 2.0)),
     "diffuse channel requires coherent mode"),
    (dict(diffuse=(np.ones(N - 1), PH, 2.0)), "diffuse amp shape"),
    (dict(gamma=np.zeros(N - 1)), "per-facet gamma shape"),
    (dict(roughness=(0.1, 5.0, PH, 20, "exponential")), "area-only D_Phi"),
    (dict(pattern=("horn", np.zeros((2, 3)), 0.0, 0.0)),
     "unknown pattern kind"),
    (dict(precision="fp16"), "unknown precision"),
])
def test_refracted_argument_errors(kw, match):
    with pytest.raises(ValueError, match=match):
        _refracted(**kw)


def test_refracted_stack_errors():
    # joint padding needs room between the surface and the platform
    high = _grid(600.0)
    with pytest.raises(ValueError, match="platform above the surface"):
        _refracted(crossed=(high,), refraction="joint", pad_to=2)
    with pytest.raises(ValueError, match="pad_to"):
        _refracted(crossed=(SURF, _grid(-20.0)), eps=(1.0, 2.0, 3.15),
                   refraction="joint", pad_to=1)
    with pytest.raises(ValueError, match="len\\(crossed\\) \\+ 1"):
        _refracted(eps=(1.0,))
    with pytest.raises(ValueError, match="takes 1..40"):
        _refracted(crossed=(), eps=(1.0,))


def test_incoherent_and_multifreq_argument_errors():
    with pytest.raises(ValueError, match="unknown pattern kind"):
        incoherent_cluttergram(POS, UCT, BED.centers, BED.normals,
                               BED.areas, t0=0.0, dt=1e-8, n_samples=64,
                               c=C, pattern=("horn", np.zeros((2, 3)), 0, 0))
    with pytest.raises(ValueError, match="block_size"):
        incoherent_cluttergram(POS, UCT, BED.centers, BED.normals,
                               BED.areas, t0=0.0, dt=1e-8, n_samples=64,
                               c=C, block_size=0)
    tw = 2 * 550.0 / C + np.arange(16) * 1e-8
    common = dict(f0=60e6, bandwidth=15e6, c=C, twtt=tw, n_freq=32)
    with pytest.raises(ValueError, match="freeze_amplitudes"):
        multifreq_traces(POS, BED.centers, BED.normals, BED.areas, BED.e1,
                         BED.e2, gamma=-0.3, roughness=(0.1, 5.0, PH, 20),
                         **common)
    with pytest.raises(ValueError, match="per-facet gamma shape"):
        multifreq_traces(POS, BED.centers, BED.normals, BED.areas, BED.e1,
                         BED.e2, gamma=np.zeros(N + 2), **common)


def test_range_compression_plan_and_apply_check_arguments_first():
    """The pulse-compression plan and apply entry points refuse bad sizes,
    precisions, null pointers and short plan buffers with their status
    codes before any device work (a call that reached a kernel launch on
    this host would return SS_ERR_CUDA instead)."""
    import ctypes as C
    from radar_sounder_simulator_gb300 import _lib
    L = _lib.lib()
    split, fp64 = _lib.PREC["split"], _lib.PREC["fp64"]
    ok = _lib.WaveformOpts(4, 2048, 1, 1201, 600, 0, 0)
    # plan sizes: 32 N bytes (double-float), 24 N bytes (float64), N = 4096
    assert L.ss_range_compress_plan_bytes(C.byref(ok), split) == 32 * 4096
    assert L.ss_range_compress_plan_bytes(C.byref(ok), fp64) == 24 * 4096
    assert L.ss_range_compress_plan_bytes(C.byref(ok), 7) == 0
    big = _lib.WaveformOpts(4, 8000, 1, 1201, 600, 0, 0)
    assert L.ss_range_compress_plan_bytes(C.byref(big), split) == 0
    dummy = C.c_void_p(256)   # never dereferenced: every call below fails
    nb = 32 * 4096
    bad_center = _lib.WaveformOpts(4, 2048, 1, 1201, 1201, 0, 0)
    cases = [
        (L.ss_range_compress_plan(C.byref(ok), split, None, dummy, nb, None),
         _lib.SS_ERR_ARG),
        (L.ss_range_compress_plan(C.byref(bad_center), split, dummy, dummy,
                                  nb, None), _lib.SS_ERR_ARG),
        (L.ss_range_compress_plan(C.byref(ok), 7, dummy, dummy, nb, None),
         _lib.SS_ERR_ARG),
        (L.ss_range_compress_plan(C.byref(big), split, dummy, dummy, nb,
                                  None), _lib.SS_ERR_UNSUPPORTED),
        (L.ss_range_compress_plan(C.byref(ok), split, dummy, dummy, nb - 16,
                                  None), _lib.SS_ERR_SCRATCH),
        (L.ss_range_compress_apply(C.byref(ok), split, dummy, nb, None, dummy,
                                   None), _lib.SS_ERR_ARG),
        (L.ss_range_compress_apply(C.byref(ok), fp64, dummy, 24 * 4096 - 1,
                                   dummy, dummy, None), _lib.SS_ERR_SCRATCH),
        (L.ss_range_compress_apply(C.byref(bad_center), split, dummy, nb,
                                   dummy, dummy, None), _lib.SS_ERR_ARG),
    ]
    for got, want in cases:
        assert got == want


@pytest.mark.parametrize("args,kw", [
    ((np.ones(3), 3, 100), {}),                       # center past the taps
    ((np.ones(3), 1, 0), {}),                         # no samples
    ((np.ones(1201), 600, 8000), {}),                 # above the FFT limit
    ((np.ones(3), 1, 100), {"precision": "fp16"}),    # unknown precision
])
def test_range_compressor_checks_arguments_before_the_device(args, kw):
    """Bad pulse-plan arguments raise ValueError before any device
    resolution, allocation or copy (on this host a device step would raise
    a CUDA error instead)."""
    from radar_sounder_simulator_gb300.waveform import RangeCompressor
    with pytest.raises(ValueError):
        RangeCompressor(*args, **kw)
