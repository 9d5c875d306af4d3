"""Properties the reference's own multilayer tests hold
(tests/test_multilayer.py:59-107, :225-254; tests/test_multilayer_joint.py:
212-242), checked on the GPU drop-in: index-matched crossings reduce the
refracted path to the single-interface kernel, padding the joint solve is a
no-op, a larger Newton budget does not move converged fields, and invalid
(shadowed) paths go to the dropped channel as finite power with the
binned + dropped total independent of the window."""

import numpy as np
import pytest

from radar_sounder_simulator_gb300.coherent import coherent_cluttergram
from radar_sounder_simulator_gb300.multilayer import refracted_cluttergram
from radar_sounder_simulator_gb300.scenes import facets_from_vertices

pytestmark = pytest.mark.gpu
C = 299792458.0
K0 = 2 * np.pi * 60e6 / C
P = np.array([[-40.0, 10.0, 500.0], [0.0, -5.0, 505.0], [35.0, 0.0, 498.0]])
UCT = np.tile([0.0, -1.0, 0.0], (3, 1))
FLAT = lambda x, y: 0.0 * x  # noqa: E731


def surface_facets(extent, d, fn, z0=0.0):
    ax = np.arange(-extent / 2, extent / 2 + 1e-9, d)
    X, Y = np.meshgrid(ax, ax)
    return facets_from_vertices(X, Y, z0 + fn(X, Y))


def _fresnel(e1, e2):
    n1, n2 = np.sqrt(e1), np.sqrt(e2)
    return (n1 - n2) / (n1 + n2)


def _firn_case():
    eps = [1.0, 1.5, 1.55, 1.6, 1.65]
    crossed = [surface_facets(80.0, 4.0, FLAT),
               surface_facets(80.0, 4.0, FLAT, z0=-8.0),
               surface_facets(80.0, 4.0, FLAT, z0=-17.0)]
    tgt = surface_facets(80.0, 4.0,
                         lambda x, y: 0.1 * np.sin(2 * np.pi * y / 30.0),
                         z0=-40.0)
    kw = dict(mode="coherent", t0=3.3e-6, dt=1e-8, n_samples=80, c=C,
              gamma=_fresnel(eps[3], eps[4]), k0=K0)
    return tgt, crossed, eps[:4], kw


def _highcontrast_case():
    mid = lambda x, y: 0.3 * np.cos(2 * np.pi * x / 40.0)  # noqa: E731
    bed = lambda x, y: 0.5 * np.sin(2 * np.pi * y / 30.0)  # noqa: E731
    eps = [1.0, 2.2, 4.5]
    crossed = [surface_facets(80.0, 4.0, FLAT),
               surface_facets(80.0, 4.0, mid, z0=-20.0)]
    tgt = surface_facets(80.0, 4.0, bed, z0=-60.0)
    kw = dict(mode="coherent", t0=3.3e-6, dt=1e-8, n_samples=100, c=C,
              gamma=_fresnel(eps[1], eps[2]), k0=K0)
    return tgt, crossed, eps, kw


def _run(tgt, crossed, eps, kw, precision, **extra):
    out, drop = refracted_cluttergram(P, UCT, tgt, crossed, eps,
                                      [0.0] * len(eps), **kw, **extra,
                                      precision=precision,
                                      out_dtype=np.complex128)
    return out, drop


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-9), ("split", 1e-5)])
def test_padding_is_exact_noop(precision, tol):
    tgt, crossed, eps, kw = _firn_case()
    base, _ = _run(tgt, crossed, eps, kw, precision, refraction="joint")
    assert np.abs(base).max() > 0
    # 4 crossings run the register-resident solve, 8 and 16 the deep-stack
    # instantiation (its arrays in local memory) in the split form
    for pad in (4, 8, 16):
        padded, _ = _run(tgt, crossed, eps, kw, precision,
                         refraction="joint", pad_to=pad)
        d = np.abs(padded - base).max() / np.abs(base).max()
        assert d < tol, (pad, d)
    with pytest.raises(ValueError):
        _run(tgt, crossed, eps, kw, precision, refraction="joint",
             pad_to=41)


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-9), ("split", 1e-5)])
def test_joint_budget_converged(precision, tol):
    tgt, crossed, eps, kw = _highcontrast_case()
    base, _ = _run(tgt, crossed, eps, kw, precision, refraction="joint")
    more, _ = _run(tgt, crossed, eps, kw, precision, refraction="joint",
                   joint_newton=24, joint_backtrack=10)
    assert np.abs(more - base).max() / np.abs(base).max() < tol


@pytest.mark.parametrize("precision", ["fp64", "split"])
def test_index_matched_crossing_reduces_to_surface_kernel(precision):
    """eps = 1 on both sides of the crossed interface and no attenuation:
    the bed's refracted field is the single-interface field of the bed
    facets (the reference's gate: 5e-3 of the peak)."""
    surf = surface_facets(120.0, 4.0,
                          lambda x, y: 0.5 * np.sin(x / 9.0) * np.cos(y / 13.0))
    bed = surface_facets(120.0, 4.0,
                         lambda x, y: 0.8 * np.cos(x / 11.0) + 0.2 * y / 60,
                         z0=-30.0)
    gamma = _fresnel(1.0, 6.0)
    kw = dict(t0=2 * 500.0 / C, dt=1e-8, n_samples=128, c=C)
    ref, _ = refracted_cluttergram(P, UCT, bed, [surf], [1.0, 1.0],
                                   [0.0, 0.0], mode="coherent", gamma=gamma,
                                   k0=K0, precision=precision,
                                   out_dtype=np.complex128, **kw)
    one, _ = coherent_cluttergram(P, UCT, bed.centers, bed.normals,
                                  bed.areas, bed.e1, bed.e2, k=K0,
                                  gamma=gamma, precision=precision,
                                  out_dtype=np.complex128, **kw)
    peak = np.abs(one).max()
    assert peak > 0
    assert np.abs(ref - one).max() < 5e-3 * peak


@pytest.mark.parametrize("precision", ["fp64", "split"])
def test_steep_bed_invalid_paths_dropped_not_nan(precision):
    """A bed tilted through the surface plane: same-side geometry has no
    refracted path; those pairs land in dropped, outputs stay finite, and
    binned + dropped power does not depend on the window."""
    surf = surface_facets(200.0, 5.0, FLAT)
    bed = surface_facets(200.0, 5.0, lambda x, y: np.tan(np.radians(14.0)) * x,
                         z0=-10.0)
    assert bed.centers[:, 2].max() > 0.0          # part of the bed above
    args = (P, UCT, bed, [surf], [1.0, 3.17], [0.0, 0.0])
    common = dict(mode="incoherent", c=C, precision=precision)
    wide, dw = refracted_cluttergram(*args, t0=0.0, dt=1e-8, n_samples=1250,
                                     **common)
    narrow, dn = refracted_cluttergram(*args, t0=3.45e-6, dt=1e-8,
                                       n_samples=30, **common)
    for out, drop in ((wide, dw), (narrow, dn)):
        assert np.isfinite(out).all() and np.isfinite(drop).all()
        assert (drop > 0).all()
    tot_w = wide.sum(axis=1) + dw
    tot_n = narrow.sum(axis=1) + dn
    np.testing.assert_allclose(tot_w, tot_n, rtol=1e-4)
    assert (dn > dw).all()
