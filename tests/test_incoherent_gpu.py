"""GPU incoherent kernel (ss_incoherent_fwd through the drop-in
incoherent_cluttergram) against the reference's outputs and the float32
oracle.

Tolerances: bins are integer decisions and must match exactly -- checked
through the nonzero pattern of one-facet-per-bin cases and of the golden
histograms. Powers are float32 per pair (the kernel uses a reciprocal square
root where the reference divides) and summed in float32 per CTA chunk, so
each histogram is within 1e-5 relative L2 of the reference's and the
oracle's (the path's float bound is 1e-4)."""

import numpy as np
import pytest

from oracle import incoherent as oi
from radar_sounder_simulator_gb300.incoherent import incoherent_cluttergram

pytestmark = pytest.mark.gpu
C = 299792458.0
UCT = np.array([0.0, -1.0, 0.0])


def _rel(a, b):
    return np.linalg.norm(np.asarray(a, np.float64) - b) / np.linalg.norm(b)


@pytest.mark.parametrize("name", ["iso", "split", "dipole", "blocks"])
def test_matches_reference_golden(golden, name):
    g = golden("incoherent")
    surf = [g[f"surf_{k}"] for k in ("centers", "normals", "areas")]
    kw = dict(t0=float(g["t0"]), dt=float(g["dt"]),
              n_samples=int(g["n_samples"]), c=C)
    pat = (str(g["ant_kind"]), g["ant_pv"], g["ant_pa"], g["ant_pb"])
    kw.update({"iso": {}, "split": dict(split_sides=True),
               "dipole": dict(pattern=pat),
               "blocks": dict(block_size=100)}[name])
    p, d = incoherent_cluttergram(g["pos"], g["uct"], *surf, **kw)
    ref, dref = g[f"inc_{name}_power"], g[f"inc_{name}_dropped"]
    assert p.dtype == np.float32 and d.dtype == np.float32
    assert p.shape == ref.shape
    np.testing.assert_array_equal(p > 0, ref > 0)
    assert _rel(p, ref) <= 1e-5
    np.testing.assert_allclose(d, dref, rtol=1e-5)


def test_fast_bins_match_far_from_edges():
    """High altitude, fine bins: most pairs take the fast bin path and all
    agree with the oracle. Each facet's power is distinct and bins hold a
    few facets, so one facet in a wrong bin would move the relative L2
    error by about 1e-2, three orders above the tolerance."""
    rng = np.random.default_rng(31)
    nf = 4000
    centers = np.column_stack([rng.uniform(-300, 300, nf),
                               rng.uniform(-300, 300, nf),
                               rng.uniform(-60, 60, nf)])
    normals = np.tile([0.0, 0.0, 1.0], (nf, 1))
    areas = rng.uniform(10.0, 40.0, nf)
    p = np.array([[0.0, 0.0, 3000.0], [15.0, -7.0, 3010.0]])
    kw = dict(t0=2 * 2930.0 / C, dt=1e-9, n_samples=1000, c=C)
    got, gd = incoherent_cluttergram(p, np.tile(UCT, (2, 1)), centers,
                                     normals, areas, **kw)
    ref, rd = oi.incoherent_cluttergram(p, np.tile(UCT, (2, 1)), centers,
                                        normals, areas, **kw)
    np.testing.assert_array_equal(got > 0, ref > 0)
    assert _rel(got, ref) <= 1e-5
    np.testing.assert_allclose(gd, rd, rtol=1e-5)


def test_edge_pairs_bin_like_the_reference():
    """Facets placed within 2e-4 bin of a bin edge -- below the float32
    resolution of u there, where a fast evaluation alone would guess -- land
    in the oracle's bins (same detection argument as above)."""
    p = np.array([[0.0, 0.0, 2000.0]])
    t0, dt = 2 * 1900.0 / C, 2e-9
    rng = np.random.default_rng(5)
    n = 3000
    xs = rng.uniform(-400, 400, n)
    ys = rng.uniform(-400, 400, n)
    centers = np.column_stack([xs, ys, np.zeros(n)])
    r = np.linalg.norm(p[0] - centers, axis=1)
    u = (2 * r / C - t0) / dt
    target = np.round(u) + rng.uniform(-2e-4, 2e-4, n)
    r_t = (target * dt + t0) * C / 2
    centers[:, 2] = p[0, 2] - np.sqrt(r_t ** 2 - xs ** 2 - ys ** 2)
    normals = np.tile([0.0, 0.0, 1.0], (n, 1))
    areas = rng.uniform(1.0, 2.0, n)
    kw = dict(t0=t0, dt=dt, n_samples=700, c=C)
    got, gd = incoherent_cluttergram(p, UCT[None], centers, normals, areas,
                                     **kw)
    ref, rd = oi.incoherent_cluttergram(p, UCT[None], centers, normals,
                                        areas, **kw)
    np.testing.assert_array_equal(got > 0, ref > 0)
    assert _rel(got, ref) <= 1e-5
    np.testing.assert_allclose(gd, rd, rtol=1e-5)


@pytest.mark.parametrize("split", [False, True])
def test_ragged_sizes_and_many_chunks(split):
    """Trace and facet counts not multiples of the trace block or CTA size,
    a facet count large enough for several chunks per trace block."""
    rng = np.random.default_rng(9)
    n = 20011
    centers = np.column_stack([rng.uniform(-2000, 2000, n),
                               rng.uniform(-2000, 2000, n),
                               rng.normal(0, 20, n)])
    nrm = rng.normal(0, 0.1, (n, 3))
    nrm[:, 2] = 1.0
    nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
    areas = rng.uniform(100, 900, n)
    T = 11
    pos = np.column_stack([np.linspace(-500, 500, T), rng.uniform(-5, 5, T),
                           np.full(T, 1500.0)])
    kw = dict(t0=2 * 1480.0 / C, dt=1.0 / 30e6, n_samples=333, c=C,
              split_sides=split)
    got, gd = incoherent_cluttergram(pos, np.tile(UCT, (T, 1)), centers, nrm,
                                     areas, **kw)
    ref, rd = oi.incoherent_cluttergram(pos, np.tile(UCT, (T, 1)), centers,
                                        nrm, areas, **kw)
    np.testing.assert_array_equal(got > 0, ref > 0)
    assert _rel(got, ref) <= 1e-5
    np.testing.assert_allclose(gd, rd, rtol=1e-5)


@pytest.mark.parametrize("kind", ["array", "tabulated", "finite_dipole"])
def test_patterns_weight_power_by_g4(kind):
    """Pattern kinds through the kernel against the oracle's g^4."""
    rng = np.random.default_rng(12)
    n = 3000
    centers = np.column_stack([rng.uniform(-800, 800, n),
                               rng.uniform(-800, 800, n), np.zeros(n)])
    normals = np.tile([0.0, 0.0, 1.0], (n, 1))
    areas = np.full(n, 50.0)
    T = 3
    pos = np.column_stack([np.zeros(T), np.linspace(-30, 30, T),
                           np.full(T, 1200.0)])
    if kind == "array":
        pv = np.tile(np.array([[0.0, -1.0, 0.0], [0.0, 0.0, -1.0]]),
                     (T, 1, 1))
        pat = (kind, pv, 4.0, np.array([0.5, 1.0, 2.0, 1.0]))
    elif kind == "tabulated":
        th = np.linspace(0.0, np.pi / 2, 91)
        pat = (kind, np.tile([0.0, 0.0, -1.0], (T, 1)), th,
               np.cos(th) ** 2 + 0.05)
    else:
        pat = (kind, np.tile([1.0, 0.0, 0.0], (T, 1)), 1.5, 0.0)
    kw = dict(t0=2 * 1150.0 / C, dt=1e-8, n_samples=300, c=C, pattern=pat)
    got, gd = incoherent_cluttergram(pos, np.tile(UCT, (T, 1)), centers,
                                     normals, areas, **kw)
    ref, rd = oi.incoherent_cluttergram(pos, np.tile(UCT, (T, 1)), centers,
                                        normals, areas, **kw)
    np.testing.assert_array_equal(got > 0, ref > 0)
    assert _rel(got, ref) <= 2e-5
    np.testing.assert_allclose(gd, rd, rtol=2e-5)


def test_oversized_window_is_refused():
    c = np.zeros((1, 3))
    with pytest.raises(ValueError):
        incoherent_cluttergram(np.array([[0.0, 0.0, 100.0]]), UCT[None], c,
                               np.array([[0.0, 0.0, 1.0]]), np.ones(1),
                               t0=0.0, dt=1e-9, n_samples=60000, c=C)
