"""Properties the reference's own kernel tests hold for this path
(tests/test_coherent_kernel.py:203-317), checked on the GPU forms through
the drop-in API: phase precision at 20 km / 195 MHz against the float64
per-facet field, energy bookkeeping between binned and dropped power, the
two sides of a split summing to the combined field, and block-size
independence. Each runs for both precisions."""

import numpy as np
import pytest

from oracle import lpa
from radar_sounder_simulator_gb300.coherent import coherent_cluttergram

pytestmark = pytest.mark.gpu
C = 299792458.0
UCT = np.array([0.0, -1.0, 0.0])
PRECISIONS = ["fp64", "split"]


def _plate(n, L, centers):
    e1 = np.tile([L, 0.0, 0.0], (n, 1))
    e2 = np.tile([0.0, L, 0.0], (n, 1))
    normals = np.tile([0.0, 0.0, 1.0], (n, 1))
    return normals, np.full(n, L * L), e1, e2


def _grid(ncell=20, d=3.0, amp=1.5):
    """Small undulating facet grid (vertex heights -> corner rule)."""
    ax = np.arange(ncell + 1) * d - ncell * d / 2
    X, Y = np.meshgrid(ax, ax)
    Z = amp * np.sin(X / 3.1) * np.cos(Y / 4.7)
    V = np.stack([X, Y, Z], axis=-1)
    v00, v01, v10, v11 = V[:-1, :-1], V[:-1, 1:], V[1:, :-1], V[1:, 1:]
    e1 = ((v01 + v11) - (v00 + v10)) / 2.0
    e2 = ((v10 + v11) - (v00 + v01)) / 2.0
    c = ((v00 + v01 + v10 + v11) / 4.0).reshape(-1, 3)
    raw = np.cross(e1, e2).reshape(-1, 3)
    a = np.linalg.norm(raw, axis=1)
    return c, raw / a[:, None], a, e1.reshape(-1, 3), e2.reshape(-1, 3)


@pytest.mark.parametrize("precision", PRECISIONS)
def test_phase_precision_20km_195mhz(precision):
    """One facet per bin: each bin's phase equals the float64 facet field's
    to well inside lambda/50 of range (the reference's gate)."""
    lam = C / 195e6
    k = 2 * np.pi / lam
    rng = np.random.default_rng(21)
    nf = 16
    centers = np.column_stack([rng.uniform(-2500, 2500, nf),
                               rng.uniform(-2500, 2500, nf),
                               rng.uniform(-40, 40, nf)])
    normals, areas, e1, e2 = _plate(nf, 4.0, centers)
    p = np.array([[0.0, 0.0, 20000.0]])
    r = np.linalg.norm(p[0] - centers, axis=1)
    t0, dt = 2 * r.min() / C - 1e-8, 5e-9
    b = np.floor((2 * r / C - t0) / dt).astype(int)
    assert len(set(b)) == nf
    field, _ = coherent_cluttergram(p, UCT[None], centers, normals, areas,
                                    e1, e2, k=k, gamma=-0.3, t0=t0, dt=dt,
                                    n_samples=1024, c=C, precision=precision,
                                    out_dtype=np.complex128)
    q = [np.asarray(v, np.float32).astype(np.float64)
         for v in (centers, normals, areas, e1, e2)]
    ref, _ = lpa.lpa_field(p[0], *q, k, -0.3)
    dphi = np.abs(np.angle(field[0, b] / ref))
    assert dphi.max() / (2 * k) < lam / 50
    assert dphi.max() < (1e-9 if precision == "fp64" else 1e-3)


@pytest.mark.parametrize("precision", PRECISIONS)
def test_energy_bookkeeping(precision):
    """Facets in distinct bins: binned power + dropped equals the total, and
    dropped is exactly the out-of-window facets' power."""
    nf = 10
    rng = np.random.default_rng(22)
    centers = np.column_stack([rng.uniform(-30, 30, nf),
                               rng.uniform(-30, 30, nf),
                               55.0 * np.arange(nf) - 150.0])
    normals, areas, e1, e2 = _plate(nf, 2.0, centers)
    p = np.array([[0.0, 0.0, 900.0]])
    r = np.linalg.norm(p[0] - centers, axis=1)
    k = 2 * np.pi / 5.0
    t0, dt = 2 * r.min() / C - 1e-8, 4e-8
    b = np.floor((2 * r / C - t0) / dt).astype(int)
    assert len(set(b)) == nf
    n_samples = int(np.sort(b)[-3])
    field, dropped = coherent_cluttergram(
        p, UCT[None], centers, normals, areas, e1, e2, k=k, gamma=-0.3,
        t0=t0, dt=dt, n_samples=n_samples, c=C, precision=precision,
        out_dtype=np.complex128)
    q = [np.asarray(v, np.float32).astype(np.float64)
         for v in (centers, normals, areas, e1, e2)]
    contrib, _ = lpa.lpa_field(p[0], *q, k, -0.3)
    out = b >= n_samples
    assert out.sum() >= 2
    total = (np.abs(contrib) ** 2).sum()
    binned = (np.abs(field[0]) ** 2).sum()
    np.testing.assert_allclose(binned + dropped[0], total, rtol=1e-5)
    np.testing.assert_allclose(dropped[0], (np.abs(contrib[out]) ** 2).sum(),
                               rtol=1e-5)


@pytest.mark.parametrize("precision", PRECISIONS)
def test_split_sides_sum_to_combined(precision):
    c, n, a, e1, e2 = _grid()
    p = np.array([[5.0, 2.0, 150.0], [-8.0, -3.0, 160.0]])
    uct = np.tile(UCT, (2, 1))
    kw = dict(k=2 * np.pi / 5.0, gamma=-0.3, t0=2 * 140.0 / C, dt=2e-9,
              n_samples=64, c=C, precision=precision,
              out_dtype=np.complex128)
    comb, d0 = coherent_cluttergram(p, uct, c, n, a, e1, e2, **kw)
    split, d1 = coherent_cluttergram(p, uct, c, n, a, e1, e2,
                                     split_sides=True, **kw)
    assert split.shape == comb.shape + (2,)
    assert np.abs(split[..., 0]).sum() > 0 and np.abs(split[..., 1]).sum() > 0
    tol = 1e-12 if precision == "fp64" else 1e-6
    assert np.abs(split.sum(axis=-1) - comb).max() <= tol * np.abs(comb).max()
    np.testing.assert_allclose(d0, d1, rtol=1e-5)


@pytest.mark.parametrize("precision", PRECISIONS)
def test_block_size_does_not_change_the_result(precision):
    c, n, a, e1, e2 = _grid()
    p = np.array([[5.0, 2.0, 150.0]])
    kw = dict(k=2 * np.pi / 5.0, gamma=-0.3, t0=2 * 140.0 / C, dt=2e-9,
              n_samples=64, c=C, precision=precision,
              out_dtype=np.complex128)
    x, dx = coherent_cluttergram(p, UCT[None], c, n, a, e1, e2, **kw)
    y, dy = coherent_cluttergram(p, UCT[None], c, n, a, e1, e2,
                                 block_size=97, **kw)
    tol = 1e-12 if precision == "fp64" else 1e-6
    assert np.abs(x - y).max() <= tol * np.abs(x).max()
    np.testing.assert_allclose(dx, dy, rtol=1e-5)


@pytest.mark.parametrize("precision", PRECISIONS)
def test_window_before_every_facet_drops_everything(precision):
    """No facet bins inside the window: the field is zero and the dropped
    power is the whole scene's (drop, never wrap)."""
    c, n, a, e1, e2 = _grid()
    p = np.array([[5.0, 2.0, 150.0]])
    k = 2 * np.pi / 5.0
    kw = dict(k=k, gamma=-0.3, t0=2 * 400.0 / C, dt=2e-9, n_samples=64, c=C,
              window_cull=False, precision=precision,
              out_dtype=np.complex128)
    field, dropped = coherent_cluttergram(p, UCT[None], c, n, a, e1, e2, **kw)
    assert not np.any(field)
    q = [np.asarray(v, np.float32).astype(np.float64) for v in (c, n, a, e1,
                                                               e2)]
    contrib, _ = lpa.lpa_field(p[0], *q, k, -0.3)
    np.testing.assert_allclose(dropped[0], (np.abs(contrib) ** 2).sum(),
                               rtol=1e-5)


def test_oversized_window_is_refused_not_truncated():
    """A per-trace histogram beyond the shared-memory budget is an error
    (ValueError), never a silently shortened window."""
    c, n, a, e1, e2 = _grid(ncell=4)
    p = np.array([[0.0, 0.0, 150.0]])
    with pytest.raises(ValueError):
        coherent_cluttergram(p, UCT[None], c, n, a, e1, e2,
                             k=2 * np.pi / 5.0, gamma=-0.3, t0=0.0, dt=1e-9,
                             n_samples=40000, c=C, precision="split")


@pytest.mark.parametrize("precision", PRECISIONS)
def test_ragged_sizes(precision):
    """Trace and facet counts that are not multiples of any block or tile."""
    c, n, a, e1, e2 = _grid(ncell=13)
    rng = np.random.default_rng(23)
    T = 7
    p = np.column_stack([rng.uniform(-10, 10, T), rng.uniform(-10, 10, T),
                         rng.uniform(140, 160, T)])
    kw = dict(k=2 * np.pi / 5.0, gamma=-0.3, t0=2 * 130.0 / C, dt=2e-9,
              n_samples=77, c=C, block_size=17)
    got, _ = coherent_cluttergram(p, np.tile(UCT, (T, 1)), c, n, a, e1, e2,
                                  **kw, precision=precision,
                                  out_dtype=np.complex128)
    ref, _ = lpa.coherent_cluttergram(p, np.tile(UCT, (T, 1)), c, n, a, e1,
                                      e2, **kw)
    tol = 1e-9 if precision == "fp64" else 1e-4
    assert np.linalg.norm(got - ref) <= tol * np.linalg.norm(ref)
