"""The device form of the culling plan (stable sort and window searches on
the GPU) gives the host plan's permutation and windows exactly: ties keep
index order, -0.0 sorts with +0.0, as NumPy's stable argsort does."""

import numpy as np
import pytest

from radar_sounder_simulator_gb300.geometry import cull_plan

pytestmark = pytest.mark.gpu
C = 299792458.0


def _both(pos, cen, **kw):
    h = cull_plan(pos, cen, **kw)
    d = cull_plan(pos, cen, device="cuda", **kw)
    return h, d


@pytest.mark.parametrize("bs", [None, 64, 4096])
def test_device_plan_equals_host_plan(golden, bs):
    g = golden("coherent")
    pos, cen = g["pos"], g["surf_centers"]
    h, d = _both(pos, cen, t0=2 * 1400.0 / C, dt=1e-8, n_samples=64, c=C,
                 block_size=bs, target_pairs=1 << 12)
    np.testing.assert_array_equal(d.order.cpu().numpy(), h.order)
    np.testing.assert_array_equal(d.off, h.off)
    assert (d.block_size, d.n_blocks, d.n_win) == (h.block_size, h.n_blocks,
                                                  h.n_win)


def test_ties_and_signed_zero_keep_index_order():
    rng = np.random.default_rng(2)
    n = 5000
    x = rng.integers(-20, 20, n).astype(np.float64)   # many exact ties
    x[::97] = -0.0
    x[1::97] = 0.0
    cen = np.column_stack([x, rng.uniform(-5, 5, n), np.zeros(n)])
    pos = np.column_stack([np.linspace(-30, 30, 9), np.zeros(9),
                           np.full(9, 100.0)])
    for wc in (True, False):
        h, d = _both(pos, cen, t0=2 * 90.0 / C, dt=1e-8, n_samples=32, c=C,
                     block_size=128, target_pairs=1 << 12, window_cull=wc)
        np.testing.assert_array_equal(d.order.cpu().numpy(), h.order)
        np.testing.assert_array_equal(d.off, h.off)
        assert d.n_win == h.n_win


def test_regrouping_within_blocks_matches_host(golden):
    """Facets regrouped by a per-facet key inside each culling block: the
    device permutation equals the host one, and block membership (every
    trace's window) is unchanged."""
    from radar_sounder_simulator_gb300.geometry import group_within_blocks
    g = golden("coherent")
    pos, cen = g["pos"], g["surf_centers"]
    kw = dict(t0=2 * 1400.0 / C, dt=1e-8, n_samples=64, c=C, block_size=64,
              target_pairs=1 << 12)
    key = np.random.default_rng(3).lognormal(0, 1, len(cen))
    key[::7] = key[0]                      # ties keep their order
    h = group_within_blocks(cull_plan(pos, cen, **kw), key)
    d = group_within_blocks(cull_plan(pos, cen, device="cuda", **kw), key)
    np.testing.assert_array_equal(d.order.cpu().numpy(), h.order)
    base = cull_plan(pos, cen, **kw).order
    for b in range(0, len(base), 64):
        assert set(h.order[b:b + 64]) == set(base[b:b + 64])
