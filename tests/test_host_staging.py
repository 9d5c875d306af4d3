"""Host staging of the drop-in, run on CPU tensors: the culling plan, the
float32 facet records in culling order, the refraction lookup constants and
the joint solve's padding planes, each against the oracle (which restates
kernels/coherent.py:284-301 and kernels/multilayer.py:269-330). The staging
code is the same on a CUDA device; only the kernels need a GPU."""

import numpy as np
import pytest
import torch

from oracle import geometry as ogeom
from oracle import refracted as oref
from radar_sounder_simulator_gb300.coherent import prepare_coherent
from radar_sounder_simulator_gb300.geometry import cull_plan
from radar_sounder_simulator_gb300.multilayer import (grid_consts_device,
                                                      prepare_refracted)
from radar_sounder_simulator_gb300.scenes import (facets_from_vertices,
                                                  random_field)

C = 299792458.0


def _surface(n, d, z0, rms, seed):
    ax = np.arange(n + 1) * d - n * d / 2
    X, Y = np.meshgrid(ax, ax)
    Z = z0 + random_field(n + 1, d, 8 * d, rms, np.random.default_rng(seed))
    return facets_from_vertices(X, Y, Z)


def _track(T, z, dx=7.0, tilt=0.3):
    s = np.arange(T) * dx - T * dx / 2
    pos = np.column_stack([s, tilt * s + 3.0, np.full(T, z)])
    u = np.tile([0.0, -1.0, 0.0], (T, 1))
    return pos, u


@pytest.mark.parametrize("bs,t0,ns,cull", [
    (64, 2 * 480.0 / C, 32, True), (None, 2 * 450.0 / C, 128, True),
    (100, 0.0, 16, True), (64, 2 * 480.0 / C, 32, False)])
def test_cull_plan_matches_oracle(bs, t0, ns, cull):
    f = _surface(32, 10.0, 0.0, 2.0, 3)
    pos, _ = _track(40, 500.0)
    kw = dict(t0=t0, dt=1e-8, n_samples=ns, c=C, block_size=bs,
              target_pairs=1 << 12, window_cull=cull)
    got = cull_plan(pos, f.centers, **kw)
    order, b, nb, off, nw = ogeom.culling_plan(pos, f.centers, **kw)
    np.testing.assert_array_equal(got.order, order)
    assert (got.block_size, got.n_blocks, got.n_win) == (b, nb, nw)
    np.testing.assert_array_equal(got.off, off)


def test_staged_facets_are_float32_records_in_cull_order():
    f = _surface(24, 12.0, 0.0, 3.0, 5)
    pos, u = _track(16, 600.0)
    n = len(f.centers)
    gam = np.random.default_rng(2).uniform(-0.5, -0.1, n)
    sig = np.random.default_rng(3).lognormal(-1.0, 0.5, n)
    ph = np.exp(1j * np.random.default_rng(4).uniform(0, 6.3, n))
    plan = prepare_coherent(pos, u, f.centers, f.normals, f.areas, f.e1,
                            f.e2, k=1.2, gamma=gam, t0=2 * 560.0 / C,
                            dt=1e-8, n_samples=64, c=C,
                            roughness=(sig, np.full(n, 5.0), ph, 30),
                            device="cpu")
    order = plan.cull.order
    assert sorted(order) == list(range(n))
    fac = plan.keep[0]
    want = np.concatenate([f.centers, f.normals, f.e1, f.e2,
                           f.areas[:, None]], 1).astype(np.float32)[order].T
    np.testing.assert_array_equal(fac.soa.numpy(), want)
    ex = fac.extras
    np.testing.assert_array_equal(ex["gamma_f32"].numpy(),
                                  gam.astype(np.float32)[order])
    np.testing.assert_array_equal(ex["sigma"].numpy(),
                                  sig.astype(np.float32)[order])
    np.testing.assert_array_equal(
        ex["phasor"].numpy().view(np.complex64),
        ph.astype(np.complex64)[order])
    # per-facet rms heights regroup facets inside each culling block only
    base = cull_plan(pos, f.centers, t0=2 * 560.0 / C, dt=1e-8,
                     n_samples=64, c=C, block_size=None,
                     target_pairs=1 << 19).order
    bs = plan.cull.block_size
    for b in range(0, n, bs):
        assert set(order[b:b + bs]) == set(base[b:b + bs])


def test_lookup_constants_match_oracle():
    for f in (_surface(20, 25.0, 0.0, 4.0, 7),
              _surface(16, 40.0, -300.0, 1.0, 8)):
        tab, coef, mp, mn = grid_consts_device(f, torch.device("cpu"))
        gc, gn, ocoef, omp, omn = oref.grid_consts(f)
        np.testing.assert_array_equal(tab[..., :3].numpy(), gc)
        np.testing.assert_array_equal(tab[..., 3:].numpy(), gn)
        # normal equations of the centred frame vs the SVD least squares
        np.testing.assert_allclose(coef, ocoef, rtol=0, atol=1e-9)
        np.testing.assert_allclose(mp, omp, rtol=1e-13, atol=1e-9)
        np.testing.assert_allclose(mn, omn, rtol=0, atol=1e-14)


def test_joint_padding_planes_match_oracle():
    surf = _surface(12, 20.0, 0.0, 2.0, 9)
    h1 = _surface(12, 20.0, -40.0, 1.0, 10)
    bed = _surface(12, 20.0, -90.0, 3.0, 11)
    pos, u = _track(6, 400.0)
    for pad in (2, 4, 8):
        plan = prepare_refracted(pos, u, bed, [surf, h1], [1.0, 2.0, 3.15],
                                 [0.0, 5.0, 10.0], mode="incoherent",
                                 t0=0.0, dt=1e-8, n_samples=128, c=C,
                                 refraction="joint", pad_to=pad,
                                 device="cpu")
        gc, gn, coef, shp, mp, mn, k = oref.joint_consts(
            [surf, h1], pad, pos[:, 2].min())
        o = plan.opts
        assert (o.n_crossed, o.k_pad, o.n_legs) == (pad, k, pad + 1)
        for j in range(pad):
            it = plan.ifaces[j]
            np.testing.assert_allclose(list(it.mean_point), mp[j],
                                       rtol=1e-13, atol=1e-9)
            np.testing.assert_allclose(list(it.mean_normal), mn[j],
                                       atol=1e-14)
            tab = plan.keep[1][j].numpy()
            if j < k:       # no-op air planes: one flat cell at the height
                assert (it.ny, it.nx) == (1, 1)
                np.testing.assert_array_equal(tab[0, 0, :3], gc[j, 0, 0])
                np.testing.assert_array_equal(tab[0, 0, 3:], gn[j, 0, 0])
            else:
                assert (it.ny, it.nx) == tuple(shp[j])
                np.testing.assert_array_equal(tab[..., :3], gc[j])
                np.testing.assert_array_equal(tab[..., 3:], gn[j])
                np.testing.assert_allclose(
                    np.array(list(it.coef)).reshape(3, 2), coef[j], rtol=0,
                    atol=1e-9)
        n_leg = np.ctypeslib.as_array(o.n_leg, (o.n_legs,))
        np.testing.assert_array_equal(
            n_leg, np.sqrt([1.0] * k + [1.0, 2.0, 3.15]))
