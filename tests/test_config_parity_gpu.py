"""GPU parity at the benchmark configurations' own sizes.

The golden cases are small scenes (16^2-20^2 facets, a few traces). These
tests run the two configurations the split form is measured on, at their
full size:

* the multilayer scene (surface, horizons at 300 m and 1200 m, bed at
  2500 m; 512^2 facets of 50 m each; 20 km altitude; 60 MHz): the FP64 form
  against the float64 oracle on two traces of every target (<= 1e-9 of the
  peak per bin, the same occupied bins, dropped power to 1e-5), and the
  split form against the FP64 form on 64 traces (relative L2 <= 1e-4, phase
  <= 1e-3 rad, power <= 0.01 dB over bins above -60 dB of the target's
  peak, the same occupied bins);
* the same scene with the horizons and the bed reached by the sequential
  chain (two and three crossings, which the joint solve otherwise serves):
  split against FP64 with equal bins and relative L2 <= 1e-4, phase and
  power to the looser bound stated in that test;
* the roughness configuration (rough surface and a rough bed under 1000 m
  of ice, 512^2 facets of 25 m, per-facet log-normal rms heights,
  exponential ACF with the area-only series and taper) in each of its four
  bands on the central 32 of its 2048 traces: split against FP64 for both
  targets to the same bounds.
"""

import multiprocessing as mp
from concurrent.futures import ProcessPoolExecutor

import numpy as np
import pytest
import torch

from tests.util import field_errors, oracle_config2_target

pytestmark = pytest.mark.gpu

ORACLE_TRACES = (311, 702)


@pytest.fixture(scope="module")
def cfg2():
    from radar_sounder_simulator_gb300 import scenes
    return scenes.config2()


def _plan(cfg, j, pos, uct, precision, refraction=None):
    from radar_sounder_simulator_gb300.coherent import prepare_coherent
    from radar_sounder_simulator_gb300.multilayer import prepare_refracted
    L = cfg.layers
    if j == 0:
        f = L[0]
        return prepare_coherent(
            pos, uct, f.centers, f.normals, f.areas, f.e1, f.e2, k=cfg.k0,
            gamma=cfg.gammas[0], t0=cfg.t0, dt=cfg.dt,
            n_samples=cfg.n_samples, c=cfg.c, precision=precision,
            device="cuda")
    refr = refraction or ("joint" if j > 1 else "sequential")
    return prepare_refracted(
        pos, uct, L[j], L[:j], cfg.eps[:j + 1], cfg.att[:j + 1],
        mode="coherent", t0=cfg.t0, dt=cfg.dt, n_samples=cfg.n_samples,
        c=cfg.c, gamma=cfg.gammas[j], k0=cfg.k0, refraction=refr,
        precision=precision, device="cuda")


def _host(field):
    f = field.cpu().numpy()
    return f[..., 0] + 1j * f[..., 1]


def _occupied(a, b):
    """Bins that either form fills above 1e-12 of the peak amplitude: rough
    facets whose roughness series underflows float32 leave float64 bins of
    1e-15 to 1e-90 of the peak that the split form holds as exact zeros
    (a misbinned pair moves far more than 1e-12 of the peak)."""
    floor = 1e-12 * np.abs(b).max()
    return np.abs(a) > floor, np.abs(b) > floor


def _check_split(a, b, what, phase=1e-3, power=0.01):
    err = field_errors(a, b)
    oa, ob = _occupied(a, b)
    assert np.array_equal(oa, ob), (what, "occupied bins differ")
    assert err["rel_l2"] <= 1e-4, (what, err)
    assert err["phase_rad"] <= phase, (what, err)
    assert err["power_db"] <= power, (what, err)
    return err


def test_config2_fp64_vs_oracle_full_size(cfg2):
    """FP64 form of all four targets against the float64 oracle, two traces
    of the full 512^2 x 4 scene (the oracle runs in spawned workers)."""
    sel = np.asarray(ORACLE_TRACES)
    ctx = mp.get_context("spawn")
    with ProcessPoolExecutor(max_workers=8, mp_context=ctx) as ex:
        futs = {(j, t): ex.submit(oracle_config2_target, j, [t])
                for j in range(4) for t in ORACLE_TRACES}
        ref = {k: f.result() for k, f in futs.items()}
    for j in range(4):
        plan = _plan(cfg2, j, cfg2.pos[sel], cfg2.uct[sel], "fp64")
        field, dropped = plan.run()
        got = _host(field)
        want = np.concatenate([ref[(j, t)][0] for t in ORACLE_TRACES])
        want_drop = np.concatenate([ref[(j, t)][1] for t in ORACLE_TRACES])
        scale = np.abs(want).max()
        assert scale > 0
        assert np.array_equal(got != 0, want != 0), (j, "occupied bins")
        assert np.abs(got - want).max() <= 1e-9 * scale, j
        np.testing.assert_allclose(dropped.cpu().numpy(), want_drop,
                                   rtol=1e-5, atol=1e-9 * scale ** 2)


def test_config2_split_vs_fp64_64_traces(cfg2):
    """Split form against the FP64 form on 64 traces of every target."""
    sel = slice(480, 544)
    for j in range(4):
        plan = _plan(cfg2, j, cfg2.pos[sel], cfg2.uct[sel], "split")
        a = _host(plan.run()[0])
        b = _host(plan.run("fp64")[0])
        _check_split(a, b, cfg2.names[j])


@pytest.mark.parametrize("j", [2, 3])
def test_config2_sequential_chain_split_vs_fp64(cfg2, j):
    """The second horizon (two crossings) and the bed (three) by the
    sequential chain, whose upper crossings are not stationary: split bins
    equal the FP64 form's and relative L2 is within 1e-4 on 64 traces. The
    upper crossings' float32 in-plane error (~mm) reaches each pair's
    amplitude at first order (~7e-6 relative, median), which deep speckle
    fades raise to 3-5e-3 rad and 0.036 dB in their weakest bins above
    -60 dB; this path is held to 1e-2 rad and 0.05 dB. The benchmark
    scenes reach targets under two or more interfaces by the joint solve,
    which meets the 1e-3 rad / 0.01 dB bound."""
    sel = slice(480, 544)
    plan = _plan(cfg2, j, cfg2.pos[sel], cfg2.uct[sel], "split",
                 refraction="sequential")
    a = _host(plan.run()[0])
    b = _host(plan.run("fp64")[0])
    _check_split(a, b, f"{cfg2.names[j]} sequential", phase=1e-2,
                 power=0.05)


@pytest.fixture(scope="module")
def cfg3():
    from radar_sounder_simulator_gb300 import scenes
    return scenes.config3()


@pytest.mark.parametrize("f0", [30e6, 60e6, 150e6, 450e6])
def test_config3_band_split_vs_fp64(cfg3, f0):
    """Rough surface and rough bed of one band of the roughness
    configuration, central 32 traces, split against FP64."""
    from radar_sounder_simulator_gb300 import scenes
    from radar_sounder_simulator_gb300.coherent import prepare_coherent
    from radar_sounder_simulator_gb300.multilayer import prepare_refracted
    band = scenes.config3_band(cfg3, f0)
    s, b = cfg3.surface, cfg3.bed
    rs, rb = cfg3.rough["surface"], cfg3.rough["bed"]
    mid = len(cfg3.pos) // 2
    sel = slice(mid - 16, mid + 16)
    pos, uct = cfg3.pos[sel], cfg3.uct[sel]
    common = dict(t0=band["t0"], dt=band["dt"], n_samples=band["n_s"],
                  c=cfg3.c, d_phi_area=True, taper_s=0.05, precision="split",
                  device="cuda")
    ps = prepare_coherent(
        pos, uct, s.centers, s.normals, s.areas, s.e1, s.e2, k=band["k0"],
        gamma=cfg3.gamma_surface,
        roughness=(rs["sigma"], rs["corr"], rs["phasors"], band["nt_s"],
                   "exponential"), **common)
    pb = prepare_refracted(
        pos, uct, b, [s], cfg3.eps, cfg3.att, mode="coherent",
        gamma=cfg3.gamma_bed, k0=band["k0"],
        roughness=(rb["sigma"], rb["corr"], rb["phasors"], band["nt_b"],
                   "exponential"), refraction="sequential", **common)
    for name, p in (("surface", ps), ("bed", pb)):
        a = _host(p.run()[0])
        bb = _host(p.run("fp64")[0])
        _check_split(a, bb, f"{f0 / 1e6:.0f} MHz {name}")
    torch.cuda.synchronize()
