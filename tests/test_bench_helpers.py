"""The benchmark's roofline and error arithmetic, on CPU: the canonical
per-pair FLOP counts the roofline divides by, and the split-vs-FP64 error
measures (relative L2, max phase and max dB over bins above -60 dB)."""

import numpy as np
import pytest
import torch

import bench


def test_canonical_pair_flops():
    # smooth pair (coherent.py:107-128 + binning), one sequential crossing
    # (35 Snell iterations of 20 + lookup / plane / Fresnel 60, radiometry),
    # and the joint path through three crossings at the default budgets
    assert bench.pair_flops(0, False) == 47.0
    assert bench.pair_flops(1, False) == 865.0
    assert bench.pair_flops(2, False) == 1650.0
    assert bench.pair_flops(3, True) == 11135.0
    assert bench.pair_flops(2, True) > 2 * bench.pair_flops(2, False)


def _field(T, B, seed):
    g = torch.Generator().manual_seed(seed)
    return torch.randn(T, B, 2, dtype=torch.float64, generator=g)


def test_split_error_measures():
    f = _field(4, 64, 0)
    zero = bench.split_error([(f, None)], [(f.clone(), None)])
    assert zero["rel_l2"] == 0.0
    assert zero["phase_rad"] < 1e-15 and zero["power_db"] < 1e-12
    # a pure phase rotation of 1e-3 rad: rel L2 ~ 1e-3, phase 1e-3, 0 dB
    c = torch.view_as_complex(f.contiguous())
    rot = torch.view_as_real(c * np.exp(1j * 1e-3))
    e = bench.split_error([(rot, None)], [(f, None)])
    assert e["rel_l2"] == pytest.approx(1e-3, rel=1e-3)
    assert e["phase_rad"] == pytest.approx(1e-3, rel=1e-6)
    assert e["power_db"] < 1e-9
    # a gain of 0.01 dB in amplitude squared on every bin
    g = 10 ** (0.01 / 20)
    e = bench.split_error([(f * g, None)], [(f, None)])
    assert e["power_db"] == pytest.approx(0.01, rel=1e-6)
    # the worst layer is reported
    e2 = bench.split_error([(f, None), (f * g, None)],
                           [(f, None), (f, None)])
    assert e2["power_db"] == pytest.approx(0.01, rel=1e-6)


def test_errors_ignore_bins_below_minus_60_db():
    b = torch.ones(8, dtype=torch.complex128)
    b[3] = 1e-4                      # -80 dB: outside the measured set
    a = b.clone()
    a[3] = -1e-4                     # pi rad off, but not counted
    e = bench._errors(a, b)
    assert e["phase_rad"] == 0.0 and e["power_db"] == 0.0
    assert e["rel_l2"] > 0.0


def test_plain_surface_cpu_baseline_and_row_guard():
    from radar_sounder_simulator_gb300 import scenes
    cfg = scenes.config1()
    cb = bench.cfg1_cpu_baseline(cfg, 0.01)      # one 8-trace slice
    assert cb["value"] > 0 and cb["cores"] == 1 and cb["kind"] == "port"
    assert cb["sample"].startswith("8 traces x 16384 facets")
    assert bench._cpu_or_error(lambda: cb, 0.0) is None
    err = bench._cpu_or_error(lambda: 1 / 0, 1.0)
    assert err["error"].startswith("ZeroDivisionError")


def test_mode_f_cpu_baseline_one_position():
    from radar_sounder_simulator_gb300 import scenes
    cfg = scenes.config1()
    tw = cfg.kw["t0"] + np.arange(64) * cfg.kw["dt"]
    # K = 1024 keeps the referee's alias guard satisfied (K/B > delay span)
    cb = bench.modef_cpu_baseline(cfg, tw, 1024, 1e-6)   # one position
    assert cb["value"] > 0 and cb["unit"] == "pair-frequencies/s"
    assert cb["sample"].startswith("1 positions x 16384 facets x 1024")


def test_roughness_cpu_baseline_one_trace():
    from radar_sounder_simulator_gb300 import scenes
    cfg = scenes.config3(n_cells=32, n_traces=8)
    f0 = 60e6
    dt = 1.0 / (2.0 * cfg.frac_bw * f0)
    k0 = 2 * np.pi * f0 / cfg.c
    n_s = 256
    t0 = scenes.window(cfg.pos, cfg.surface.centers, n_samples=n_s, dt=dt)
    band = dict(k0=k0, t0=t0, dt=dt, n_s=n_s, nt_s=15, nt_b=60)
    cb = bench.cfg3_cpu_baseline(cfg, band, 0.0)     # one trace
    assert cb["value"] > 0 and cb["unit"] == "contribs/s"
    assert cb["sample"].startswith("1 traces x 2048 facets (surface + bed) "
                                   "at 60 MHz")


def test_sweep_cpu_baseline_one_slice():
    cb = bench.cfg4_cpu_baseline(0.0)                  # one 8-trace slice
    assert cb["value"] > 0 and cb["unit"] == "contribs/s"
    assert cb["sample"].startswith("8 traces x ")


def test_summary_is_compact_and_carries_row_errors():
    import json
    import bench
    err = {"rel_l2": 1.234e-6, "phase_rad": 2.5e-4, "power_db": 3.1e-3}
    line = {"value": 8.0e9, "ms_per_step": 130.123, "error_vs_fp64": err,
            "roofline": {"frac": 0.5123},
            "rows": {"peaks_tflops": {"fp32": 78.0},
                     "cfg1": {"value": 1e10, "error_vs_fp64": err,
                              "roofline": {"frac": 0.1}},
                     "cfg3": {"value": 1e10, "bands": {
                         "450MHz": {"ms": 123.4, "error_vs_fp64": err,
                                    "roofline": {"frac": 0.2}}}},
                     "cfg5": {"value": 4e9, "fd_subset_max_rel_err": {
                         "reflectivity_db": 1e-5, "traces": 32}},
                     "broken": {"error": "RuntimeError: x" * 50}}}
    s = bench.summarize(line)
    assert s["headline"]["err"] == [1.23e-6, 2.5e-4, 3.1e-3]
    assert s["cfg3"]["bands"]["450MHz"]["err"][1] == 2.5e-4
    assert s["cfg5"]["fd"] == {"reflectivity_db": 1e-5}
    assert "peaks_tflops" not in s
    assert len(s["broken"]["error"]) <= 120
    assert len(json.dumps(s)) < 1200
