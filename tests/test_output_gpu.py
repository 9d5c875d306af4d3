"""GPU per-trace output products (ss_trace_products through
radar_sounder_simulator_gb300.output) against the reference's outputs and
the oracle: integer results (facet indices) and the float64 twtts are
exact -- the screen only decides which pairs are evaluated in float64, in
the reference's operation order, and ties go to the first facet."""

import sys
import types

import numpy as np
import pytest

from oracle import output as oo
from radar_sounder_simulator_gb300 import output as go

pytestmark = pytest.mark.gpu
C = 299792458.0


def test_products_match_reference(golden):
    g = golden("output")
    r = go.trace_products(g["surf_centers"], g["pos"], t0=float(g["t0"]),
                          dt=float(g["dt"]), n_samples=int(g["n_samples"]),
                          c=C)
    np.testing.assert_array_equal(r["nadir_twtt"], g["nadir_twtt"])
    np.testing.assert_array_equal(r["first_twtt"], g["first_return_twtt"])
    c = g["surf_centers"]
    np.testing.assert_array_equal(c[r["first_index"], 0],
                                  g["first_return_lat"])
    assert r["first_index"][-1] == 0 and np.isinf(r["first_twtt"][-1])


@pytest.mark.parametrize("dup", [False, True])
def test_products_match_oracle_with_ties(dup):
    """A larger ragged case, optionally with every centre duplicated so the
    first-index tie rule decides both products."""
    rng = np.random.default_rng(5)
    n = 30011
    cen = np.column_stack([rng.uniform(-3000, 3000, n),
                           rng.uniform(-3000, 3000, n),
                           rng.normal(0, 30, n)])
    if dup:
        cen = np.repeat(cen, 2, axis=0)[: n + 7]
    T = 37
    pos = np.column_stack([np.linspace(-2500, 2500, T),
                           rng.uniform(-100, 100, T), np.full(T, 1500.0)])
    kw = dict(t0=2 * 1480.0 / C, dt=1.0 / 30e6, n_samples=300, c=C)
    r = go.trace_products(cen, pos, **kw)
    nt, ni, ft, fi = oo.trace_products(cen, pos, kw["t0"], kw["dt"],
                                       kw["n_samples"], C)
    np.testing.assert_array_equal(r["nadir_index"], ni)
    np.testing.assert_array_equal(r["nadir_twtt"], nt)
    np.testing.assert_array_equal(r["first_index"], fi)
    np.testing.assert_array_equal(r["first_twtt"], ft)


def test_build_dataset_through_xarray_stand_in(golden, monkeypatch):
    from tests.golden import xrshim
    monkeypatch.setitem(sys.modules, "xarray", xrshim.install())
    g = golden("output")
    T, n_s = len(g["pos"]), int(g["n_samples"])
    radar = types.SimpleNamespace(
        c=C, t0=float(g["t0"]), dt=float(g["dt"]), f0=60e6,
        wavelength=C / 60e6, waveform=types.SimpleNamespace(kind="delta"))
    cfg = types.SimpleNamespace(radar=radar, mode="coherent",
                                model_dump_json=lambda: "{}")
    scene = types.SimpleNamespace(nav_llh=g["pos"], name="golden",
                                  crs="local", params={})
    frame = types.SimpleNamespace(lat0=0.0, lon0=0.0, h0=0.0,
                                  local_to_llh=lambda enu: np.asarray(enu))
    facets = types.SimpleNamespace(centers=g["surf_centers"])
    ds = go.build_dataset(np.zeros((T, n_s), np.float32), np.zeros(T),
                          scene=scene, frame=frame, facets=facets,
                          track=types.SimpleNamespace(positions=g["pos"]),
                          sim_config=cfg,
                          field=np.zeros((T, n_s), np.complex64))
    for k in ("nadir_twtt", "first_return_twtt", "first_return_lat",
              "first_return_lon"):
        np.testing.assert_array_equal(ds[k].values, g[k], err_msg=k)
    assert ds.attrs["wavelength"] == C / 60e6 and "field" in ds


def test_window_edges_decided_in_float64():
    """Facets a few millimetres either side of the window's start and end
    (inside the screen's uncertain bands) next to facets well inside: the
    first return is the earliest facet truly in the window."""
    rng = np.random.default_rng(6)
    p = np.array([[0.0, 0.0, 1500.0]])
    t0, dt, n_s = 2 * 1990.0 / C, 1e-8, 40
    r_start, r_end = C * t0 / 2, C * (t0 + n_s * dt) / 2
    rs = np.concatenate([r_start + rng.uniform(-5e-3, 5e-3, 200),
                         r_end + rng.uniform(-5e-3, 5e-3, 200),
                         rng.uniform(r_start + 1.0, r_end - 1.0, 50)])
    az = rng.uniform(0, 2 * np.pi, len(rs))
    h = np.sqrt(rs ** 2 - (1500.0 - 10.0) ** 2)
    cen = np.column_stack([h * np.cos(az), h * np.sin(az),
                           np.full(len(rs), 10.0)])
    kw = dict(t0=t0, dt=dt, n_samples=n_s, c=C)
    r = go.trace_products(cen, p, **kw)
    nt, ni, ft, fi = oo.trace_products(cen, p, t0, dt, n_s, C)
    np.testing.assert_array_equal(r["first_index"], fi)
    np.testing.assert_array_equal(r["first_twtt"], ft)
    np.testing.assert_array_equal(r["nadir_index"], ni)
