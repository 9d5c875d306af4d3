"""Shared helpers for the test-suite (fixture unpacking, error metrics)."""

from types import SimpleNamespace

import numpy as np


def facets_from(g, prefix):
    """Facets-like namespace from a golden fixture's ``<prefix>_*`` arrays."""
    return SimpleNamespace(
        centers=g[f"{prefix}_centers"], normals=g[f"{prefix}_normals"],
        areas=g[f"{prefix}_areas"], e1=g[f"{prefix}_e1"],
        e2=g[f"{prefix}_e2"], cell=g[f"{prefix}_cell"],
        grid_shape=tuple(int(v) for v in g[f"{prefix}_grid"]),
        phase_keys=None)


def rel_l2(a, b):
    """||a - b|| / ||b|| over all elements (complex-aware)."""
    a = np.asarray(a, np.complex128)
    b = np.asarray(b, np.complex128)
    den = np.linalg.norm(b.ravel())
    return float(np.linalg.norm((a - b).ravel()) / max(den, 1e-300))


def field_errors(test, ref, floor_db=-60.0):
    """The parity metrics: relative L2 of the complex traces, max phase error
    (rad) and max power error (dB) over bins within ``floor_db`` of the
    peak power (per trace set)."""
    test = np.asarray(test, np.complex128)
    ref = np.asarray(ref, np.complex128)
    p_ref = np.abs(ref) ** 2
    keep = p_ref > p_ref.max() * 10 ** (floor_db / 10.0)
    ph = np.abs(np.angle(test[keep] / ref[keep]))
    db = np.abs(10 * np.log10(np.abs(test[keep]) ** 2 / p_ref[keep]))
    return dict(rel_l2=rel_l2(test, ref),
                phase_rad=float(ph.max()) if ph.size else 0.0,
                power_db=float(db.max()) if db.size else 0.0)


def oracle_config2_target(j, traces, n_cells=512, n_traces=1024,
                          refraction=None):
    """Float64 oracle field and dropped power of target ``j`` (0 surface,
    1 first horizon, 2 second horizon, 3 bed) of the multilayer benchmark
    scene for the trace indices ``traces``. The scene is rebuilt from its
    seed here, so the function can run in a spawned worker process."""
    from oracle import lpa
    from oracle import refracted as oref
    from radar_sounder_simulator_gb300 import scenes
    cfg = scenes.config2(n_cells=n_cells, n_traces=n_traces)
    sel = np.asarray(traces)
    pos, uct = cfg.pos[sel], cfg.uct[sel]
    L = cfg.layers
    if j == 0:
        f = L[0]
        return lpa.coherent_cluttergram(
            pos, uct, f.centers, f.normals, f.areas, f.e1, f.e2, k=cfg.k0,
            gamma=cfg.gammas[0], t0=cfg.t0, dt=cfg.dt,
            n_samples=cfg.n_samples, c=cfg.c)
    refr = refraction or ("joint" if j > 1 else "sequential")
    return oref.refracted_cluttergram(
        pos, uct, L[j], L[:j], cfg.eps[:j + 1], cfg.att[:j + 1],
        mode="coherent", t0=cfg.t0, dt=cfg.dt, n_samples=cfg.n_samples,
        c=cfg.c, gamma=cfg.gammas[j], k0=cfg.k0, refraction=refr)
