"""Batched refracted targets: one persistent work-queue launch for many
jobs of one path class (plus batched fix-up and reduce), against the float64
oracle per job and the one-call split form; the roughness configuration's
eight (target, band) jobs as one CUDA-graph replay against their per-call
results."""

import numpy as np
import pytest
import torch

from oracle import refracted as oref
from radar_sounder_simulator_gb300.batch import (BatchGraph, CoherentBatch,
                                                 RefractedBatch)
from radar_sounder_simulator_gb300.multilayer import prepare_refracted
from tests.test_oracle_golden import refracted_case
from tests.util import field_errors, rel_l2

pytestmark = pytest.mark.gpu


def _host(field):
    f = field.cpu().numpy()
    return f[..., 0] + 1j * f[..., 1]


def _jobs(g, cases, scale_k=(1.0,)):
    out = []
    for case in cases:
        for sk in scale_k:
            pos, uct, tgt, crossed, e, a, kw = refracted_case(g, case)
            kw = dict(kw)
            if "k0" in kw:
                kw["k0"] = kw["k0"] * sk
            out.append((pos, uct, tgt, crossed, e, a, kw))
    return out


def _check(jobs):
    plans = [prepare_refracted(*j[:6], **j[6], precision="split")
             for j in jobs]
    b = RefractedBatch(plans)
    outs = b.run()
    for j, p, (field, dropped) in zip(jobs, plans, outs):
        got = _host(field)
        ref, ref_drop = oref.refracted_cluttergram(*j[:6], **j[6])
        ref = ref.reshape(got.shape)
        e = field_errors(got, ref)
        assert e["rel_l2"] <= 1e-4 and e["phase_rad"] <= 1e-3 and \
            e["power_db"] <= 0.01, e
        one = _host(p.run()[0])
        assert rel_l2(got, one) <= 1e-5
        np.testing.assert_allclose(dropped.cpu().numpy(), ref_drop,
                                   rtol=1e-3, atol=1e-6 * np.abs(ref).max()
                                   ** 2)
    return b


def test_sequential_batch(golden):
    g = golden("refracted")
    b = _check(_jobs(g, ["seq1", "seq2"], scale_k=(1.0, 1.5)))
    assert b.info.n_jobs == 4 and b.info.path_class == 0


def test_joint_batch(golden):
    g = golden("refracted")
    b = _check(_jobs(g, ["joint2"], scale_k=(1.0, 0.7, 1.3)))
    assert b.info.path_class == 2


def test_mixed_path_classes_are_refused(golden):
    g = golden("refracted")
    jobs = _jobs(g, ["seq1", "joint2"])
    plans = [prepare_refracted(*j[:6], **j[6], precision="split")
             for j in jobs]
    with pytest.raises(ValueError):
        RefractedBatch(plans)


def test_roughness_configuration_bands_in_one_replay():
    """The roughness configuration's surface and bed in all four bands
    (central 16 traces): one CoherentBatch (four rough surface jobs) and one
    RefractedBatch (four rough bed jobs) captured in one CUDA graph; every
    job equals its per-call split result and the FP64 form within the
    parity bounds."""
    from radar_sounder_simulator_gb300 import scenes
    from radar_sounder_simulator_gb300.coherent import prepare_coherent
    cfg = scenes.config3()
    s, bd = cfg.surface, cfg.bed
    rs, rb = cfg.rough["surface"], cfg.rough["bed"]
    mid = len(cfg.pos) // 2
    sel = slice(mid - 8, mid + 8)
    pos, uct = cfg.pos[sel], cfg.uct[sel]
    surf_plans, bed_plans = [], []
    for f0 in cfg.bands:
        band = scenes.config3_band(cfg, f0)
        common = dict(t0=band["t0"], dt=band["dt"], n_samples=band["n_s"],
                      c=cfg.c, d_phi_area=True, taper_s=0.05,
                      precision="split", device="cuda")
        surf_plans.append(prepare_coherent(
            pos, uct, s.centers, s.normals, s.areas, s.e1, s.e2,
            k=band["k0"], gamma=cfg.gamma_surface,
            roughness=(rs["sigma"], rs["corr"], rs["phasors"], band["nt_s"],
                       "exponential"), **common))
        bed_plans.append(prepare_refracted(
            pos, uct, bd, [s], cfg.eps, cfg.att, mode="coherent",
            gamma=cfg.gamma_bed, k0=band["k0"],
            roughness=(rb["sigma"], rb["corr"], rb["phasors"], band["nt_b"],
                       "exponential"), refraction="sequential", **common))
    cb = CoherentBatch(surf_plans)
    rbt = RefractedBatch(bed_plans)
    graph = BatchGraph([cb.run, rbt.run])
    graph.capture()
    for o in cb.outputs + rbt.outputs:
        o[0].zero_()
    graph.replay()
    torch.cuda.synchronize()
    for plans, outs in ((surf_plans, cb.outputs), (bed_plans, rbt.outputs)):
        for p, (field, _) in zip(plans, outs):
            got = _host(field)
            one = _host(p.run()[0])
            assert rel_l2(got, one) <= 1e-5
            e = field_errors(got, _host(p.run("fp64")[0]))
            assert e["rel_l2"] <= 1e-4 and e["phase_rad"] <= 1e-3 and \
                e["power_db"] <= 0.01, e
