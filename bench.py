"""Benchmark: facet.trace contributions/s of the coherent facet path on
GB300, multilayer refraction configuration (surface + 2 horizons + bed, 512^2
facets of 50 m each, 1024 traces at 20 km, 60 MHz / 15 MHz).

One step = the whole forward pass over that scene: the surface coherent sum
plus the three refracted targets (first horizon sequential, second horizon
and bed joint), split-precision form, inputs resident in HBM, L2 flushed
before every step. Also measured: the float64 form's rate (``fp64``), the
drop-in NumPy-in/NumPy-out path with host copies in the timed region
(``e2e``), the split form's error against the float64 form, the dominant
kernel's roofline position and a CPU baseline.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
"""

import argparse
import json
import os
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = ("facet·trace contribs/s, split-FP32 vs FP64 GPU form, at "
          "≤0.01 dB vs FP64")
UNIT = "contribs/s"
WORKLOAD = "multilayer_refraction_512sq_x4_1024tr"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--n-cells", type=int, default=512)
    ap.add_argument("--n-traces", type=int, default=1024)
    ap.add_argument("--cpu-seconds", type=float, default=15.0,
                    help="host time of the headline's CPU baseline; the "
                         "one-core baselines of the plain-surface, Mode F, "
                         "roughness and sweep rows take at most 5 s each "
                         "and 0 skips them (the smaller rows time a fixed "
                         "small sample)")
    ap.add_argument("--skip-fp64", action="store_true",
                    help="skip the float64-form step and the error check")
    ap.add_argument("--skip-e2e", action="store_true",
                    help="skip the drop-in (host buffers) step")
    ap.add_argument("--traffic", type=float, default=188.2e6,
                    help="DRAM bytes per launch of the dominant kernel from "
                         "an ncu capture of the same workload (reported in "
                         "the roofline object; default: the one-pass capture "
                         "of the bed launch at the default size)")
    ap.add_argument("--rows",
                    default="cfg1,modef,cfg3,cfg4,cfg5,incoh,focus,scene,"
                            "output",
                    help="secondary workloads measured after the headline "
                         "(comma list, or 'none')")
    ap.add_argument("--batch-instances", type=int, default=96)
    ap.add_argument("--kernel-only", default=None,
                    choices=["surface", "h1", "h2", "bed", "rough450",
                             "plain128", "compress"],
                    help="run only this target -- a multilayer-scene "
                         "target, the rough bed at 450 MHz, the plain 128^2 "
                         "surface's facet sum or its pulse compression "
                         "(warm-up + steps launches, for profiling) -- and "
                         "print its mean time")
    ap.add_argument("--fp64-traces", type=int, default=256,
                    help="traces of the float64-form step (its rate is per "
                         "pair; the error check covers these traces)")
    return ap.parse_args()


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def line_offset(rank):
    """Cross-track offset of rank ``rank``'s flight line (m): each GPU flies
    its own line over the shared scene, so ranks share no work and no
    exchange (weak scaling, no collective on the data path)."""
    return 200.0 * rank


def max_over_ranks(ms, device, ws):
    """The slowest rank's step time (the job's time); identity at ws = 1."""
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(ms)], dtype=torch.float64, device=device)
    if ws > 1:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_rate(pairs_per_rank, ws, ms_max):
    """Whole-job contributions/s: every rank's pairs over the slowest
    rank's time."""
    return pairs_per_rank * ws / (ms_max * 1e-3)


def config_dict(args, ws):
    return {"workload": WORKLOAD, "layers": 4,
            "facets_per_layer": args.n_cells ** 2, "facet_m": 50.0,
            "traces_per_gpu": args.n_traces, "n_samples": 2048,
            "f0_hz": 60e6, "bandwidth_hz": 15e6,
            "refraction": "joint for targets under >= 2 interfaces",
            "l2": "flushed before every step (256 MiB write)",
            "parallelism": f"independent lines x{ws}"}


# --------------------------------------------------------------------------
# workload
# --------------------------------------------------------------------------
def build_plans(cfg, precision, device):
    """Device-resident plans for the four targets of one step."""
    from radar_sounder_simulator_gb300.coherent import prepare_coherent
    from radar_sounder_simulator_gb300.multilayer import prepare_refracted
    L = cfg.layers
    plans = [prepare_coherent(
        cfg.pos, cfg.uct, L[0].centers, L[0].normals, L[0].areas, L[0].e1,
        L[0].e2, k=cfg.k0, gamma=cfg.gammas[0], t0=cfg.t0, dt=cfg.dt,
        n_samples=cfg.n_samples, c=cfg.c, precision=precision,
        device=device)]
    for j in range(1, 4):
        refr = cfg.refraction if j > 1 else "sequential"
        plans.append(prepare_refracted(
            cfg.pos, cfg.uct, L[j], L[:j], cfg.eps[:j + 1], cfg.att[:j + 1],
            mode="coherent", t0=cfg.t0, dt=cfg.dt, n_samples=cfg.n_samples,
            c=cfg.c, gamma=cfg.gammas[j], k0=cfg.k0, refraction=refr,
            precision=precision, device=device))
    return plans


def drop_in_step(cfg, precision, device):
    """The reference-facing call sequence with host buffers (e2e)."""
    from radar_sounder_simulator_gb300.coherent import coherent_cluttergram
    from radar_sounder_simulator_gb300.multilayer import refracted_cluttergram
    L = cfg.layers
    outs = [coherent_cluttergram(
        cfg.pos, cfg.uct, L[0].centers, L[0].normals, L[0].areas, L[0].e1,
        L[0].e2, k=cfg.k0, gamma=cfg.gammas[0], t0=cfg.t0, dt=cfg.dt,
        n_samples=cfg.n_samples, c=cfg.c, precision=precision,
        device=device)]
    for j in range(1, 4):
        refr = cfg.refraction if j > 1 else "sequential"
        outs.append(refracted_cluttergram(
            cfg.pos, cfg.uct, L[j], L[:j], cfg.eps[:j + 1], cfg.att[:j + 1],
            mode="coherent", t0=cfg.t0, dt=cfg.dt, n_samples=cfg.n_samples,
            c=cfg.c, gamma=cfg.gammas[j], k0=cfg.k0, refraction=refr,
            precision=precision, device=device))
    return outs


def host_bytes(cfg):
    """Bytes the drop-in path copies host->device and device->host per
    step (counted from the arrays it uploads and downloads)."""
    T = len(cfg.pos)
    h2d = d2h = 0
    for j, f in enumerate(cfg.layers):
        n = len(f.centers)
        h2d += 13 * 8 * n + 8 * n               # float64 facet arrays + order
        h2d += T * (3 * 8 * 2 + 4)              # positions, u_ct, windows
        if j > 0 and np.ndim(cfg.gammas[j]):
            h2d += 8 * n                        # per-facet gamma
        for g in cfg.layers[:j]:
            h2d += 72 * len(g.centers)          # centres, normals, areas,
            #                                     cells of crossed interfaces
        d2h += T * cfg.n_samples * 8 + T * 8    # complex64 field + dropped
    return h2d, d2h


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during a region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,"
              "clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}",
                 f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE,
                stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *exc):
        self.rows = []
        if self.proc is None:
            return False
        self.proc.terminate()
        try:
            out, _ = self.proc.communicate(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
            out, _ = self.proc.communicate()
        for line in out.splitlines():
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 9:
                self.rows.append(parts)
        return False

    def summary(self):
        if not getattr(self, "rows", None):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [],
                    "samples": 0}
        sm = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown",
                 "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows for i in range(4)
                          if r[5 + i].lower().startswith("active")})
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "samples": len(self.rows)}


# --------------------------------------------------------------------------
# CPU baseline / reference arm: the reference formulas restated in C++17
# (float64, OpenMP over traces, every host core), test infrastructure under
# oracle/ and pinned there to the NumPy oracle and the reference fixtures
# --------------------------------------------------------------------------
CPU_KIND_NOTE = ("reference formulas, host restatement: C++17 OpenMP "
                 "float64 (oracle/cpu_ref.cpp), the reference's JAX CPU "
                 "path being unavailable (jax is not installed)")


def cpu_batch(cfg, sel):
    """One sample batch: the traces ``sel`` through all four targets of the
    multilayer scene on the host restatement. Returns the pairs done."""
    from oracle import cpu_ref
    L = cfg.layers
    pairs = 0
    for j in range(4):
        if j == 0:
            f = L[0]
            cpu_ref.coherent_cluttergram(
                cfg.pos[sel], cfg.uct[sel], f.centers, f.normals, f.areas,
                f.e1, f.e2, k=cfg.k0, gamma=cfg.gammas[0], t0=cfg.t0,
                dt=cfg.dt, n_samples=cfg.n_samples, c=cfg.c)
        else:
            cpu_ref.refracted_cluttergram(
                cfg.pos[sel], cfg.uct[sel], L[j], L[:j], cfg.eps[:j + 1],
                cfg.att[:j + 1], mode="coherent", t0=cfg.t0, dt=cfg.dt,
                n_samples=cfg.n_samples, c=cfg.c, gamma=cfg.gammas[j],
                k0=cfg.k0, refraction=cfg.refraction if j > 1
                else "sequential")
        pairs += len(L[j].centers) * len(sel)
    return pairs


def cpu_sample_rate(cfg, seconds, start=0):
    """Host restatement pairs/s on a bounded sample of the benchmark
    workload: batches of seeded trace picks (one trace per thread at
    least), each through all four whole targets, until about ``seconds``
    have passed (at least one batch). Returns (rate, sample text, threads,
    seconds, next start)."""
    from oracle import cpu_ref
    cpu_ref.build()
    th = cpu_ref.threads()
    T = len(cfg.pos)
    picks = np.random.default_rng(0).permutation(T)
    per = max(th, 8)
    t0 = time.perf_counter()
    done = n_tr = 0
    k = start
    while done == 0 or time.perf_counter() - t0 < seconds:
        lo = (k * per) % T
        sel = np.sort(picks[lo:lo + per])
        done += cpu_batch(cfg, sel)
        n_tr += len(sel)
        k += 1
    el = time.perf_counter() - t0
    return (done / el, f"{done} pairs ({n_tr} traces x 4 whole targets) "
                       f"in {el:.1f} s on {th} threads", th, el, k)


def run_reference(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    from radar_sounder_simulator_gb300 import scenes
    cfg = scenes.config2(n_cells=args.n_cells, n_traces=args.n_traces)
    per_step = max(args.cpu_seconds / 4.0, 0.5)
    k = 0
    for _ in range(args.warmup):
        _, _, _, _, k = cpu_sample_rate(cfg, 0.0, k)
    rates, secs, pairs = [], [], 0
    th, sample = 1, ""
    for _ in range(args.steps):
        v, sample, th, el, k = cpu_sample_rate(cfg, per_step, k)
        rates.append(v)
        secs.append(el)
        pairs += v * el
    value = pairs / sum(secs)
    line = {"impl": "reference", "metric": METRIC, "value": value,
            "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup,
            "ms_per_step": float(np.mean(secs)) * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64", "data": "synthetic (seeded config-2 scene)",
            "config": config_dict(args, ws),
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": th,
                             "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0},
            "note": "each step is a bounded sample of the workload (one "
                    "batch of traces through all four whole targets); "
                    "ms_per_step is that sample's time. " + CPU_KIND_NOTE}
    print(json.dumps(line), flush=True)


# --------------------------------------------------------------------------
# GPU arm
# --------------------------------------------------------------------------
def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
        return
    import torch
    import torch.distributed as dist
    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    device = torch.device("cuda", local)
    if ws > 1:
        dist.init_process_group("nccl", device_id=device)

    from radar_sounder_simulator_gb300 import scenes
    cfg = scenes.config2(n_cells=args.n_cells, n_traces=args.n_traces,
                         line_offset_y=line_offset(rank))
    pairs_step = sum(len(f.centers) for f in cfg.layers) * len(cfg.pos)

    plans = build_plans(cfg, "split", device)
    if args.kernel_only:
        run_kernel_only(args, plans, device)
        return
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=device)
    stream = torch.cuda.current_stream(device)

    def step(record=None):
        flush.fill_(1)
        outs = []
        for i, p in enumerate(plans):
            if record is not None:
                record[i][0].record(stream)
            outs.append(p.run())
            if record is not None:
                record[i][1].record(stream)
        return outs

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    ev = [[(torch.cuda.Event(enable_timing=True),
            torch.cuda.Event(enable_timing=True)) for _ in plans]
          for _ in range(args.steps)]
    t_start = torch.cuda.Event(enable_timing=True)
    t_end = torch.cuda.Event(enable_timing=True)
    if ws > 1:
        dist.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        t_start.record(stream)
        for s in range(args.steps):
            outs = step(ev[s])
        t_end.record(stream)
        torch.cuda.synchronize()
    if ws > 1:
        dist.barrier()
    ms = t_start.elapsed_time(t_end) / args.steps
    ms = max_over_ranks(ms, device, ws)
    value = job_rate(pairs_step, ws, ms)
    per_kernel = [float(np.mean([ev[s][i][0].elapsed_time(ev[s][i][1])
                                 for s in range(args.steps)]))
                  for i in range(len(plans))]

    # float64 form on the first traces of the same scene (one step) and the
    # split form's error on those traces
    fp64 = None
    err = None
    if not args.skip_fp64:
        sub = scenes.config2(n_cells=args.n_cells, n_traces=args.n_traces,
                             line_offset_y=line_offset(rank))
        nt = min(args.fp64_traces, args.n_traces)
        sub.pos, sub.uct = cfg.pos[:nt], cfg.uct[:nt]
        sub.t0 = cfg.t0
        plans64 = build_plans(sub, "fp64", device)
        plans32 = build_plans(sub, "split", device)
        outs32 = [p.run() for p in plans32]
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        flush.fill_(1)
        e0.record(stream)
        outs64 = [p.run() for p in plans64]
        e1.record(stream)
        torch.cuda.synchronize()
        ms64 = e0.elapsed_time(e1)
        pairs64 = sum(len(f.centers) for f in sub.layers) * nt
        fp64 = {"value": pairs64 / (ms64 * 1e-3), "unit": UNIT,
                "ms_per_step": ms64 * len(cfg.pos) / nt,
                "traces_timed": nt}
        err = split_error(outs32, outs64)
        del plans64, outs64, plans32, outs32

    # end to end through the drop-in API with host buffers
    h2d, d2h = host_bytes(cfg)
    e2e_s = None
    if not args.skip_e2e:
        drop_in_step(cfg, "split", device)      # warm-up (page-locked pool)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            drop_in_step(cfg, "split", device)
        torch.cuda.synchronize()
        e2e_s = max_over_ranks((time.perf_counter() - t0) / args.steps *
                               1e3, device, ws) * 1e-3

    launches = args.steps * sum(p.kernel_launches() for p in plans)
    peak = fp32_peak_tflops(device)
    roof = roofline(per_kernel, [len(f.centers) * len(cfg.pos)
                                 for f in cfg.layers], peak,
                    traffic=args.traffic)
    if rank == 0:
        cpu = None
        if ws == 1 and args.cpu_seconds > 0:
            v, sample, th, _, _ = cpu_sample_rate(cfg, args.cpu_seconds)
            cpu = {"value": v, "unit": UNIT, "cores": th, "kind": "port",
                   "sample": sample, "note": CPU_KIND_NOTE}
        rows = run_rows(args, device, peak) if ws == 1 else None
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws,
                "steps": args.steps, "warmup": args.warmup,
                "ms_per_step": ms, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64",
                "data": "synthetic (seeded config-2 scene)",
                "config": config_dict(args, ws),
                "e2e": ({"value": job_rate(pairs_step, ws, e2e_s * 1e3),
                         "unit": UNIT,
                         "h2d_bytes_per_step": h2d,
                         "d2h_bytes_per_step": d2h} if e2e_s else None),
                "fp64": fp64,
                "split_over_fp64": (value / ws / fp64["value"]) if fp64
                else None,
                "error_vs_fp64": err,
                "per_kernel_ms": dict(zip(["surface", "h1_seq", "h2_joint",
                                           "bed_joint"], per_kernel)),
                "gpu_launches": launches, "roofline": roof,
                "clocks": clk.summary(), "cpu_baseline": cpu, "rows": rows}
        # last key, so a reader that keeps only the line's tail still has
        # every row's rate and split-vs-FP64 error
        line["summary"] = summarize(line)
        print(json.dumps(line), flush=True)
    if ws > 1:
        dist.destroy_process_group()


def rough_bed_450_plan(device):
    """The roughness configuration's slowest job: the rough bed under the
    surface (sequential refraction, area-only exponential series, taper) in
    the 450 MHz band, all 2048 traces."""
    from radar_sounder_simulator_gb300 import scenes
    from radar_sounder_simulator_gb300.multilayer import prepare_refracted
    cfg = scenes.config3()
    bd = scenes.config3_band(cfg, 450e6)
    rb = cfg.rough["bed"]
    return prepare_refracted(
        cfg.pos, cfg.uct, cfg.bed, [cfg.surface], cfg.eps, cfg.att,
        mode="coherent", t0=bd["t0"], dt=bd["dt"], n_samples=bd["n_s"],
        c=cfg.c, gamma=cfg.gamma_bed, k0=bd["k0"],
        roughness=(rb["sigma"], rb["corr"], rb["phasors"], bd["nt_b"],
                   "exponential"), d_phi_area=True, taper_s=0.05,
        refraction="sequential", precision="split", device=device)


def plain_surface_plan(device, compress):
    """The plain 128^2 surface's split facet sum over 256 traces, or (with
    ``compress``) the double-float FFT compression of its field with the
    20 us chirp (1201 taps, N = 4096), as a plan-like object."""
    from types import SimpleNamespace
    from radar_sounder_simulator_gb300 import scenes
    from radar_sounder_simulator_gb300.coherent import prepare_coherent
    from radar_sounder_simulator_gb300.waveform import (RangeCompressor,
                                                         compressed_pulse)
    cfg = scenes.config1()
    f = cfg.facets
    pl = prepare_coherent(cfg.pos, cfg.uct, f.centers, f.normals, f.areas,
                          f.e1, f.e2, **cfg.kw, precision="split",
                          device=device)
    if not compress:
        return pl
    pulse, m = compressed_pulse(cfg.bw, cfg.pulse_length, cfg.kw["dt"],
                                "hann", "chirp")
    rc = RangeCompressor(pulse, m, cfg.kw["n_samples"], precision="split",
                         device=device)
    fld, _ = pl.run()
    return SimpleNamespace(run=lambda: rc.run(fld))


def run_kernel_only(args, plans, device):
    """One target's plan alone (main pass, fix-up, reduce): warm-up and
    timed launches, mean event time printed (the profiling entry point)."""
    import torch
    if args.kernel_only == "rough450":
        p = rough_bed_450_plan(device)
    elif args.kernel_only in ("plain128", "compress"):
        p = plain_surface_plan(device, args.kernel_only == "compress")
    else:
        p = plans[["surface", "h1", "h2", "bed"].index(args.kernel_only)]
    for _ in range(args.warmup):
        p.run()
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(args.steps):
        p.run()
    e1.record()
    torch.cuda.synchronize()
    print(json.dumps({"kernel_only": args.kernel_only,
                      "ms": e0.elapsed_time(e1) / max(args.steps, 1)}),
          flush=True)


# --------------------------------------------------------------------------
# secondary workloads (the other configurations), measured after the line's
# headline on rank 0; each entry states its own units and errors
# --------------------------------------------------------------------------
def _events_ms(fn, reps, flush=None):
    import torch
    fn()
    torch.cuda.synchronize()
    ts = []
    for _ in range(reps):
        if flush is not None:
            flush.fill_(1)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        fn()
        e1.record()
        torch.cuda.synchronize()
        ts.append(e0.elapsed_time(e1))
    return float(np.median(ts))


def _complex(field):
    import torch
    return torch.view_as_complex(field.contiguous())


def _errors(a, b):
    """rel L2, max phase and max dB over samples above -60 dB of the peak."""
    import torch
    rel = (torch.linalg.vector_norm(a - b) /
           torch.linalg.vector_norm(b)).item()
    p = b.abs() ** 2
    keep = p > p.max() * 1e-6
    ph = torch.angle(a[keep] / b[keep]).abs().max().item()
    db = (10 * torch.log10(a[keep].abs() ** 2 / p[keep])).abs().max().item()
    return {"rel_l2": rel, "phase_rad": ph, "power_db": db}


def _roof(flop, ms, peak, bound, per_unit, note):
    achieved = flop / (ms * 1e-3) / 1e12
    return {"bound": bound, "achieved": achieved, "peak": peak,
            "unit": "TFLOP/s", "frac": achieved / peak,
            "flop_per_unit": per_unit, "ms": ms, "note": note}


def cfg1_cpu_baseline(cfg, seconds):
    """The float64 NumPy oracle's coherent facet sum (the reference's
    formulas) on one host core, over consecutive 8-trace slices of the
    plain-surface track until about ``seconds`` have passed (at least one
    slice)."""
    from oracle import lpa
    f = cfg.facets
    T, N = len(cfg.pos), len(f.centers)
    t0 = time.perf_counter()
    done = 0
    while done < T and (done == 0 or time.perf_counter() - t0 < seconds):
        sl = slice(done, min(done + 8, T))
        lpa.coherent_cluttergram(cfg.pos[sl], cfg.uct[sl], f.centers,
                                 f.normals, f.areas, f.e1, f.e2, **cfg.kw)
        done = sl.stop
    el = time.perf_counter() - t0
    return {"value": done * N / el, "unit": "contribs/s", "cores": 1,
            "kind": "port",
            "sample": f"{done} traces x {N} facets, float64 NumPy oracle, "
                      f"{el:.1f} s"}


def df_fft_flop(n_fft):
    """FP32 FLOP of one row's double-float FFT convolution (FMA = 2): per
    radix-4 butterfly 16 double-float additions (11) and 3 twiddle products
    (two exact-product dot products of 25), per radix-2 butterfly 4
    additions, per point one spectrum product (50); two transforms."""
    lg = int(np.log2(n_fft))
    per_fft = (lg // 2) * (n_fft // 4) * (16 * 11 + 3 * 50) + \
        (lg % 2) * (n_fft // 2) * 44
    return 2.0 * per_fft + 50.0 * n_fft


def row_cfg1(device, flush, peaks, cpu_seconds=0.0):
    """Plain surface, delta-binned coherent sum + LFM pulse compression,
    the pulse transformed once per precision (``RangeCompressor``)."""
    from radar_sounder_simulator_gb300 import scenes
    from radar_sounder_simulator_gb300.coherent import prepare_coherent
    from radar_sounder_simulator_gb300.waveform import (RangeCompressor,
                                                         compressed_pulse)
    cfg = scenes.config1()
    f = cfg.facets
    args = (cfg.pos, cfg.uct, f.centers, f.normals, f.areas, f.e1, f.e2)
    pl = {p: prepare_coherent(*args, **cfg.kw, precision=p, device=device)
          for p in ("split", "fp64")}
    pulse, m = compressed_pulse(cfg.bw, cfg.pulse_length, cfg.kw["dt"],
                                "hann", "chirp")
    B = cfg.kw["n_samples"]
    rc = {p: RangeCompressor(pulse, m, B, precision=p, device=device)
          for p in ("split", "fp64")}
    out = {}

    def step(prec):
        fld, _ = pl[prec].run()
        out[prec] = rc[prec].run(fld)
    ms = _events_ms(lambda: step("split"), 5, flush)
    ms64 = _events_ms(lambda: step("fp64"), 2, flush)
    ms_k = _events_ms(lambda: pl["split"].run(), 5, flush)
    fld, _ = pl["split"].run()
    ms_rc = _events_ms(lambda: rc["split"].run(fld), 5, flush)
    ms_rc64 = _events_ms(lambda: rc["fp64"].run(fld), 3, flush)
    pairs = len(f.centers) * len(cfg.pos)
    T = len(cfg.pos)
    n_fft = 1 << int(np.ceil(np.log2(B + len(pulse) - 1)))
    fft_flop = 2 * 5.0 * n_fft * np.log2(n_fft) + 6.0 * n_fft
    return {"workload": "surface_128sq_100m_256tr_2048bins_chirp_20us",
            "unit": "contribs/s", "value": pairs / (ms * 1e-3),
            "ms_per_step": ms, "fp64_value": pairs / (ms64 * 1e-3),
            "split_over_fp64": ms64 / ms,
            "roofline": _roof(pairs * 47.0, ms_k, peaks["fp32"], "fp32", 47.0,
                              "surface facet sum (main pass + reduce), 47 "
                              "FLOP per smooth isotropic pair"),
            "range_compression": {
                "taps": len(pulse), "ms": ms_rc, "method": "fft, "
                "double-float transforms, pulse planned once",
                "samples_per_s": T * B / (ms_rc * 1e-3),
                "roofline": _roof(T * df_fft_flop(n_fft), ms_rc,
                                  peaks["fp32"], "fp32", df_fft_flop(n_fft),
                                  f"double-float FFT convolution per row, "
                                  f"N = {n_fft} (FP32 FLOP, FMA = 2)"),
                "fp64_ms": ms_rc64,
                "fp64_roofline": _roof(T * fft_flop, ms_rc64, peaks["fp64"],
                                       "fp64", fft_flop,
                                       f"float64 FFT convolution per row: "
                                       f"2 x 5 N log2 N + 6 N, N = {n_fft}")},
            "error_vs_fp64": _errors(out["split"], out["fp64"]),
            "cpu_baseline": _cpu_or_error(
                lambda: cfg1_cpu_baseline(cfg, cpu_seconds), cpu_seconds)}


def _cpu_or_error(fn, seconds):
    """A row's CPU baseline, None when not asked for, the error text when
    it fails (the row's GPU figures still stand)."""
    if not seconds:
        return None
    try:
        return fn()
    except Exception as exc:  # reported, not hidden
        return {"error": f"{type(exc).__name__}: {exc}"}


def modef_cpu_baseline(cfg, twtt, n_freq, seconds):
    """The float64 NumPy oracle's frequency-sampled profile (the reference's
    multifreq_profile steps) on one host core, position by position along
    the plain-surface track until about ``seconds`` have passed (at least
    one position)."""
    from oracle import multifreq as omf
    f = cfg.facets
    t0 = time.perf_counter()
    done = 0
    while done < len(cfg.pos) and (done == 0 or
                                   time.perf_counter() - t0 < seconds):
        omf.multifreq_profile(cfg.pos[done], f.centers, f.normals, f.areas,
                              f.e1, f.e2, gamma=cfg.kw["gamma"], f0=cfg.f0,
                              bandwidth=cfg.bw, c=cfg.kw["c"], twtt=twtt,
                              n_freq=n_freq, freeze_amplitudes=True)
        done += 1
    el = time.perf_counter() - t0
    return {"value": done * len(f.centers) * n_freq / el,
            "unit": "pair-frequencies/s", "cores": 1, "kind": "port",
            "sample": f"{done} positions x {len(f.centers)} facets x "
                      f"{n_freq} frequencies, float64 NumPy oracle, "
                      f"{el:.1f} s"}


def row_modef(device, flush, peaks, cpu_seconds=0.0):
    """Frequency-sampled synthesis of the config-1 scene, K = 1024."""
    from radar_sounder_simulator_gb300 import scenes
    from radar_sounder_simulator_gb300.multifreq import prepare_multifreq
    cfg = scenes.config1()
    f = cfg.facets
    tw = cfg.kw["t0"] + np.arange(cfg.kw["n_samples"]) * cfg.kw["dt"]
    res, ms = {}, {}
    for prec in ("split", "fp64"):
        pl = prepare_multifreq(cfg.pos, f.centers, f.normals, f.areas, f.e1,
                               f.e2, gamma=cfg.kw["gamma"], f0=cfg.f0,
                               bandwidth=cfg.bw, c=cfg.kw["c"], twtt=tw,
                               n_freq=1024, freeze_amplitudes=True,
                               precision=prec, device=device)
        ms[prec] = _events_ms(pl.run, 3 if prec == "split" else 1, flush)
        res[prec] = _complex(pl.run())
        if prec == "split":
            ms_resp = _events_ms(pl.response, 3, flush)
    units = len(f.centers) * len(cfg.pos) * 1024
    return {"workload": "surface_128sq_100m_256tr_K1024_frozen",
            "unit": "pair-frequencies/s", "value": units / (ms["split"] * 1e-3),
            "ms_per_step": ms["split"],
            "fp64_value": units / (ms["fp64"] * 1e-3),
            "split_over_fp64": ms["fp64"] / ms["split"],
            "roofline": _roof(units * 8.0, ms_resp, peaks["fp32"], "fp32",
                              8.0, "band response (main pass + reduce), 8 "
                              "FLOP per pair-frequency (complex rotate and "
                              "accumulate, frozen amplitudes)"),
            "error_vs_fp64": _errors(res["split"], res["fp64"]),
            "cpu_baseline": _cpu_or_error(
                lambda: modef_cpu_baseline(cfg, tw, 1024, cpu_seconds),
                cpu_seconds)}


def cfg3_cpu_baseline(cfg, band, seconds):
    """The float64 NumPy oracle on one host core for one band of the
    roughness configuration -- the rough surface's coherent sum and the
    rough bed refracted through it -- trace by trace from the middle of the
    track until about ``seconds`` have passed (at least one trace)."""
    from oracle import lpa
    from oracle import refracted as oref
    s, b = cfg.surface, cfg.bed
    rs, rb = cfg.rough["surface"], cfg.rough["bed"]
    common = dict(t0=band["t0"], dt=band["dt"], n_samples=band["n_s"],
                  c=cfg.c, d_phi_area=True, taper_s=0.05)
    T = len(cfg.pos)
    mid = T // 2
    t0 = time.perf_counter()
    done = 0
    while mid + done < T and (done == 0 or
                              time.perf_counter() - t0 < seconds):
        sl = slice(mid + done, mid + done + 1)
        lpa.coherent_cluttergram(
            cfg.pos[sl], cfg.uct[sl], s.centers, s.normals, s.areas, s.e1,
            s.e2, k=band["k0"], gamma=cfg.gamma_surface,
            roughness=(rs["sigma"], rs["corr"], rs["phasors"], band["nt_s"],
                       "exponential"), **common)
        oref.refracted_cluttergram(
            cfg.pos[sl], cfg.uct[sl], b, [s], cfg.eps, cfg.att,
            mode="coherent", gamma=cfg.gamma_bed, k0=band["k0"],
            roughness=(rb["sigma"], rb["corr"], rb["phasors"], band["nt_b"],
                       "exponential"), refraction="sequential", **common)
        done += 1
    el = time.perf_counter() - t0
    n = len(s.centers) + len(b.centers)
    return {"value": done * n / el, "unit": "contribs/s", "cores": 1,
            "kind": "port",
            "sample": f"{done} traces x {n} facets (surface + bed) at "
                      f"{band['k0'] * cfg.c / (2 * np.pi) / 1e6:.0f} MHz, "
                      f"float64 NumPy oracle, {el:.1f} s"}


def row_cfg3(device, flush, peaks, cfg3_error_traces=32, cpu_seconds=0.0):
    """Rough surface and bed, four bands: per band the surface coherent sum
    and the refracted bed sum (per-facet sigma, l; exponential ACF with the
    area-only series and taper), each pulse-compressed."""
    from radar_sounder_simulator_gb300 import scenes
    from radar_sounder_simulator_gb300.coherent import prepare_coherent
    from radar_sounder_simulator_gb300.multilayer import prepare_refracted
    from radar_sounder_simulator_gb300.waveform import (RangeCompressor,
                                                         compressed_pulse)
    cfg = scenes.config3()
    s, b = cfg.surface, cfg.bed
    c = cfg.c
    bands = {}
    total_ms, total_pairs = 0.0, 0
    for f0 in cfg.bands:
        bd = scenes.config3_band(cfg, f0)
        bw, dt, k0, n_s, t0 = bd["bw"], bd["dt"], bd["k0"], bd["n_s"], bd["t0"]
        nt_s, nt_b = bd["nt_s"], bd["nt_b"]
        rs, rb = cfg.rough["surface"], cfg.rough["bed"]

        def plans(pos, uct, nts=nt_s, ntb=nt_b):
            ps = prepare_coherent(
                pos, uct, s.centers, s.normals, s.areas, s.e1, s.e2, k=k0,
                gamma=cfg.gamma_surface, t0=t0, dt=dt, n_samples=n_s, c=c,
                roughness=(rs["sigma"], rs["corr"], rs["phasors"], nts,
                           "exponential"), d_phi_area=True, taper_s=0.05,
                precision="split", device=device)
            pb = prepare_refracted(
                pos, uct, b, [s], cfg.eps, cfg.att, mode="coherent", t0=t0,
                dt=dt, n_samples=n_s, c=c, gamma=cfg.gamma_bed, k0=k0,
                roughness=(rb["sigma"], rb["corr"], rb["phasors"], ntb,
                           "exponential"), d_phi_area=True, taper_s=0.05,
                refraction="sequential", precision="split", device=device)
            return ps, pb
        ps, pb = plans(cfg.pos, cfg.uct)
        pulse, m = compressed_pulse(bw, 10e-6, dt, "hann", "chirp")
        rc = RangeCompressor(pulse, m, n_s, precision="split", device=device)

        def step():
            f1, _ = ps.run()
            f2, _ = pb.run()
            rc.run(f1)
            rc.run(f2)
        ms = _events_ms(step, 2, flush)
        ms_k = _events_ms(lambda: (ps.run(), pb.run()), 2, flush)
        T = len(cfg.pos)
        pairs = (len(s.centers) + len(b.centers)) * T
        # canonical per-pair work: smooth pair (surface) or sequential
        # refracted pair (bed), taper, rough overhead, and 10 FLOP + 2 MUFU
        # per series term with the per-facet term count
        # n_terms_for((2 k_local sigma_i)^2)
        def terms(k_loc, sig):
            x = (2.0 * k_loc * np.asarray(sig, np.float64)) ** 2
            return np.clip(np.ceil(x + 6.0 * np.sqrt(x) + 5.0), 10, 300)
        n_s_i = terms(k0, rs["sigma"])
        n_b_i = terms(k0 * np.sqrt(cfg.eps[1]), rb["sigma"])
        flop = T * (np.sum(47.0 + 6 + 20 + 10 * n_s_i) +
                    np.sum(pair_flops(1, False) + 6 + 20 + 10 * n_b_i))
        mufu = T * (np.sum(8.0 + 1 + 3 + 2 * n_s_i) +
                    np.sum(113.0 + 1 + 3 + 2 * n_b_i))
        t_fp32 = flop / (peaks["fp32"] * 1e12)
        t_mufu = mufu / (peaks["mufu_tops"] * 1e12)
        bound = "mufu" if t_mufu > t_fp32 else "fp32"
        bands[f"{f0 / 1e6:.0f}MHz"] = {
            "ms": ms, "kernel_ms": ms_k, "n_terms": [nt_s, nt_b],
            "n_samples": n_s, "contribs_per_s": pairs / (ms * 1e-3),
            "roofline": {"bound": bound,
                         "frac": max(t_fp32, t_mufu) / (ms_k * 1e-3),
                         "fp32_tflops": flop / (ms_k * 1e-3) / 1e12,
                         "mufu_tops": mufu / (ms_k * 1e-3) / 1e12,
                         "mean_terms": [float(n_s_i.mean()),
                                        float(n_b_i.mean())]}}
        # converged series: the parity runs keep the reference's 300-term
        # cap (n_terms_for), which truncates D_Phi for the rough tail in the
        # upper bands; the same runs with ceil(x + 6 sqrt(x) + 5) terms for
        # the largest surface and 0.999-quantile bed x, where that fits the
        # kernels' 4096-term limit
        key = f"{f0 / 1e6:.0f}MHz"
        try:
            xs = (2 * k0 * rs["sigma"].max()) ** 2
            xb = (2 * k0 * np.sqrt(3.15) *
                  np.quantile(rb["sigma"], 0.999)) ** 2
            cs, cb = (max(10, int(np.ceil(x + 6.0 * np.sqrt(x) + 5.0)))
                      for x in (xs, xb))
            if (cs, cb) == (nt_s, nt_b):
                conv = {"n_terms": [cs, cb], "same_as_parity": True}
            elif max(cs, cb) <= 4096:
                cps, cpb = plans(cfg.pos, cfg.uct, cs, cb)
                ms_c = _events_ms(lambda: (cps.run(), cpb.run()), 2, flush)
                conv = {"n_terms": [cs, cb], "kernel_ms": ms_c,
                        "contribs_per_s": pairs / (ms_c * 1e-3)}
                del cps, cpb
            else:
                conv = {"n_terms": [cs, cb],
                        "note": "above the kernels' 4096-term limit"}
        except Exception as exc:  # reported, not hidden
            conv = {"error": f"{type(exc).__name__}: {exc}"}
        bands[key]["converged_series"] = conv
        if f0 == 60e6:
            bands[key]["cpu_baseline"] = _cpu_or_error(
                lambda: cfg3_cpu_baseline(
                    cfg, dict(k0=k0, t0=t0, dt=dt, n_s=n_s, nt_s=nt_s,
                              nt_b=nt_b), cpu_seconds), cpu_seconds)
        # split form against the FP64 form on the central traces (both
        # targets' binned fields); a failure here is reported in the band
        if cfg3_error_traces:
            try:
                mid = len(cfg.pos) // 2
                sub = slice(mid - cfg3_error_traces // 2,
                            mid + cfg3_error_traces // 2)
                qs, qb = plans(cfg.pos[sub], cfg.uct[sub])
                outs = [qs.run(), qb.run()]
                outs64 = [qs.run("fp64"), qb.run("fp64")]
                err = {"traces": cfg3_error_traces,
                       **split_error(outs, outs64)}
                del qs, qb, outs, outs64
            except Exception as exc:  # reported, not hidden
                err = {"error": f"{type(exc).__name__}: {exc}"}
            bands[f"{f0 / 1e6:.0f}MHz"]["error_vs_fp64"] = err
        total_ms += ms
        total_pairs += pairs
        del ps, pb
    try:
        batched = cfg3_batched(cfg, device, flush, total_pairs,
                               sum(b["kernel_ms"] for b in bands.values()))
    except Exception as exc:  # reported, not hidden
        batched = {"error": f"{type(exc).__name__}: {exc}"}
    return {"workload": "rough_surface_bed_512sq_25m_2048tr_4bands",
            "unit": "contribs/s", "value": total_pairs / (total_ms * 1e-3),
            "ms_per_step": total_ms, "bands": bands, "batched": batched,
            "roofline_note": "per band: the slower of the FP32 and MUFU "
                             "pipes at the canonical per-pair counts (FP32 "
                             "47 or the sequential refracted pair + 6 taper "
                             "+ 20 rough + 10 per term; MUFU 8 or 113 + 1 + "
                             "3 + 2 per term; terms per facet from its "
                             "sigma) over the kernels' event time, against "
                             "the FMA and MUFU rates measured in this run"}


def cfg3_batched(cfg, device, flush, pairs, per_call_ms):
    """The roughness configuration's eight (target, band) jobs as one
    persistent surface batch and one persistent refracted batch, captured
    in one CUDA graph and replayed once per step; every job's field is
    checked against its own per-call result."""
    import torch
    from radar_sounder_simulator_gb300 import scenes
    from radar_sounder_simulator_gb300.batch import (BatchGraph,
                                                     CoherentBatch,
                                                     RefractedBatch)
    from radar_sounder_simulator_gb300.coherent import prepare_coherent
    from radar_sounder_simulator_gb300.multilayer import prepare_refracted
    s, b = cfg.surface, cfg.bed
    rs, rb = cfg.rough["surface"], cfg.rough["bed"]
    surf, bed = [], []
    for f0 in cfg.bands:
        bd = scenes.config3_band(cfg, f0)
        common = dict(t0=bd["t0"], dt=bd["dt"], n_samples=bd["n_s"],
                      c=cfg.c, d_phi_area=True, taper_s=0.05,
                      precision="split", device=device)
        surf.append(prepare_coherent(
            cfg.pos, cfg.uct, s.centers, s.normals, s.areas, s.e1, s.e2,
            k=bd["k0"], gamma=cfg.gamma_surface,
            roughness=(rs["sigma"], rs["corr"], rs["phasors"], bd["nt_s"],
                       "exponential"), **common))
        bed.append(prepare_refracted(
            cfg.pos, cfg.uct, b, [s], cfg.eps, cfg.att, mode="coherent",
            gamma=cfg.gamma_bed, k0=bd["k0"],
            roughness=(rb["sigma"], rb["corr"], rb["phasors"], bd["nt_b"],
                       "exponential"), refraction="sequential", **common))
    cb, rbt = CoherentBatch(surf), RefractedBatch(bed)
    graph = BatchGraph([cb.run, rbt.run], device)
    graph.capture()
    ms = _events_ms(graph.replay, 3, flush)
    torch.cuda.synchronize()
    worst = 0.0
    for plans, outs in ((surf, cb.outputs), (bed, rbt.outputs)):
        for p, (field, _) in zip(plans, outs):
            one = p.run()[0]
            a, r = _complex(field), _complex(one)
            worst = max(worst, float(torch.linalg.vector_norm(a - r) /
                                     torch.linalg.vector_norm(r)))
    out = {"jobs": len(surf) + len(bed), "graph_replays_per_step": 1,
           "kernel_launches": cb.kernel_launches() + rbt.kernel_launches(),
           "ms": ms, "contribs_per_s": pairs / (ms * 1e-3),
           "per_call_kernel_ms": per_call_ms,
           "max_rel_l2_vs_per_call": worst}
    del graph, cb, rbt, surf, bed
    return out


def cfg4_cpu_baseline(seconds):
    """The float64 NumPy oracle on one host core for the sweep's first
    instance (tabulated antenna pattern): 8-trace slices from the middle of
    its track, every facet of every trace (no culling), until about
    ``seconds`` have passed (at least one slice)."""
    from oracle import lpa
    from radar_sounder_simulator_gb300 import scenes
    inst = scenes.config4_instance(0)
    f = inst.facets
    T, N = len(inst.pos), len(f.centers)
    kind, pv, pa, pb = inst.kw["pattern"]
    pv = np.asarray(pv, np.float64).reshape(T, -1)
    kw = {k: v for k, v in inst.kw.items() if k != "pattern"}
    mid = T // 2
    t0 = time.perf_counter()
    done = 0
    while mid + done < T and (done == 0 or
                              time.perf_counter() - t0 < seconds):
        sl = slice(mid + done, min(mid + done + 8, T))
        lpa.coherent_cluttergram(inst.pos[sl], inst.uct[sl], f.centers,
                                 f.normals, f.areas, f.e1, f.e2,
                                 pattern=(kind, pv[sl], pa, pb),
                                 window_cull=False, **kw)
        done = sl.stop - mid
    el = time.perf_counter() - t0
    return {"value": done * N / el, "unit": "contribs/s", "cores": 1,
            "kind": "port",
            "sample": f"{done} traces x {N} facets of instance 0 (every "
                      f"pair, tabulated pattern), float64 NumPy oracle, "
                      f"{el:.1f} s"}


def row_cfg4(device, n_inst, flush, peaks, cpu_seconds=0.0):
    """Batched design sweep: one persistent work-queue launch over all
    instances, captured in a CUDA graph, autotuned decomposition."""
    import torch
    from radar_sounder_simulator_gb300 import scenes
    from radar_sounder_simulator_gb300.batch import CoherentBatch
    from radar_sounder_simulator_gb300.coherent import prepare_coherent
    t_host = time.perf_counter()
    plans, plans64, pairs = [], [], 0
    for i in range(n_inst):
        inst = scenes.config4_instance(i)
        f = inst.facets
        args = (inst.pos, inst.uct, f.centers, f.normals, f.areas, f.e1,
                f.e2)
        p = prepare_coherent(*args, **inst.kw, precision="split",
                             device=device)
        plans.append(p)
        pairs += int(np.sum(np.minimum(
            (p.cull.off.astype(np.int64) + p.cull.n_win) * p.cull.block_size,
            p.N) - np.minimum(p.cull.off.astype(np.int64) *
                              p.cull.block_size, p.N)))
        if i < 8:
            plans64.append(prepare_coherent(*args, **inst.kw,
                                            precision="fp64", device=device))
    host_s = time.perf_counter() - t_host
    batch = CoherentBatch(plans)
    tun, tune_ms = batch.autotune(
        candidates=[(512, 8, 16, 0), (512, 6, 16, 0), (256, 8, 16, 0),
                    (256, 4, 16, 0), (128, 8, 16, 0), (512, 6, 64, 0),
                    (256, 8, 64, 0), (128, 4, 64, 0)],
        reps=1)
    batch.capture()
    ms = _events_ms(batch.replay, 3, flush)
    # FP64 form and error on the first 8 instances (one-call entry point
    # against the batch's split output)
    sub_pairs = sum(p.T * min(p.cull.n_win * p.cull.block_size, p.N)
                    for p in plans64)
    b64 = CoherentBatch(plans64)
    ms64 = _events_ms(b64.run, 1, flush)
    bsp = CoherentBatch(plans[:8])
    bsp.run()
    b64.run()
    torch.cuda.synchronize()
    err = {"rel_l2": 0.0, "phase_rad": 0.0, "power_db": 0.0}
    for (fs, _), (fd, _) in zip(bsp.outputs, b64.outputs):
        e = _errors(_complex(fs), _complex(fd))
        err = {k: max(err[k], e[k]) for k in err}
    ms_sub = _events_ms(bsp.run, 2, flush)
    return {"workload": f"design_sweep_{n_inst}_instances",
            "unit": "contribs/s", "value": pairs / (ms * 1e-3),
            "ms_per_step": ms, "pairs": pairs, "launches_per_step": 2,
            "roofline": _roof(pairs * 57.0, ms, peaks["fp32"], "fp32", 57.0,
                              "persistent kernel + batched reduce, 47 FLOP "
                              "per pair + 10 for the tabulated antenna"),
            "cuda_graph": True, "tuning": list(tun),
            "host_prep_s": host_s,
            "fp64_subset": {"instances": len(plans64),
                            "split_ms": ms_sub, "fp64_ms": ms64,
                            "split_over_fp64": ms64 / ms_sub,
                            "window_pairs": sub_pairs},
            "error_vs_fp64": err,
            "cpu_baseline": _cpu_or_error(
                lambda: cfg4_cpu_baseline(cpu_seconds), cpu_seconds)}


def cfg5_fd_subset(cfg, device, n_traces=32, n_check=16):
    """Adjoint of the split form against central differences of the FP64
    GPU forward on the central ``n_traces`` traces of the configuration:
    ``n_check`` seeded facets per kind among the most-illuminated tenth,
    relative step 2^-13. Returns the largest per-entry relative error per
    kind (absolute floor 1e-5 of the kind's largest checked gradient)."""
    import torch
    from radar_sounder_simulator_gb300.adjoint import (WindowPowerModel,
                                                       db_misfit)
    mid = len(cfg.pos) // 2
    sl = slice(mid - n_traces // 2, mid + n_traces // 2)

    def model(prec):
        return WindowPowerModel(
            cfg.pos[sl], cfg.uct[sl], cfg.bed, [cfg.surface], cfg.eps,
            [0.0, cfg.alpha], t0=cfg.t0, dt=cfg.dt, n_samples=cfg.n_samples,
            c=cfg.c, k0=cfg.k0, window=cfg.window, alpha_legs=(1,),
            corr_length=cfg.corr, phasors=cfg.phasors, n_terms=cfg.n_terms,
            precision=prec, device=device)
    m32, m64 = model("split"), model("fp64")
    dev = m32.device

    def t(v):
        return torch.tensor(v, dtype=torch.float64, device=dev)
    with torch.no_grad():
        P_hat = m64.power(t(cfg.R_hat), t(cfg.sig_hat), t(cfg.alpha + 1.0))
    R = t(cfg.R).requires_grad_(True)
    sg = t(cfg.sig).requires_grad_(True)
    a = t(cfg.alpha).requires_grad_(True)
    db_misfit(m32.power(R, sg, a), P_hat).backward()

    def loss(Rv, sv, av):
        with torch.no_grad():
            return float(db_misfit(m64.power(Rv, sv, av), P_hat))
    rng = np.random.default_rng(55)
    h = 2.0 ** -13
    out = {}
    for name, g, base in (("reflectivity_db", R.grad, cfg.R),
                          ("rms_height", sg.grad, cfg.sig)):
        gm = g.abs().cpu().numpy()
        top = np.argsort(gm)[-max(len(gm) // 10, n_check):]
        idx = rng.choice(top, size=n_check, replace=False)
        fd = []
        for i in idx:
            vp, vm = base.copy(), base.copy()
            d = h * abs(base[i])
            vp[i] += d
            vm[i] -= d
            if name == "reflectivity_db":
                fd.append((loss(t(vp), t(cfg.sig), t(cfg.alpha)) -
                           loss(t(vm), t(cfg.sig), t(cfg.alpha))) / (2 * d))
            else:
                fd.append((loss(t(cfg.R), t(vp), t(cfg.alpha)) -
                           loss(t(cfg.R), t(vm), t(cfg.alpha))) / (2 * d))
        fd = np.array(fd)
        got = g.cpu().numpy()[idx]
        floor = 1e-5 * np.abs(fd).max()
        out[name] = float((np.abs(got - fd) / (np.abs(fd) + floor)).max())
    da = h * cfg.alpha
    fda = (loss(t(cfg.R), t(cfg.sig), t(cfg.alpha + da)) -
           loss(t(cfg.R), t(cfg.sig), t(cfg.alpha - da))) / (2 * da)
    out["alpha"] = float(abs(float(a.grad) - fda) / abs(fda))
    out.update(traces=n_traces, params_per_kind=n_check,
               referee="central differences of the FP64 GPU forward, "
                       "relative step 2^-13")
    return out


def cfg5_cpu_baseline(cfg, seconds):
    """The float64 NumPy oracle forward of the bed on one host core, trace
    by trace from the middle of the track (at least one trace). There is
    no CPU adjoint: a CPU gradient by central differences would cost two
    such forwards per parameter."""
    from oracle import refracted as oref
    T = len(cfg.pos)
    mid = T // 2
    t0 = time.perf_counter()
    done = 0
    while mid + done < T and (done == 0 or
                              time.perf_counter() - t0 < seconds):
        sl = slice(mid + done, mid + done + 1)
        oref.refracted_cluttergram(
            cfg.pos[sl], cfg.uct[sl], cfg.bed, [cfg.surface], cfg.eps,
            [0.0, cfg.alpha], mode="coherent", t0=cfg.t0, dt=cfg.dt,
            n_samples=cfg.n_samples, c=cfg.c, gamma=10.0 ** (cfg.R / 20.0),
            k0=cfg.k0, roughness=(cfg.sig, cfg.corr, cfg.phasors,
                                  cfg.n_terms, "exponential"),
            d_phi_area=True, taper_s=0.05, refraction="sequential")
        done += 1
    el = time.perf_counter() - t0
    n = len(cfg.bed.centers)
    return {"value": done * n / el, "unit": "contribs/s", "cores": 1,
            "kind": "port",
            "sample": f"{done} traces x {n} bed facets, float64 NumPy "
                      f"oracle forward (no CPU adjoint exists), {el:.1f} s"}


def row_cfg5(device, flush, peaks, cpu_seconds=0.0):
    """Adjoint: forward bed power and hand-written backward of the dB
    misfit, 512^2 bed facets x 1024 traces; a finite-difference subset on
    the central traces; roofline of the backward pass."""
    import torch
    from radar_sounder_simulator_gb300 import scenes
    from radar_sounder_simulator_gb300.adjoint import (WindowPowerModel,
                                                       db_misfit)
    cfg = scenes.config5()
    model = WindowPowerModel(
        cfg.pos, cfg.uct, cfg.bed, [cfg.surface], cfg.eps, [0.0, cfg.alpha],
        t0=cfg.t0, dt=cfg.dt, n_samples=cfg.n_samples, c=cfg.c, k0=cfg.k0,
        window=cfg.window, alpha_legs=(1,), corr_length=cfg.corr,
        phasors=cfg.phasors, n_terms=cfg.n_terms, precision="split",
        device=device)
    dev = model.device
    with torch.no_grad():
        P_hat = model.power(torch.tensor(cfg.R_hat, device=dev),
                            torch.tensor(cfg.sig_hat, device=dev),
                            torch.tensor(cfg.alpha + 1.0, device=dev))
    R = torch.tensor(cfg.R, device=dev, requires_grad=True)
    sg = torch.tensor(cfg.sig, device=dev, requires_grad=True)
    a = torch.tensor(cfg.alpha, dtype=torch.float64, device=dev,
                     requires_grad=True)
    ts = {}

    def fwd():
        return db_misfit(model.power(R, sg, a), P_hat)
    ts["forward_ms"] = _events_ms(fwd, 2, flush)
    L = fwd()
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record()
    L.backward()
    e1.record()
    torch.cuda.synchronize()
    ts["backward_ms"] = e0.elapsed_time(e1)
    T, n = len(cfg.pos), len(cfg.bed.centers)
    pairs = n * T
    # canonical backward work per pair: the sequential refracted pair, taper
    # and rough overhead, 12 FLOP per series term (the series and its
    # x-derivative sum) over each facet's own term count, and 24 for the
    # three gradient accumulations
    x = (2.0 * cfg.k0 * np.sqrt(cfg.eps[1]) * np.asarray(cfg.sig)) ** 2
    terms = np.clip(np.ceil(x + 6.0 * np.sqrt(x) + 5.0), 10, cfg.n_terms)
    flop = T * np.sum(pair_flops(1, False) + 6 + 20 + 12 * terms + 24)
    roof = _roof(flop, ts["backward_ms"], peaks["fp32"], "fp32",
                 float(flop / pairs),
                 "backward pass (adjoint + fix-up), canonical per-pair "
                 "FLOP: sequential refracted pair 865, taper 6, rough 20, "
                 "12 per series term, 24 accumulation")
    try:
        fdsub = cfg5_fd_subset(cfg, device)
    except Exception as exc:  # reported, not hidden
        fdsub = {"error": f"{type(exc).__name__}: {exc}"}
    return {"workload": "adjoint_bed_512sq_1024tr", "unit": "contribs/s",
            "value": pairs / (ts["backward_ms"] * 1e-3), **ts,
            "n_terms": cfg.n_terms, "roofline": roof,
            "fd_subset_max_rel_err": fdsub,
            "cpu_baseline": _cpu_or_error(
                lambda: cfg5_cpu_baseline(cfg, cpu_seconds), cpu_seconds),
            "grad_norms": {"reflectivity_db": float(R.grad.norm()),
                           "rms_height": float(sg.grad.norm()),
                           "alpha": float(a.grad)}}


def row_incoh(device, flush, peaks):
    """Incoherent (power) facet sum of the multilayer scene's surface: every
    facet for every trace, as the reference's incoherent kernel does."""
    from radar_sounder_simulator_gb300 import scenes
    from radar_sounder_simulator_gb300.incoherent import prepare_incoherent
    cfg = scenes.config2()
    f = cfg.layers[0]
    pl = prepare_incoherent(cfg.pos, cfg.uct, f.centers, f.normals, f.areas,
                            t0=cfg.t0, dt=cfg.dt, n_samples=cfg.n_samples,
                            c=cfg.c, device=device)
    ms = _events_ms(pl.run, 5, flush)
    pairs = len(f.centers) * len(cfg.pos)
    # CPU baseline: the float32 oracle (the reference's algorithm in NumPy)
    # on 32 traces of the same scene, one core
    from oracle import incoherent as oinc
    t0 = time.perf_counter()
    oinc.incoherent_cluttergram(cfg.pos[:32], cfg.uct[:32], f.centers,
                                f.normals, f.areas, t0=cfg.t0, dt=cfg.dt,
                                n_samples=cfg.n_samples, c=cfg.c)
    cpu_s = time.perf_counter() - t0
    return {"workload": "surface_512sq_50m_1024tr_20km_2048bins_incoherent",
            "unit": "contribs/s", "value": pairs / (ms * 1e-3),
            "ms_per_step": ms,
            "cpu_baseline": {"value": 32 * len(f.centers) / cpu_s,
                             "unit": "contribs/s", "cores": 1,
                             "kind": "port",
                             "sample": "32 traces x 262144 facets, float32 "
                                       "NumPy oracle"},
            "roofline": _roof(pairs * 25.0, ms, peaks["fp32"], "fp32", 25.0,
                              "incoherent facet sum (main pass + reduce), 25 "
                              "FLOP per pair: range 9, incidence 6, power 5, "
                              "bin 5")}


def row_focus(device, flush, peaks):
    """Focused SAR (time-domain backprojection) of a 1024-trace, 2048-bin
    line at 20 km, 25 m spacing, 60 MHz, 1.9 km hann aperture."""
    import torch
    from radar_sounder_simulator_gb300.processing import (along_track,
                                                          focus_tensor)
    rng = np.random.default_rng(7)
    T, nb, lam, dt, ap = 1024, 2048, 299792458.0 / 60e6, 1.0 / 30e6, 1900.0
    pos = np.column_stack([25.0 * np.arange(T), np.zeros(T),
                           np.full(T, 20000.0)])
    twtt = 2 * 19800.0 / 299792458.0 + np.arange(nb) * dt
    F = (rng.standard_normal((T, nb)) + 1j * rng.standard_normal((T, nb))
         ).astype(np.complex64)
    ft = torch.as_tensor(F, device=device)
    tw = torch.as_tensor(twtt, device=device)
    s = along_track(pos)
    st = torch.as_tensor(s, device=device)
    n_terms = int(sum(np.count_nonzero(np.abs(s - si) <= ap / 2)
                      for si in s)) * nb
    res, ms = {}, {}
    for prec in ("split", "fp64"):
        def run():
            return focus_tensor(ft, tw, st, wavelength=lam, aperture_m=ap,
                                precision=prec, out_dtype=torch.complex128)
        ms[prec] = _events_ms(run, 5 if prec == "split" else 2, flush)
        res[prec] = run()[0]
    # CPU baseline: the float64 oracle (the reference's loop) on a 96-trace
    # piece of the line, one core
    from oracle import processing as oproc
    Ts = 96
    s_s = along_track(pos[:Ts])
    n_cpu = int(sum(np.count_nonzero(np.abs(s_s - si) <= ap / 2)
                    for si in s_s)) * nb
    t0 = time.perf_counter()
    oproc.focused_sar(F[:Ts], twtt, pos[:Ts], lam, ap, "hann")
    cpu_s = time.perf_counter() - t0
    return {"workload": "focus_1024tr_2048bins_20km_25m_1900m_hann",
            "unit": "terms/s", "value": n_terms / (ms["split"] * 1e-3),
            "cpu_baseline": {"value": n_cpu / cpu_s, "unit": "terms/s",
                             "cores": 1, "kind": "port",
                             "sample": f"{Ts} output traces of the same "
                                       "line, float64 NumPy oracle"},
            "terms": n_terms, "ms_per_step": ms["split"],
            "fp64_value": n_terms / (ms["fp64"] * 1e-3),
            "split_over_fp64": ms["fp64"] / ms["split"],
            "roofline": _roof(n_terms * 33.0, ms["split"], peaks["fp32"],
                              "fp32", 33.0, "backprojection (bounds + main "
                              "pass), 33 FLOP per aperture term: delay 12, "
                              "interpolation 9, phase 4, weight and "
                              "accumulate 8"),
            "error_vs_fp64": _errors(res["split"], res["fp64"])}


def row_scene(device, flush):
    """Scene assembly: a 513 x 513 EPSG:3413 DEM window (50 m posting) to
    262,144 local-frame facets, their keyed speckle phasors and a 300 m
    offset interface."""
    import torch
    from oracle import scene as osc
    from radar_sounder_simulator_gb300 import scene as gsc
    rng = np.random.default_rng(11)
    cx, cy = osc.polar_stereo_forward(-40.0, 75.0, "EPSG:3413")
    n, post = 513, 50.0
    tr = (post, 0.0, cx - n * post / 2, 0.0, -post, cy + n * post / 2)
    dem = 800.0 + np.cumsum(rng.normal(0, 1.0, (n, n)), axis=1)
    frame = gsc.LocalFrame(75.0, -40.0, 0.0)

    def dev_step():
        f = gsc.build_facets(dem, tr, "EPSG:3413", frame, device=device,
                             as_tensors=True)
        gsc.speckle_phasors_tensor(f.phase_keys, (3, 1))
        return f
    ms = _events_ms(dev_step, 5, flush)
    f = gsc.build_facets(dem, tr, "EPSG:3413", frame, device=device)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    f = gsc.build_facets(dem, tr, "EPSG:3413", frame, device=device)
    gsc.speckle_phasors_for_keys(f.phase_keys, (3, 1), device=device)
    gsc.offset_facets(f, frame, -300.0, device=device)
    e2e_ms = (time.perf_counter() - t0) * 1e3
    nf = len(f.centers)
    # CPU baseline: the float64 NumPy oracle (the reference's algorithm,
    # projection restated), one core, the same window
    ofr = osc.LocalFrame(75.0, -40.0, 0.0)

    def to_ecef(E, N, h):
        lo, la = osc.polar_stereo_inverse(E, N, "EPSG:3413")
        return osc.geodetic_to_ecef(la, lo, h)
    t0 = time.perf_counter()
    ref = osc.build_facets(dem, tr, to_ecef, ofr.ecef_to_local)
    osc.speckle_phasors_for_keys(ref["phase_keys"], (3, 1))
    osc.offset_centers(ref["centers"], ofr, -300.0)
    cpu_s = time.perf_counter() - t0
    return {"workload": "dem_513sq_epsg3413_to_262144_facets",
            "unit": "facets/s", "value": nf / (ms * 1e-3),
            "ms_per_step": ms,
            "e2e": {"value": nf / (e2e_ms * 1e-3), "ms": e2e_ms,
                    "note": "host DEM in, NumPy facets, phasors and offset "
                            "interface out"},
            "cpu_baseline": {"value": nf / cpu_s, "unit": "facets/s",
                             "cores": 1, "kind": "port",
                             "sample": "the same window, float64 NumPy "
                                       "oracle (facets, phasors, offset)"},
            "note": "device-resident step: lattice upload, vertices, "
                    "corner rule, keyed phasors"}


def row_output(device, flush):
    """Per-trace output products (nadir and first return over every facet)
    of the multilayer scene's surface under its 1024-trace line."""
    import torch
    from radar_sounder_simulator_gb300 import _lib, scenes
    import ctypes as C_
    cfg = scenes.config2()
    f = cfg.layers[0]
    cen = torch.as_tensor(np.ascontiguousarray(f.centers), device=device)
    pos = torch.as_tensor(np.ascontiguousarray(cfg.pos), device=device)
    T, N = len(cfg.pos), len(f.centers)
    L = _lib.lib()
    nb = L.ss_trace_products_scratch_bytes(T, N)
    scratch = torch.empty(nb, dtype=torch.uint8, device=device)
    res = [torch.empty(T, dtype=torch.int64, device=device),
           torch.empty(T, dtype=torch.float64, device=device),
           torch.empty(T, dtype=torch.int64, device=device),
           torch.empty(T, dtype=torch.float64, device=device)]
    o = _lib.TraceProductsOut(*[r.data_ptr() for r in res])
    opts = _lib.TraceProductsOpts(cfg.t0, cfg.dt, cfg.c, cfg.n_samples)
    stream = C_.c_void_p(torch.cuda.current_stream(device).cuda_stream)

    def run():
        _lib.check(L.ss_trace_products(
            C_.byref(opts), C_.c_void_p(cen.data_ptr()), N,
            C_.c_void_p(pos.data_ptr()), T, C_.byref(o),
            C_.c_void_p(scratch.data_ptr()), nb, stream),
            "ss_trace_products")
    ms = _events_ms(run, 5, flush)
    from oracle import output as oout
    t0 = time.perf_counter()
    oout.trace_products(f.centers, cfg.pos[:8], cfg.t0, cfg.dt,
                        cfg.n_samples, cfg.c)
    cpu_s = time.perf_counter() - t0
    return {"workload": "trace_products_262144_facets_1024tr",
            "unit": "pairs/s", "value": T * N / (ms * 1e-3),
            "ms_per_step": ms,
            "cpu_baseline": {"value": 8 * N / cpu_s, "unit": "pairs/s",
                             "cores": 1, "kind": "port",
                             "sample": "8 traces x 262144 facets, float64 "
                                       "NumPy oracle"},
            "note": "nadir facet and first in-window arrival per trace, "
                    "float32 screen + float64 decisions"}


def run_rows(args, device, peak32):
    import torch
    want = [] if args.rows == "none" else args.rows.split(",")
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=device)
    rows = {}
    if not want:
        return rows
    peaks = {"fp32": peak32, "fp64": fp32_peak_tflops(device, fp64=True),
             "mufu_tops": fp32_peak_tflops(device, mufu=True)}
    rows["peaks_tflops"] = {**peaks, "source": "probes measured in this run "
                            "(ss_fp32_fma_probe, ss_fp64_fma_probe, "
                            "ss_mufu_probe)"}
    fns = {"cfg1": lambda: row_cfg1(device, flush, peaks,
                                    min(args.cpu_seconds, 5.0)),
           "modef": lambda: row_modef(device, flush, peaks,
                                      min(args.cpu_seconds, 5.0)),
           "cfg3": lambda: row_cfg3(device, flush, peaks,
                                    0 if args.skip_fp64 else 32,
                                    min(args.cpu_seconds, 5.0)),
           "cfg4": lambda: row_cfg4(device, args.batch_instances, flush,
                                    peaks, min(args.cpu_seconds, 5.0)),
           "cfg5": lambda: row_cfg5(device, flush, peaks,
                                    min(args.cpu_seconds, 5.0)),
           "incoh": lambda: row_incoh(device, flush, peaks),
           "focus": lambda: row_focus(device, flush, peaks),
           "scene": lambda: row_scene(device, flush),
           "output": lambda: row_output(device, flush)}
    for name in want:
        t0 = time.perf_counter()
        try:
            rows[name] = fns[name]()
        except Exception as exc:  # reported, not hidden: the line still prints
            rows[name] = {"error": f"{type(exc).__name__}: {exc}"}
        rows[name]["wall_s"] = time.perf_counter() - t0
        torch.cuda.empty_cache()
    return rows


def _short(err):
    if not isinstance(err, dict) or "rel_l2" not in err:
        return err
    return [float(f"{err['rel_l2']:.2e}"), float(f"{err['phase_rad']:.2e}"),
            float(f"{err['power_db']:.2e}")]


def summarize(line):
    """Compact per-row rates and split-vs-FP64 errors ([rel L2, rad, dB])
    of a bench line."""
    out = {"headline": {"value": float(f"{line['value']:.4g}"),
                        "ms": round(line["ms_per_step"], 2),
                        "err": _short(line.get("error_vs_fp64")),
                        "frac": round(line["roofline"]["frac"], 3)}}
    ex = line["roofline"].get("executed")
    if ex:
        out["headline"]["executed_frac"] = round(ex["frac"], 3)
    rows = line.get("rows") or {}
    for name, r in rows.items():
        if not isinstance(r, dict) or name == "peaks_tflops":
            continue
        if "error" in r:
            out[name] = {"error": r["error"][:120]}
            continue
        e = {"value": float(f"{r.get('value', 0.0):.4g}")}
        if "error_vs_fp64" in r:
            e["err"] = _short(r["error_vs_fp64"])
        if "roofline" in r and isinstance(r["roofline"], dict):
            e["frac"] = round(r["roofline"].get("frac", 0.0), 3)
        if "fd_subset_max_rel_err" in r:
            fd = r["fd_subset_max_rel_err"]
            e["fd"] = ({k: float(f"{v:.2e}") for k, v in fd.items()
                        if isinstance(v, float)} if "error" not in fd
                       else fd["error"][:80])
        if name == "cfg3":
            e["bands"] = {b: {"ms": round(v["ms"], 1),
                              "err": _short(v.get("error_vs_fp64")),
                              "frac": round(v["roofline"]["frac"], 3)}
                          for b, v in r["bands"].items()}
            bt = r.get("batched") or {}
            e["batched"] = ({"ms": round(bt["ms"], 1),
                             "per_call_ms": round(bt["per_call_kernel_ms"],
                                                  1),
                             "rel_l2": float(
                                 f"{bt['max_rel_l2_vs_per_call']:.2e}")}
                            if "ms" in bt else bt.get("error", "")[:80])
        out[name] = e
    return out


def split_error(outs, outs64):
    """Relative L2, max phase error and max power error (dB, bins above -60
    dB of each layer's peak) of the split form against the float64 form."""
    import torch
    worst = {"rel_l2": 0.0, "phase_rad": 0.0, "power_db": 0.0}
    for (f, _), (g, _) in zip(outs, outs64):
        a = torch.view_as_complex(f.contiguous())
        b = torch.view_as_complex(g.contiguous())
        rel = (torch.linalg.vector_norm(a - b) /
               torch.linalg.vector_norm(b)).item()
        p = b.abs() ** 2
        keep = p > p.max() * 1e-6
        ph = torch.angle(a[keep] / b[keep]).abs().max().item()
        db = (10 * torch.log10(a[keep].abs() ** 2 / p[keep])).abs().max().item()
        worst = {"rel_l2": max(worst["rel_l2"], rel),
                 "phase_rad": max(worst["phase_rad"], ph),
                 "power_db": max(worst["power_db"], db)}
    return worst


# --------------------------------------------------------------------------
# roofline: algorithmic FLOP per pair and the measured FP32 FMA rate
# --------------------------------------------------------------------------
# Floating-point operations per (trace, facet) pair of the reference
# algorithm at its fixed budgets (an FMA counts 2; sqrt, divide and the
# transcendental functions count 1 each and are also MUFU work):
#   * smooth isotropic pair, delta-binned (kernels/coherent.py:107-128 plus
#     geometry.py:18-24 and the accumulate): 47;
#   * one sequential crossing (multilayer.py:352-406): 10 + 25 Snell
#     iterations of 20 (multilayer.py:225-240) plus 60 for the facet lookup,
#     plane set-up and Fresnel: 760;
#   * joint path over C crossings, S = C + 1 segments
#     (multilayer.py:408-457, refraction_joint.py:143-322): mean-plane lookup
#     chain 260 C, chain initialiser 560 C, six Newton steps of
#     5 G + 28 S + 61 C + 54 (C - 1) + 58 C + 40 C (one geometry evaluation
#     G = 25 C + 15 S for the step and four for the step-halving candidates,
#     the W blocks, the block-tridiagonal assembly and block-Thomas solve),
#     final polyline 12 S + 80 C;
#   * final leg, radiometry, amplitude, carrier phase and bin: 25 C + 80.
def pair_flops(n_crossed, joint):
    if n_crossed == 0:
        return 47.0
    C = n_crossed
    if not joint:
        return 760.0 * C + 25.0 * C + 80.0
    S = C + 1
    G = 25.0 * C + 15.0 * S
    newton = 5 * G + 28 * S + 61 * C + 54 * (C - 1) + 58 * C + 40 * C
    return (260.0 * C + 560.0 * C + 6 * newton + 12 * S + 80 * C +
            25.0 * C + 80.0)


LAYER_PATHS = [(0, False), (1, False), (2, True), (3, True)]


def fp32_peak_tflops(device, repeats=5, fp64=False, mufu=False):
    """FP32 (or FP64) FMA rate of this GPU in TFLOP/s, or with ``mufu`` the
    MUFU rate in Tops/s, measured with the library's probe kernels (best of
    ``repeats`` launches)."""
    import ctypes as C
    import torch
    from radar_sounder_simulator_gb300 import _lib
    sms = torch.cuda.get_device_properties(device).multi_processor_count
    blocks = 8 * sms
    iters = 1000 if fp64 else (10000 if mufu else 40000)
    out = torch.empty(blocks * 256, dtype=torch.float64 if fp64 else
                      torch.float32, device=device)
    stream = torch.cuda.current_stream(device)
    L = _lib.lib()
    probe = (L.ss_fp64_fma_probe if fp64 else
             L.ss_mufu_probe if mufu else L.ss_fp32_fma_probe)

    def launch():
        _lib.check(probe(blocks, iters, C.c_void_p(out.data_ptr()),
                         C.c_void_p(stream.cuda_stream)), "fma probe")
    for _ in range(3):
        launch()
    best = 0.0
    for _ in range(repeats):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        launch()
        e1.record(stream)
        torch.cuda.synchronize()
        flop = blocks * 256 * 8 * iters * (1.0 if mufu else 2.0)
        best = max(best, flop / (e0.elapsed_time(e1) * 1e-3) / 1e12)
    return best


# FP32 FLOP the bed kernel executes per pair, from the full ncu capture of
# `python bench.py --kernel-only bed` (profiles/refracted_split_bed_512sq_
# 1024tr_full.md): (2 FFMA + FADD + FMUL) per cycle x clock x duration /
# pairs. The canonical count above follows the reference's float64 solve;
# this one is what the float32 pipe runs (fewer Newton steps, table seeds).
EXECUTED_FP32_FLOP_PER_PAIR = {"bed_joint": 3151.0}


def roofline(per_kernel_ms, pairs, peak_tflops, traffic=None):
    """Dominant launch sequence's position against the FP32 pipe."""
    i = int(np.argmax(per_kernel_ms))
    names = ["surface", "h1_seq", "h2_joint", "bed_joint"]
    kernels = ["coherent_split_kernel", "refracted_split_kernel<0>",
               "refracted_split_kernel<2>", "refracted_split_kernel<3>"]
    C, joint = LAYER_PATHS[i]
    fl = pair_flops(C, joint)
    achieved = pairs[i] * fl / (per_kernel_ms[i] * 1e-3) / 1e12
    executed = None
    if names[i] in EXECUTED_FP32_FLOP_PER_PAIR:
        xf = EXECUTED_FP32_FLOP_PER_PAIR[names[i]]
        xa = pairs[i] * xf / (per_kernel_ms[i] * 1e-3) / 1e12
        executed = {"flop_per_pair": xf, "achieved": xa,
                    "frac": xa / peak_tflops,
                    "source": "ncu FFMA/FADD/FMUL counts of this kernel "
                              "(profiles/refracted_split_bed_512sq_1024tr_"
                              "full.md) x the pairs timed here"}
    return {"bound": "fp32", "achieved": achieved, "peak": peak_tflops,
            "unit": "TFLOP/s", "frac": achieved / peak_tflops,
            "executed": executed,
            "traffic": traffic, "kernel": kernels[i], "layer": names[i],
            "flop_per_pair": fl, "pairs_per_launch": pairs[i],
            "ms_per_launch": per_kernel_ms[i],
            "peak_source": "FP32 FMA probe (ss_fp32_fma_probe) measured in "
                           "this run; the measured-peaks file has no FP32 "
                           "figure",
            "timed": "main pass + fix-up + chunk reduce of that layer, CUDA "
                     "events on the launching stream"}


if __name__ == "__main__":
    main()
