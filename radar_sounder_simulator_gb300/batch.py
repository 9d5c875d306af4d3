"""Batched coherent facet sums: one persistent work-queue launch for many
independent jobs, replayed as a CUDA graph, with an autotuned work
decomposition.

The reference calls ``coherent_cluttergram`` (kernels/coherent.py:247-362)
once per scene; a design sweep (many instruments, altitudes, frequencies,
track lengths and scene sizes) is then a long series of small, uneven
launches. ``CoherentBatch`` takes the device plans of any number of such
calls (``prepare_coherent``) and runs them together:

* ``ss_coherent_batch_prepare`` cuts every job into work items of about
  equal size (trace block x facet chunk) and uploads the job table once;
* ``run()`` is one persistent kernel pulling items from a global queue plus
  one batched reduce -- stream operations only;
* ``capture()`` records ``run()`` into a ``torch.cuda.CUDAGraph``;
  ``replay()`` relaunches it with no host work;
* ``autotune()`` times candidate decompositions (CTA size, traces per item,
  items per SM) on the batch itself and keeps the fastest; results are
  cached per batch signature for the process (and optionally in a JSON
  file).
"""

import ctypes as C
import itertools
import json
import math
import os

import numpy as np
import torch

from . import _lib
from .coherent import prepare_coherent

_TUNE_CACHE = {}


CoherentJob = _lib.CoherentJob
BatchTuning = _lib.BatchTuning
BatchInfo = _lib.BatchInfo


DEFAULT_TUNING = (256, 8, 16, 0)
# (512-thread CTAs take smooth split-precision batches only; a batch that
# refuses a candidate skips it)
CANDIDATES = [(t, tb, ips, 0) for t, tb, ips in itertools.product(
    (128, 256, 512), (2, 4, 8), (4, 16, 64))]


class CoherentBatch:
    """Many ``prepare_coherent`` plans run as one persistent launch."""

    def __init__(self, plans, tuning=None):
        if not plans:
            raise ValueError("empty batch")
        self.plans = list(plans)
        self.device = self.plans[0].device
        precs = {p.precision for p in self.plans}
        if len(precs) != 1:
            raise ValueError("all jobs of a batch need the same precision")
        self.precision = precs.pop()
        self.L = _lib.lib()
        self.outputs = []
        jobs = (CoherentJob * len(self.plans))()
        for j, p in enumerate(self.plans):
            p.opts.precision = _lib.PREC[self.precision]
            field = torch.empty((p.T, p.n_seg, 2), dtype=torch.float64,
                                device=self.device)
            dropped = torch.empty(p.T, dtype=torch.float64,
                                  device=self.device)
            self.outputs.append((field, dropped))
            jobs[j].opts = p.opts
            jobs[j].facets = p.fst
            jobs[j].traces = p.tr
            jobs[j].pattern = p.pst
            jobs[j].rough = p.rst
            jobs[j].out = _lib.Output(field.data_ptr(), None,
                                      dropped.data_ptr())
        self.jobs = jobs
        self.scratch = None
        self.graph = None
        self.prepare(tuning or DEFAULT_TUNING)

    # -- signature of the work, the key of the tuning cache
    def signature(self):
        pairs = sum(p.T * min(p.cull.n_win * p.cull.block_size, p.N)
                    for p in self.plans)
        nseg = max(p.n_seg for p in self.plans)
        return (len(self.plans), self.precision,
                int(self.plans[0].rst.kind), int(round(math.log2(
                    max(pairs, 1)))), nseg,
                torch.cuda.get_device_name(self.device))

    def prepare(self, tuning):
        """Lay out scratch and upload the job table for ``tuning`` =
        (threads, max traces per item, items per SM, CTAs per SM)."""
        t = BatchTuning(*[int(v) for v in tuning])
        n = self.L.ss_coherent_batch_scratch_bytes(self.jobs, len(self.jobs),
                                                   C.byref(t))
        if n == 0:
            msg = self.L.ss_last_error().decode(errors="replace")
            raise ValueError(f"batch layout failed: {msg}")
        if self.scratch is None or self.scratch.numel() < n:
            self.scratch = torch.empty(n, dtype=torch.uint8,
                                       device=self.device)
        info = BatchInfo()
        torch.cuda.synchronize(self.device)
        st = self.L.ss_coherent_batch_prepare(
            self.jobs, len(self.jobs), C.byref(t),
            C.c_void_p(self.scratch.data_ptr()), n, C.byref(info))
        _lib.check(st, "ss_coherent_batch_prepare")
        self.info = info
        self.tuning = tuple(int(v) for v in tuning)
        self.graph = None
        return info

    def kernel_launches(self):
        """Library kernels one ``run()`` launches (persistent pass + batched
        reduce)."""
        return 2

    def run(self):
        """Launch on the current stream; returns [(field, dropped)] per job
        (device tensors, the ``CoherentPlan.run`` layout)."""
        stream = torch.cuda.current_stream(self.device).cuda_stream
        st = self.L.ss_coherent_batch_run(
            C.byref(self.info), C.c_void_p(self.scratch.data_ptr()),
            C.c_void_p(stream))
        _lib.check(st, "ss_coherent_batch_run")
        return self.outputs

    def capture(self):
        """Record ``run()`` into a CUDA graph (after one eager warm-up)."""
        s = torch.cuda.Stream(self.device)
        s.wait_stream(torch.cuda.current_stream(self.device))
        with torch.cuda.stream(s):
            self.run()
        torch.cuda.current_stream(self.device).wait_stream(s)
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            self.run()
        self.graph = g
        return g

    def replay(self):
        if self.graph is None:
            self.capture()
        self.graph.replay()
        return self.outputs

    def time_run(self, reps=3):
        """Median device time of ``run()`` (ms), CUDA events."""
        self.run()
        ts = []
        for _ in range(reps):
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record()
            self.run()
            e1.record()
            torch.cuda.synchronize(self.device)
            ts.append(e0.elapsed_time(e1))
        return float(np.median(ts))

    def autotune(self, candidates=None, reps=2, cache_path=None):
        """Time each candidate decomposition on this batch, keep the fastest
        (cached per signature). Returns (tuning, ms)."""
        key = repr(self.signature())
        cache = _TUNE_CACHE
        if cache_path and os.path.exists(cache_path):
            with open(cache_path) as fh:
                cache.update(json.load(fh))
        if key in cache:
            tun, ms = cache[key]
            self.prepare(tun)
            return tuple(tun), ms
        best = None
        for cand in candidates or CANDIDATES:
            try:
                self.prepare(cand)
            except ValueError:
                continue
            ms = self.time_run(reps)
            if best is None or ms < best[1]:
                best = (tuple(cand), ms)
        self.prepare(best[0])
        cache[key] = [list(best[0]), best[1]]
        if cache_path:
            with open(cache_path, "w") as fh:
                json.dump(cache, fh)
        return best

    def to_numpy(self, out_dtype=np.complex64):
        res = []
        for p, (field, dropped) in zip(self.plans, self.outputs):
            res.append(p.to_numpy(field, dropped, out_dtype))
        return res


def coherent_batch(jobs, *, precision="split", tuning=None, autotune=False,
                   out_dtype=np.complex64, device=None):
    """Run many ``coherent_cluttergram`` calls (each a dict of its positional
    arguments under ``args`` and its keywords) as one batched launch;
    returns the list of ``(field, dropped)`` NumPy results in job order."""
    plans = [prepare_coherent(*j["args"], **{k: v for k, v in j.items()
                                             if k != "args"},
                              precision=precision, device=device)
             for j in jobs]
    b = CoherentBatch(plans, tuning)
    if autotune:
        b.autotune()
    b.run()
    return b.to_numpy(out_dtype)


class RefractedBatch:
    """Many ``prepare_refracted`` plans (split form) run as one persistent
    launch: the reference's simulate() calls refracted_cluttergram once per
    target layer and band (simulate.py:338-381); here every such call of
    one path class (the sequential chain, or the joint solve through the
    same interface count), roughness kind and antenna table shares one work
    queue, one batched fix-up and one batched reduce."""

    def __init__(self, plans, tuning=None):
        if not plans:
            raise ValueError("empty batch")
        self.plans = list(plans)
        self.device = self.plans[0].device
        self.L = _lib.lib()
        self.outputs = []
        jobs = (_lib.RefractedJob * len(self.plans))()
        for j, p in enumerate(self.plans):
            p.opts.precision = _lib.PREC["split"]
            field = torch.empty((p.T, p.n_seg, 2), dtype=torch.float64,
                                device=self.device)
            dropped = torch.empty(p.T, dtype=torch.float64,
                                  device=self.device)
            self.outputs.append((field, dropped))
            jobs[j].opts = p.opts
            jobs[j].target = p.fst
            jobs[j].traces = p.tr
            jobs[j].pattern = p.pst
            jobs[j].rough = p.rst
            jobs[j].out = _lib.Output(field.data_ptr(), None,
                                      dropped.data_ptr())
        self.jobs = jobs
        self.scratch = None
        self.prepare(tuning or (512, 8, 16, 0))

    def prepare(self, tuning):
        """Lay out scratch and upload the job table for ``tuning`` =
        (threads: 512, max traces per item, items per SM, CTAs per SM)."""
        t = BatchTuning(*[int(v) for v in tuning])
        n = self.L.ss_refracted_batch_scratch_bytes(self.jobs, len(self.jobs),
                                                    C.byref(t))
        if n == 0:
            msg = self.L.ss_last_error().decode(errors="replace")
            raise ValueError(f"batch layout failed: {msg}")
        if self.scratch is None or self.scratch.numel() < n:
            self.scratch = torch.empty(n, dtype=torch.uint8,
                                       device=self.device)
        info = _lib.RefractedBatchInfo()
        torch.cuda.synchronize(self.device)
        st = self.L.ss_refracted_batch_prepare(
            self.jobs, len(self.jobs), C.byref(t),
            C.c_void_p(self.scratch.data_ptr()), n, C.byref(info))
        _lib.check(st, "ss_refracted_batch_prepare")
        self.info = info
        self.tuning = tuple(int(v) for v in tuning)
        return info

    def kernel_launches(self):
        """Library kernels one ``run()`` launches (persistent pass, batched
        fix-up, batched reduce)."""
        return 3

    def run(self):
        """Launch on the current stream; returns [(field, dropped)] per job
        (device tensors, the ``RefractedPlan.run`` layout)."""
        stream = torch.cuda.current_stream(self.device).cuda_stream
        st = self.L.ss_refracted_batch_run(
            C.byref(self.info), C.c_void_p(self.scratch.data_ptr()),
            C.c_void_p(stream))
        _lib.check(st, "ss_refracted_batch_run")
        return self.outputs

    def to_numpy(self, out_dtype=None):
        return [p.to_numpy(f, d, out_dtype)
                for p, (f, d) in zip(self.plans, self.outputs)]


class BatchGraph:
    """Several batches (and any other stream work) captured into one CUDA
    graph, so a multi-layer, multi-band step is one replay: ``steps`` are
    callables that only enqueue device work on the current stream (e.g.
    ``CoherentBatch.run``, ``RefractedBatch.run``, pulse compression)."""

    def __init__(self, steps, device=None):
        self.steps = list(steps)
        self.device = torch.device(device or "cuda")
        self.graph = None

    def run(self):
        for fn in self.steps:
            fn()

    def capture(self):
        s = torch.cuda.Stream(self.device)
        s.wait_stream(torch.cuda.current_stream(self.device))
        with torch.cuda.stream(s):
            self.run()          # eager warm-up on a side stream
        torch.cuda.current_stream(self.device).wait_stream(s)
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            self.run()
        self.graph = g
        return g

    def replay(self):
        if self.graph is None:
            self.capture()
        self.graph.replay()
