"""Trace partition of one call across ranks, on CPU: two gloo ranks each run
the float64 oracle on their contiguous slice of the track, the helper
gathers the slices, and the concatenation equals the single-rank call (the
field bit for bit: each trace's in-window contributions are summed in the
same order). Per-facet partial sums over each rank's traces, all-reduced,
equal the whole track's sums (the adjoint's gradient reduction)."""

import os
import socket

import numpy as np
import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

from radar_sounder_simulator_gb300.partition import trace_slices


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_trace_slices_cover_the_track_in_order():
    for n, ws in ((10, 3), (8, 2), (5, 8), (1024, 4)):
        sl = trace_slices(n, ws)
        assert len(sl) == ws
        idx = np.concatenate([np.arange(n)[s] for s in sl])
        np.testing.assert_array_equal(idx, np.arange(n))
        sizes = [s.stop - s.start for s in sl]
        assert max(sizes) - min(sizes) <= 1
    with pytest.raises(ValueError):
        trace_slices(4, 0)


def _facet_power(pos, f, k):
    """Per-facet sum over the given traces of |LPA contribution|^2 (a
    per-facet quantity summed over traces, like an adjoint gradient)."""
    from oracle import lpa
    acc = np.zeros(len(f.centers))
    for p in pos:
        c, _ = lpa.lpa_field(p, f.centers, f.normals, f.areas, f.e1, f.e2, k,
                             -0.279)
        acc += np.abs(c) ** 2
    return acc


def _rank(rank, ws, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port),
                      RANK=str(rank), WORLD_SIZE=str(ws))
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    from oracle import lpa
    from oracle import refracted as oref
    from radar_sounder_simulator_gb300.partition import (allreduce_sum,
                                                         sharded_call, world)
    from tests.test_oracle_golden import refracted_case
    from tests.util import facets_from
    g = dict(np.load(os.path.join(os.path.dirname(__file__), "golden",
                                  "coherent.npz")))
    f = facets_from(g, "surf")
    kw = dict(k=float(g["k"]), gamma=-0.279, t0=float(g["t0"]),
              dt=float(g["dt"]), n_samples=int(g["n_samples"]),
              c=299792458.0)
    args = (f.centers, f.normals, f.areas, f.e1, f.e2)
    field, dropped = sharded_call(lpa.coherent_cluttergram, g["pos"],
                                  g["uct"], *args, **kw)
    r = dict(np.load(os.path.join(os.path.dirname(__file__), "golden",
                                  "refracted.npz")))
    pos, uct, tgt, crossed, e, a, rkw = refracted_case(r, "joint2")
    rfield, _ = sharded_call(oref.refracted_cluttergram, pos, uct, tgt,
                             crossed, e, a, **rkw)
    # per-facet partial sums over this rank's traces, then all-reduced
    rk, n = world()
    from radar_sounder_simulator_gb300.partition import trace_slices as ts
    part = _facet_power(g["pos"][ts(len(g["pos"]), n)[rk]], f, kw["k"])
    t = torch.from_numpy(part)
    allreduce_sum(t)
    out[rank] = (field, dropped, rfield, t.numpy())
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_ranks_equal_the_single_call():
    from oracle import lpa
    from oracle import refracted as oref
    from tests.test_oracle_golden import refracted_case
    from tests.util import facets_from
    ws = 2
    port = _free_port()
    with mp.Manager() as man:
        out = man.dict()
        mp.spawn(_rank, args=(ws, port, out), nprocs=ws, join=True)
        res = dict(out)
    g = dict(np.load(os.path.join(os.path.dirname(__file__), "golden",
                                  "coherent.npz")))
    f = facets_from(g, "surf")
    kw = dict(k=float(g["k"]), gamma=-0.279, t0=float(g["t0"]),
              dt=float(g["dt"]), n_samples=int(g["n_samples"]),
              c=299792458.0)
    args = (g["pos"], g["uct"], f.centers, f.normals, f.areas, f.e1, f.e2)
    want, want_drop = lpa.coherent_cluttergram(*args, **kw)
    r = dict(np.load(os.path.join(os.path.dirname(__file__), "golden",
                                  "refracted.npz")))
    pos, uct, tgt, crossed, e, a, rkw = refracted_case(r, "joint2")
    rwant, _ = oref.refracted_cluttergram(pos, uct, tgt, crossed, e, a,
                                          **rkw)
    full_power = _facet_power(g["pos"], f, kw["k"])
    for rank in range(ws):
        field, dropped, rfield, power = res[rank]
        np.testing.assert_array_equal(field, want)
        np.testing.assert_array_equal(rfield, rwant)
        assert dropped.shape == want_drop.shape
        np.testing.assert_allclose(power, full_power, rtol=1e-12)
