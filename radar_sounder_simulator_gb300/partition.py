"""One call's traces partitioned across ranks (one process per GPU).

Every trace's bins depend only on the read-only facet set: the reference
maps its per-trace program over traces (``kernels/coherent.py:243-244``,
``kernels/multilayer.py:590-591``), so a call shards by trace with no
exchange in the forward pass. Each rank takes a contiguous slice of the
track, holds a full copy of the facets (about 21 MB per 262,144-facet
layer), runs the kernels on its slice, and the outputs are concatenated in
trace order. Per-facet gradients of a loss that sums over traces (the
adjoint's dL/dR, dL/dsigma, dL/dalpha) are sums of the ranks' partial
gradients, so one sum all-reduce finishes the backward pass.

The split is contiguous so each rank's along-track order of the facets is
the order of the whole track (the track axis of a straight line is the same
for any slice of it), which keeps every in-window contribution of a trace
in the same summation sequence as the single call. ``dropped`` counts the
out-of-window power of each rank's own culling window, as it does for any
batch of traces in the reference.

Works with any ``torch.distributed`` backend: NCCL with device tensors
between GPUs, gloo with host tensors.
"""

import numpy as np
import torch
import torch.distributed as dist


def world(group=None):
    """(rank, world size) of the default or given group; (0, 1) when the
    process group is not initialised."""
    if not (dist.is_available() and dist.is_initialized()):
        return 0, 1
    return dist.get_rank(group), dist.get_world_size(group)


def trace_slices(n_traces, world_size):
    """Contiguous, balanced slices of ``range(n_traces)``, one per rank (the
    first ``n_traces % world_size`` ranks take one extra trace)."""
    if world_size < 1:
        raise ValueError("world_size must be >= 1")
    base, extra = divmod(int(n_traces), world_size)
    out, start = [], 0
    for r in range(world_size):
        stop = start + base + (1 if r < extra else 0)
        out.append(slice(start, stop))
        start = stop
    return out


def _as_tensor(x, device):
    t = torch.as_tensor(np.ascontiguousarray(x)) if isinstance(
        x, np.ndarray) else x
    return t.to(device)


def gather_traces(local, n_traces, group=None, device=None):
    """Concatenate every rank's per-trace block (leading axis = the rank's
    traces, as ``trace_slices`` cuts them) into the whole track's array.
    ``local`` is a NumPy array or a tensor; returns the same kind. Ranks pad
    to the longest slice for the collective and trim after it."""
    rank, ws = world(group)
    is_np = isinstance(local, np.ndarray)
    if ws == 1:
        return local
    slices = trace_slices(n_traces, ws)
    dev = device or (torch.device("cpu") if is_np else local.device)
    t = _as_tensor(local, dev)
    if np.iscomplexobj(local) if is_np else t.is_complex():
        t = torch.view_as_real(t.contiguous())
    longest = max(s.stop - s.start for s in slices)
    pad = torch.zeros((longest,) + tuple(t.shape[1:]), dtype=t.dtype,
                      device=dev)
    pad[:t.shape[0]] = t
    parts = [torch.empty_like(pad) for _ in range(ws)]
    dist.all_gather(parts, pad, group=group)
    full = torch.cat([p[:s.stop - s.start] for p, s in zip(parts, slices)])
    if np.iscomplexobj(local) if is_np else local.is_complex():
        full = torch.view_as_complex(full.contiguous())
    return full.cpu().numpy() if is_np else full


def allreduce_sum(*tensors, group=None):
    """Sum every rank's partial (per-facet gradients, scalars) in place;
    returns the tensors."""
    _, ws = world(group)
    if ws > 1:
        for t in tensors:
            dist.all_reduce(t, op=dist.ReduceOp.SUM, group=group)
    return tensors


def sharded_call(fn, positions, u_ct, *args, pattern=None, group=None,
                 device=None, **kw):
    """Run ``fn(positions, u_ct, *args, pattern=..., **kw)`` -- a drop-in
    call such as ``coherent_cluttergram`` or ``refracted_cluttergram`` that
    returns ``(field, dropped)`` with traces on the leading axis -- on this
    rank's slice of the track, then gather the whole track's outputs on
    every rank. Per-trace pattern vectors (``pattern[1]``) are sliced with
    the track."""
    rank, ws = world(group)
    pos = np.asarray(positions)
    sl = trace_slices(len(pos), ws)[rank]
    if pattern is not None:
        kind, pv, pa, pb = pattern
        pattern = (kind, np.asarray(pv)[sl], pa, pb)
        kw["pattern"] = pattern
    field, dropped = fn(pos[sl], np.asarray(u_ct)[sl], *args, **kw)
    return (gather_traces(field, len(pos), group, device),
            gather_traces(dropped, len(pos), group, device))
