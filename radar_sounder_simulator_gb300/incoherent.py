"""Drop-in ``incoherent_cluttergram`` on GB300.

Mirrors soundersim ``kernels/incoherent.py:64-103``: same positional and
keyword arguments, float32 facet, position and window quantisation, NumPy in
and NumPy out (float32 power and dropped). The device program is the CUDA
library (``ss_incoherent_fwd``); there is no CPU path.

``block_size`` is accepted for signature compatibility: the reference uses
it to bound XLA's memory, and it only regroups float32 sums. Extensions:
``device``, and ``prepare_incoherent`` for device-resident inputs.
"""

import ctypes as C

import numpy as np
import torch

from . import _lib
from .coherent import _dev, pattern_struct


class IncoherentPlan:
    """Device-resident inputs of one incoherent_cluttergram call."""

    def __init__(self, **kw):
        self.__dict__.update(kw)

    def run(self, out=None):
        """Launch on the current stream; returns device tensors power
        (T, n_samples[, 2]) float32 and dropped (T,) float32."""
        L = _lib.lib()
        nbytes = L.ss_incoherent_scratch_bytes(C.byref(self.opts), self.T,
                                               self.N)
        if nbytes == 0:
            raise ValueError(
                f"n_samples={self.n_samples} exceeds the incoherent "
                "kernel's shared-memory histogram")
        if self.scratch is None or self.scratch.numel() < nbytes:
            self.scratch = torch.empty(nbytes, dtype=torch.uint8,
                                       device=self.device)
        if out is None:
            shape = (self.T, self.n_samples) + ((2,) if self.split else ())
            power = torch.empty(shape, dtype=torch.float32,
                                device=self.device)
            dropped = torch.empty(self.T, dtype=torch.float32,
                                  device=self.device)
        else:
            power, dropped = out
        o = _lib.IncoherentOutput(power.data_ptr(), dropped.data_ptr())
        stream = torch.cuda.current_stream(self.device).cuda_stream
        st = L.ss_incoherent_fwd(C.byref(self.opts), C.byref(self.fst),
                                 C.byref(self.tr), C.byref(self.pst),
                                 C.byref(o),
                                 C.c_void_p(self.scratch.data_ptr()), nbytes,
                                 C.c_void_p(stream))
        _lib.check(st, "ss_incoherent_fwd")
        return power, dropped

    def kernel_launches(self):
        """Library kernels one ``run()`` launches (main pass + reduce)."""
        return 2


def prepare_incoherent(positions, u_ct, centers, normals, areas, *, t0, dt,
                       n_samples, c, split_sides=False, pattern=None,
                       block_size=65536, device=None):
    """Host preparation of incoherent.py:81-99 and the device upload."""
    device = torch.device(device or "cuda")
    if int(block_size) <= 0:
        raise ValueError(f"block_size must be positive, got {block_size}")
    if pattern is not None and pattern[0] not in _lib.PATTERN:
        raise ValueError(f"unknown pattern kind {pattern[0]!r}")
    pos = np.asarray(positions, np.float64).reshape(-1, 3)
    T = len(pos)
    n = np.asarray(centers).shape[0]
    rows = np.empty((7, n), np.float32)
    rows[0:3] = np.asarray(centers, np.float32).T
    rows[3:6] = np.asarray(normals, np.float32).T
    rows[6] = np.asarray(areas, np.float32)
    soa = torch.from_numpy(rows).to(device)
    f = _lib.Facets()
    base, row = soa.data_ptr(), soa.stride(0) * 4
    for j, nm in enumerate(("cx", "cy", "cz", "nx", "ny", "nz", "area")):
        setattr(f, nm, base + j * row)
    f.n_facets = n
    pst, pv_t, pv_len, keep = pattern_struct(
        pattern if pattern is not None and pattern[0] != "isotropic"
        else None, T, device)
    pos_t = _dev(pos, np.float64, device)
    uct_t = _dev(np.asarray(u_ct, np.float64).reshape(T, 3), np.float64,
                 device)
    tr = _lib.Traces(pos_t.data_ptr(), uct_t.data_ptr(),
                     pv_t.data_ptr() if pv_t is not None else None, None, T,
                     pv_len)
    opts = _lib.IncoherentOpts(float(t0), float(dt), float(c), int(n_samples),
                               int(bool(split_sides)))
    return IncoherentPlan(opts=opts, fst=f, tr=tr, pst=pst,
                          keep=[soa, keep, pos_t, uct_t, pv_t], T=T, N=n,
                          n_samples=int(n_samples), split=bool(split_sides),
                          device=device, scratch=None)


def incoherent_cluttergram(positions, u_ct, centers, normals, areas, *, t0,
                           dt, n_samples, c, split_sides=False, pattern=None,
                           block_size=65536, device=None):
    """Binned incoherent power for every trace (incoherent.py:64-103).

    Returns ``(power, dropped)`` as float32 NumPy arrays: power (T,
    n_samples), or (T, n_samples, 2) [left, right] with ``split_sides``;
    dropped (T,) the out-of-window power."""
    plan = prepare_incoherent(positions, u_ct, centers, normals, areas,
                              t0=t0, dt=dt, n_samples=n_samples, c=c,
                              split_sides=split_sides, pattern=pattern,
                              block_size=block_size, device=device)
    power, dropped = plan.run()
    return power.cpu().numpy(), dropped.cpu().numpy()
