"""Drop-in ``coherent_cluttergram`` on GB300.

Mirrors soundersim ``kernels/coherent.py:247-362``: same positional and
keyword arguments, the same host conventions (float32 facet quantisation,
along-track culling, ``ValueError`` texts), NumPy in and NumPy out. The
device program is the CUDA library (``ss_coherent_fwd``); there is no CPU
path.

Extensions (keyword-only, defaults keep the reference behaviour):
``precision`` -- "fp64" (default, the float64 form) or "split" (float32 bulk
with double-float range, phase and bins); ``out_dtype`` -- complex64
(reference) or complex128; ``roughness`` may carry per-facet (N,) sigma and
correlation-length arrays in place of the scalars.
"""

import ctypes as C

import numpy as np
import torch

from . import _lib
from .geometry import cull_plan, group_within_blocks

TWO_PI = 2.0 * np.pi


def _dev(a, dtype, device):
    return torch.from_numpy(np.ascontiguousarray(a, dtype=dtype)).to(
        device, non_blocking=False)


def _ptr(t):
    return C.c_void_p(t.data_ptr()) if t is not None else C.c_void_p(0)


def to_host(t):
    """Device tensor -> NumPy array through a page-locked buffer (the fast
    device-to-host path; torch caches the page-locked blocks)."""
    if t.device.type != "cuda":
        return t.numpy()
    h = torch.empty(t.shape, dtype=t.dtype, pin_memory=True)
    h.copy_(t)
    return h.numpy()


def _field_to_host(field, out_dtype):
    """(T, n, 2) float64 re/im device field -> host complex array; the
    complex dtype is formed on the device so only its bytes cross to the
    host."""
    if np.dtype(out_dtype) == np.complex64:
        return to_host(torch.view_as_complex(field.to(torch.float32)))
    if np.dtype(out_dtype) == np.complex128:
        return to_host(torch.view_as_complex(field.contiguous()))
    f = to_host(field)
    return (f[..., 0] + 1j * f[..., 1]).astype(out_dtype)


class DeviceFacets:
    """Target facets staged on the device in along-track order (SoA)."""

    def __init__(self, soa, extras, n):
        self.soa = soa          # (13, N) float32: c(3) n(3) e1(3) e2(3) area
        self.extras = extras    # name -> tensor (gamma_f32, sigma, corr, ...)
        self.n = n

    def struct(self):
        f = _lib.Facets()
        names = ("cx", "cy", "cz", "nx", "ny", "nz", "e1x", "e1y", "e1z",
                 "e2x", "e2y", "e2z", "area")
        row = self.soa.stride(0) * 4
        base = self.soa.data_ptr()
        for j, nm in enumerate(names):
            setattr(f, nm, base + j * row)
        for nm, t in self.extras.items():
            setattr(f, nm, t.data_ptr())
        f.n_facets = self.n
        return f


def permuted(a, dtype, order, device):
    """``a[order]`` as a device tensor of ``dtype``: gathered on the device
    when the order is a device tensor, on the host otherwise."""
    a = np.ascontiguousarray(a, dtype)
    if isinstance(order, torch.Tensor):
        return torch.from_numpy(a).to(device).index_select(0, order)
    return _dev(a[order], dtype, device)


def stage_facets(centers, normals, areas, e1, e2, order, device, *,
                 gamma=None, sigma=None, corr=None, phasors=None):
    """Upload the float64 facet arrays as they are and form the float32
    facet SoA on the device: quantisation, along-track permutation (a
    gather) and transposition run there, the host does no per-facet
    arithmetic."""
    n = len(order)

    def up(a, cols):
        t = torch.from_numpy(np.ascontiguousarray(a, np.float64)).to(device)
        return t.reshape(n, cols)
    rows_t = torch.cat([up(centers, 3), up(normals, 3), up(e1, 3), up(e2, 3),
                        up(areas, 1)], 1)
    order_t = (order if isinstance(order, torch.Tensor) else
               torch.from_numpy(np.ascontiguousarray(order, np.int64)).to(
                   device))
    soa = rows_t.to(torch.float32).index_select(0, order_t).t().contiguous()
    extras = {}
    if gamma is not None:
        extras["gamma_f32"] = permuted(gamma, np.float32, order_t, device)
    if sigma is not None:
        extras["sigma"] = permuted(sigma, np.float32, order_t, device)
    if corr is not None:
        extras["corr"] = permuted(corr, np.float32, order_t, device)
    if phasors is not None:
        ph = np.ascontiguousarray(phasors, np.complex64).view(
            np.float32).reshape(n, 2)
        extras["phasor"] = permuted(ph, np.float32, order_t,
                                    device).reshape(-1)
    return DeviceFacets(soa, extras, n)


def pattern_struct(pattern, n_traces, device):
    """(kind, pv, pa, pb) tuple -> (Pattern struct, pv tensor, keep-alive)."""
    if pattern is None:
        return _lib.Pattern(0, 0, None, None), None, 0, []
    kind, pv, pa, pb = pattern
    if kind not in _lib.PATTERN:
        raise ValueError(f"unknown pattern kind {kind!r}")
    pv = np.asarray(pv, np.float64).reshape(n_traces, -1)
    pa = np.atleast_1d(np.asarray(pa, np.float64))
    pb = np.atleast_1d(np.asarray(pb, np.float64))
    n = 0
    if kind == "array_tapered":
        n = pa.shape[-1] if pa.ndim > 1 else len(pa) // 2
    elif kind == "tabulated":
        n = len(pa)
    pa_t = _dev(pa.ravel(), np.float64, device)
    pb_t = _dev(pb.ravel(), np.float64, device)
    pv_t = _dev(pv, np.float64, device)
    st = _lib.Pattern(_lib.PATTERN[kind], n, pa_t.data_ptr(), pb_t.data_ptr())
    return st, pv_t, pv.shape[1], [pa_t, pb_t]


def rough_struct(roughness, d_phi_area):
    """Reference roughness tuple -> (Roughness struct, per-facet arrays)."""
    if roughness is None:
        return _lib.Roughness(_lib.ROUGH_NONE, 0, 0.0, 0.0), None, None, None
    sigma, lcorr, phasors, n_terms, *rest = roughness
    acf = rest[0] if rest else "gaussian"
    if acf == "exponential" and not d_phi_area:
        raise ValueError("roughness acf='exponential' requires the "
                         "area-only D_Phi (d_phi_area / grazing fix)")
    if acf not in ("gaussian", "exponential"):
        raise ValueError(f"unknown roughness acf {acf!r} (want one of "
                         "('gaussian', 'exponential'))")
    kind = (_lib.ROUGH_EXP_AREA if acf == "exponential" else
            _lib.ROUGH_GAUSS_AREA if d_phi_area else _lib.ROUGH_GAUSS_FULL)
    s_arr = sigma if np.ndim(sigma) else None
    l_arr = lcorr if np.ndim(lcorr) else None
    st = _lib.Roughness(kind, int(n_terms),
                        0.0 if s_arr is not None else float(sigma),
                        0.0 if l_arr is not None else float(lcorr))
    return st, s_arr, l_arr, phasors


class CoherentPlan:
    """Device-resident inputs of one coherent_cluttergram call."""

    def __init__(self, **kw):
        self.__dict__.update(kw)

    def run(self, precision=None, out=None):
        """Launch on the current stream; returns device tensors (field
        (T, n_seg, 2) float64 re/im in the output layout, dropped (T,))."""
        self.opts.precision = _lib.PREC[precision or self.precision]
        L = _lib.lib()
        nbytes = L.ss_coherent_scratch_bytes(C.byref(self.opts), self.T,
                                             self.N)
        if nbytes == 0:
            raise ValueError("unsupported sizes for the coherent kernel")
        if self.scratch is None or self.scratch.numel() < nbytes:
            self.scratch = torch.empty(nbytes, dtype=torch.uint8,
                                       device=self.device)
        if out is None:
            field = torch.empty((self.T, self.n_seg, 2), dtype=torch.float64,
                                device=self.device)
            dropped = torch.empty(self.T, dtype=torch.float64,
                                  device=self.device)
        else:
            field, dropped = out
        o = _lib.Output(field.data_ptr(), None, dropped.data_ptr())
        stream = torch.cuda.current_stream(self.device).cuda_stream
        st = L.ss_coherent_fwd(C.byref(self.opts), C.byref(self.fst),
                               C.byref(self.tr), C.byref(self.pst),
                               C.byref(self.rst), C.byref(o),
                               C.c_void_p(self.scratch.data_ptr()), nbytes,
                               C.c_void_p(stream))
        _lib.check(st, "ss_coherent_fwd")
        return field, dropped

    def kernel_launches(self):
        """Library kernels one ``run()`` launches (main pass + chunk
        reduce)."""
        return 2

    def to_numpy(self, field, dropped, out_dtype=np.complex64):
        res = _field_to_host(field, out_dtype)
        if self.split:
            res = res.reshape(self.T, self.n_samples, 2)
        return res, to_host(dropped.to(torch.float32))


def coherent_run_count(plan):
    """Library kernels one ``run()`` launches (main pass + chunk reduce)."""
    return plan.kernel_launches()


def prepare_coherent(positions, u_ct, centers, normals, areas, e1, e2, *, k,
                     gamma, t0, dt, n_samples, c, split_sides=False,
                     interp_bins=False, pattern=None, roughness=None,
                     taper_s=None, d_phi_area=False, block_size=None,
                     window_cull=True, precision="fp64", device=None):
    """Host preparation of coherent.py:284-348 and the device upload."""
    device = torch.device(device or "cuda")
    pos = np.asarray(positions, np.float64)
    T = len(pos)
    n = np.asarray(centers).shape[0]
    # argument errors come before any device work, as in the reference
    if precision not in _lib.PREC:
        raise ValueError(f"unknown precision {precision!r}")
    gamma_arr = np.asarray(gamma, np.float32)
    gamma_facet = gamma_arr.ndim > 0
    if gamma_facet and gamma_arr.shape != (n,):
        raise ValueError(f"per-facet gamma shape {gamma_arr.shape} != ({n},)")
    rst, s_arr, l_arr, phasors = rough_struct(roughness, d_phi_area)
    if pattern is not None and pattern[0] not in _lib.PATTERN:
        raise ValueError(f"unknown pattern kind {pattern[0]!r}")
    plan = cull_plan(pos, centers, t0=t0, dt=dt, n_samples=n_samples, c=c,
                     block_size=block_size, target_pairs=1 << 19,
                     window_cull=window_cull, device=device)
    if s_arr is not None:     # per-facet rms heights: similar series lengths
        plan = group_within_blocks(plan, s_arr)   # share a warp
    fac = stage_facets(centers, normals, areas, e1, e2, plan.order, device,
                       gamma=gamma_arr if gamma_facet else None,
                       sigma=s_arr, corr=l_arr, phasors=phasors)
    pst, pv_t, pv_len, keep = pattern_struct(pattern, T, device)
    pos_t = _dev(pos, np.float64, device)
    uct_t = _dev(np.asarray(u_ct, np.float64).reshape(T, 3), np.float64,
                 device)
    off_t = _dev(plan.off, np.int32, device)
    tr = _lib.Traces(pos_t.data_ptr(), uct_t.data_ptr(),
                     pv_t.data_ptr() if pv_t is not None else None,
                     off_t.data_ptr(), T, pv_len)
    opts = _lib.CoherentOpts(
        float(k), 0.0 if gamma_facet else float(gamma), float(t0), float(dt),
        float(c), float(taper_s or 0.0), int(n_samples), plan.block_size,
        plan.n_win, int(bool(split_sides)), int(bool(interp_bins)),
        int(taper_s is not None), _lib.PREC[precision])
    return CoherentPlan(
        opts=opts, fst=fac.struct(), tr=tr, pst=pst, rst=rst,
        keep=[fac, keep, pos_t, uct_t, off_t, pv_t], T=T, N=n,
        n_samples=int(n_samples),
        n_seg=int(n_samples) * (2 if split_sides else 1),
        split=bool(split_sides), device=device, precision=precision,
        scratch=None, cull=plan)


def coherent_cluttergram(positions, u_ct, centers, normals, areas, e1, e2, *,
                         k, gamma, t0, dt, n_samples, c, split_sides=False,
                         interp_bins=False, pattern=None, roughness=None,
                         taper_s=None, d_phi_area=False, block_size=None,
                         window_cull=True, precision="fp64",
                         out_dtype=np.complex64, device=None):
    """Binned coherent field for every trace (coherent.py:247-362).

    Returns ``(field, dropped)``: field (T, n_samples) or (T, n_samples, 2)
    [left, right] with the absolute carrier phase, dropped (T,) float32
    out-of-window power."""
    plan = prepare_coherent(
        positions, u_ct, centers, normals, areas, e1, e2, k=k, gamma=gamma,
        t0=t0, dt=dt, n_samples=n_samples, c=c, split_sides=split_sides,
        interp_bins=interp_bins, pattern=pattern, roughness=roughness,
        taper_s=taper_s, d_phi_area=d_phi_area, block_size=block_size,
        window_cull=window_cull, precision=precision, device=device)
    field, dropped = plan.run()
    return plan.to_numpy(field, dropped, out_dtype)
