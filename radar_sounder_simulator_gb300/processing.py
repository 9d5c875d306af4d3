"""Focused SAR (time-domain backprojection) on GB300.

Mirrors soundersim ``processing.py:262-348`` (``focused_sar``): the same
Dataset in, Dataset out contract (a 2-D coherent ``field`` over
(slow_time, twtt), the ``wavelength`` attr, ``c`` from the run config, the
lambda/4 Doppler guard warning, the ``processing`` provenance attr), with the
per-trace backprojection loop on the GPU (``ss_focused_sar``). There is no
CPU path.

``focus_field`` is the same operation on plain arrays, and ``focus_tensor``
on device tensors (a field straight from the facet kernels). ``precision``:
"fp64" (default; the reference's float64 chain) or "split" (float32
arithmetic, about 60x faster).
"""

import ctypes as C
import json
import warnings

import numpy as np
import torch

from . import _lib

C_DEFAULT = 299792458.0
WINDOWS = {"hann": _lib.WIN_HANN, "none": _lib.WIN_RECT,
           "rect": _lib.WIN_RECT, None: _lib.WIN_RECT}


def along_track(positions):
    """Cumulative along-track arc length, s[0] = 0 (processing.py:65-69)."""
    pos = np.asarray(positions, np.float64)
    seg = np.linalg.norm(np.diff(pos, axis=0), axis=1)
    return np.concatenate([[0.0], np.cumsum(seg)])


def mean_spacing(positions):
    pos = np.asarray(positions, np.float64)
    if pos.shape[0] < 2:
        return 0.0
    return float(np.linalg.norm(np.diff(pos, axis=0), axis=1).mean())


def doppler_guard(spacing, wavelength, aperture_m, r_ref, op):
    """Warn when the trace spacing under-samples a point target's Doppler
    history: spacing > lambda / (4 sin theta_max) (processing.py:241-259)."""
    if r_ref <= 0:
        return
    theta = np.arctan((aperture_m / 2.0) / r_ref)
    st = np.sin(theta)
    if st <= 0:
        return
    crit = wavelength / (4.0 * st)
    if spacing > crit:
        warnings.warn(
            f"{op}: along-track trace spacing {spacing:.3f} m exceeds "
            f"lambda/(4 sin theta_max) = {crit:.3f} m for a {aperture_m:.0f} m "
            f"aperture at range {r_ref:.0f} m (half-angle "
            f"{np.degrees(theta):.1f} deg): coherent (point/specular) returns "
            "will alias in Doppler. Densify the track or shrink the aperture.")


def _window_code(window):
    if window not in WINDOWS:
        raise ValueError(f"unknown window {window!r} (use 'hann' or 'none')")
    return WINDOWS[window]


def focus_tensor(field, twtt, s, *, wavelength, aperture_m, window="hann",
                 c=C_DEFAULT, precision="fp64", out_dtype=torch.complex64,
                 power=True):
    """Backprojection of a device field (T, nb) complex64/complex128 with
    device float64 ``twtt`` (nb,) and arc length ``s`` (T,). Runs on the
    current stream; returns (focused field (T, nb) ``out_dtype``, power
    (T, nb) float32 or None)."""
    if field.dim() != 2:
        raise ValueError("focus needs a 2-D (slow_time, twtt) field")
    T, nb = field.shape
    if nb < 2:
        raise ValueError("focus needs at least two fast-time bins")
    if field.dtype not in (torch.complex64, torch.complex128):
        raise ValueError(f"field must be complex, got {field.dtype}")
    dev = field.device
    field = field.contiguous()
    twtt = twtt.to(dev, torch.float64).contiguous()
    s = s.to(dev, torch.float64).contiguous()
    opts = _lib.FocusOpts(float(wavelength), float(aperture_m), float(c), T,
                          nb, _window_code(window), _lib.PREC[precision],
                          int(field.dtype == torch.complex128))
    L = _lib.lib()
    nbytes = L.ss_focused_sar_scratch_bytes(C.byref(opts))
    scratch = torch.empty(max(nbytes, 1), dtype=torch.uint8, device=dev)
    out = torch.empty((T, nb), dtype=out_dtype, device=dev)
    pw = torch.empty((T, nb), dtype=torch.float32, device=dev) if power \
        else None
    o = _lib.FocusOutput(
        out.data_ptr() if out_dtype == torch.complex128 else None,
        out.data_ptr() if out_dtype == torch.complex64 else None,
        pw.data_ptr() if pw is not None else None)
    stream = torch.cuda.current_stream(dev).cuda_stream
    st = L.ss_focused_sar(C.byref(opts), C.c_void_p(field.data_ptr()),
                          C.c_void_p(twtt.data_ptr()),
                          C.c_void_p(s.data_ptr()), C.byref(o),
                          C.c_void_p(scratch.data_ptr()), nbytes,
                          C.c_void_p(stream))
    _lib.check(st, "ss_focused_sar")
    return out, pw


def focus_field(field, twtt, positions, *, wavelength, aperture_m,
                window="hann", c=C_DEFAULT, precision="fp64", device=None):
    """Focused field (complex64 (T, nb)) and power (float32) of a host field
    (processing.py:301-345 on arrays)."""
    _window_code(window)
    device = torch.device(device or "cuda")
    f = np.asarray(field)
    if f.ndim != 2:
        raise ValueError("focus needs a 2-D (slow_time, twtt) field")
    if f.dtype not in (np.complex64, np.complex128):
        f = f.astype(np.complex128)
    ft = torch.from_numpy(np.ascontiguousarray(f)).to(device)
    tw = torch.from_numpy(np.ascontiguousarray(twtt, np.float64)).to(device)
    st = torch.from_numpy(along_track(positions)).to(device)
    out, pw = focus_tensor(ft, tw, st, wavelength=wavelength,
                           aperture_m=aperture_m, window=window, c=c,
                           precision=precision)
    return out.cpu().numpy(), pw.cpu().numpy()


def _record(attrs, step):
    steps = json.loads(attrs.get("processing", "[]"))
    steps.append(step)
    attrs["processing"] = json.dumps(steps)
    return attrs


def _speed_of_light(ds):
    try:
        return float(json.loads(ds.attrs["config"])["radar"]["c"])
    except Exception:
        return C_DEFAULT


def focused_sar(ds, aperture_m, *, window="hann", precision="fp64",
                device=None):
    """Straight-track time-domain backprojection focusing through air
    (processing.py:262-348): same checks, warning, provenance record and
    returned Dataset (``field`` complex64, ``power`` float32)."""
    if ds.attrs.get("mode") != "coherent" or "field" not in ds:
        raise ValueError(
            "focused_sar() needs a coherent-mode Dataset with a complex "
            f"`field` (got mode={ds.attrs.get('mode')!r}). Coherent summation "
            "of power is not meaningful; for incoherent speckle reduction use "
            "multilook(ds, n) instead.")
    if set(ds.field.dims) != {"slow_time", "twtt"}:
        raise ValueError(
            "focused_sar needs a 2-D (slow_time, twtt) field; select a single "
            f"side/layer first (got dims {ds.field.dims})")
    if "wavelength" not in ds.attrs:
        raise ValueError("focused_sar needs the `wavelength` attr (coherent "
                         "run)")
    _window_code(window)
    c = _speed_of_light(ds)
    lam = float(ds.attrs["wavelength"])
    twtt = ds.twtt.values.astype(float)
    pos = np.column_stack([ds.x.values, ds.y.values,
                           ds.z.values]).astype(float)
    spacing = mean_spacing(pos)
    doppler_guard(spacing, lam, aperture_m, float((c * twtt / 2.0).min()),
                  "focused_sar")
    F = ds.field.transpose("slow_time", "twtt").values
    out, pw = focus_field(F, twtt, pos, wavelength=lam,
                          aperture_m=aperture_m, window=window, c=c,
                          precision=precision, device=device)
    T = F.shape[0]
    n_ap = int(np.round(aperture_m / spacing)) + 1 if spacing > 0 else T
    step = {"op": "focused_sar", "aperture_m": aperture_m, "window": window,
            "mean_spacing_m": spacing, "n_aperture_traces_approx": n_ap,
            "model": "straight-track time-domain backprojection through air "
                     "(surface-referenced); in-ice focusing out of scope"}
    attrs = _record(dict(ds.attrs), step)
    new = ds.copy()
    new.attrs.clear()
    new.attrs.update(attrs)
    new["field"] = (("slow_time", "twtt"), out, dict(ds.field.attrs))
    new["power"] = (("slow_time", "twtt"), pw, dict(ds.power.attrs))
    return new
