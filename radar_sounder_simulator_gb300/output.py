"""Output assembly on GB300: the per-trace products of soundersim
``output.py:47-146`` (``build_dataset``).

The facet scans -- nadir facet and ``nadir_twtt``, first in-window arrival
``first_return_twtt`` and its facet -- run in the CUDA library
(``ss_trace_products``) over every facet for every trace, with the
reference's float64 values and first-index tie rule; the reference builds
(T, N, 3) float64 arrays for them on the host. ``build_dataset`` mirrors the
reference's Dataset layout and needs xarray at call time (imported then);
``trace_products`` is the same work on plain arrays.
"""

import ctypes as C
import datetime
import json

import numpy as np
import torch

from . import _lib
from .coherent import to_host


def trace_products(centers, positions, *, t0, dt, n_samples, c,
                   device=None):
    """Nadir and first-return products of every trace (output.py:64-82).

    Returns a dict of NumPy arrays: ``nadir_index`` (int64), ``nadir_twtt``,
    ``first_index`` (int64; 0 when no facet is in the window) and
    ``first_twtt`` (+inf when none)."""
    device = torch.device(device or "cuda")
    cen = torch.from_numpy(np.ascontiguousarray(centers, np.float64)).to(
        device)
    pos = torch.from_numpy(np.ascontiguousarray(positions, np.float64)).to(
        device)
    T, N = pos.shape[0], cen.shape[0]
    L = _lib.lib()
    nbytes = L.ss_trace_products_scratch_bytes(T, N)
    if nbytes == 0:
        raise ValueError("trace products need at least one trace and one "
                         "facet")
    scratch = torch.empty(nbytes, dtype=torch.uint8, device=device)
    res = dict(nadir_index=torch.empty(T, dtype=torch.int64, device=device),
               nadir_twtt=torch.empty(T, dtype=torch.float64, device=device),
               first_index=torch.empty(T, dtype=torch.int64, device=device),
               first_twtt=torch.empty(T, dtype=torch.float64, device=device))
    o = _lib.TraceProductsOut(*[res[k].data_ptr() for k in (
        "nadir_index", "nadir_twtt", "first_index", "first_twtt")])
    opts = _lib.TraceProductsOpts(float(t0), float(dt), float(c),
                                  int(n_samples))
    st = L.ss_trace_products(C.byref(opts), C.c_void_p(cen.data_ptr()), N,
                             C.c_void_p(pos.data_ptr()), T, C.byref(o),
                             C.c_void_p(scratch.data_ptr()), nbytes,
                             C.c_void_p(torch.cuda.current_stream(
                                 device).cuda_stream))
    _lib.check(st, "ss_trace_products")
    return {k: to_host(v) for k, v in res.items()}


def build_dataset(power, dropped_power, *, scene, frame, facets, track,
                  sim_config, field=None, layers=None, nadir_twtt=None,
                  device=None):
    """The output Dataset of one run (output.py:47-146): same variables,
    coordinates and attrs, with the facet scans on the GPU."""
    import xarray as xr

    rc = sim_config.radar
    power = np.asarray(power, dtype=np.float32)
    n_traces, n_samples = power.shape[0], power.shape[1]
    pos = np.asarray(track.positions, np.float64)
    has_side = power.ndim == (4 if layers is not None else 3)
    prod = trace_products(facets.centers, pos, t0=rc.t0, dt=rc.dt,
                          n_samples=n_samples, c=rc.c, device=device)
    if nadir_twtt is None:
        nadir_twtt = prod["nadir_twtt"]
    nadir_dims = ("slow_time", "layer")[:np.ndim(nadir_twtt)]
    dropped_power = np.asarray(dropped_power, np.float32)
    dropped_dims = ("slow_time", "layer")[:dropped_power.ndim]
    fi = prod["first_index"]
    first_twtt = prod["first_twtt"]
    first_llh = frame.local_to_llh(np.asarray(facets.centers)[fi])
    dims = (("slow_time", "twtt") + (("side",) if has_side else ())
            + (("layer",) if layers is not None else ()))
    trace = np.arange(n_traces)
    ds = xr.Dataset(
        {
            "power": (dims, power,
                      {"units": "1", "long_name": "relative received power",
                       "comment": "relative linear power"}),
            "nadir_twtt": (nadir_dims, nadir_twtt,
                           {"units": "s", "long_name":
                            "two-way time to interface at nadir"}),
            "first_return_twtt": ("slow_time", first_twtt,
                                  {"units": "s",
                                   "long_name": "earliest in-window arrival"}),
            "first_return_lat": ("slow_time", first_llh[:, 0],
                                 {"units": "degrees_north"}),
            "first_return_lon": ("slow_time", first_llh[:, 1],
                                 {"units": "degrees_east"}),
            "dropped_power": (dropped_dims, dropped_power,
                              {"units": "1", "long_name":
                               "facet power outside the twtt window or on "
                               "invalid refracted paths"}),
        },
        coords={
            "slow_time": trace,
            "twtt": ("twtt", rc.t0 + np.arange(n_samples) * rc.dt,
                     {"units": "s",
                      "long_name": "two-way travel time (bin start)"}),
            "trace": ("slow_time", trace),
            "lat": ("slow_time", scene.nav_llh[:, 0],
                    {"units": "degrees_north"}),
            "lon": ("slow_time", scene.nav_llh[:, 1],
                    {"units": "degrees_east"}),
            "elevation": ("slow_time", scene.nav_llh[:, 2],
                          {"units": "m", "comment": "above WGS84 ellipsoid"}),
            "x": ("slow_time", pos[:, 0],
                  {"units": "m", "comment": "local scene frame"}),
            "y": ("slow_time", pos[:, 1],
                  {"units": "m", "comment": "local scene frame"}),
            "z": ("slow_time", pos[:, 2],
                  {"units": "m", "comment": "local scene frame"}),
        },
        attrs={
            "mode": sim_config.mode,
            "config": sim_config.model_dump_json(),
            "soundersim_version": "gb300:" + _lib.lib().ss_version().decode(),
            "git_commit": None,
            "created": datetime.datetime.now(
                datetime.timezone.utc).isoformat(),
            "dem_source": f"synthetic:{scene.name}",
            "dem_crs": str(scene.crs),
            "scene_params": json.dumps(scene.params),
            "scene_frame": json.dumps(
                {"origin_lat": frame.lat0, "origin_lon": frame.lon0,
                 "origin_h": frame.h0, "orientation": "ENU"}),
        },
    )
    wf = rc.waveform
    ds.attrs["waveform"] = wf.kind
    if wf.kind == "chirp":
        ds.attrs["bandwidth"] = wf.bandwidth
        ds.attrs["pulse_length"] = wf.pulse_length
        ds.attrs["waveform_window"] = wf.window
    if field is not None:
        ds["field"] = (dims, np.asarray(field, dtype=np.complex64),
                       {"units": "1", "long_name": "relative received field",
                        "comment": "complex field at the carrier; "
                                   "power = |field|^2"})
        ds.attrs["frequency"] = rc.f0
        ds.attrs["wavelength"] = rc.wavelength
    if has_side:
        ds = ds.assign_coords(side=("side", np.array(["left", "right"])))
    if layers is not None:
        ds = ds.assign_coords(layer=("layer", np.array(layers)))
    return ds
