"""Scene assembly on GB300: DEM window -> facets, keyed speckle phasors and
offset interfaces, with the per-vertex and per-facet work on the device.

Mirrors soundersim ``scene.py:126-176`` (``build_facets``),
``roughness.py:207-233`` (``speckle_phasors_for_keys``) and
``layered.py:38-53`` (``offset_facets``). The lattice of a DEM crop
(``_lattice_axis``) is a few hundred numbers per axis and stays on the host;
bilinear resampling, the affine pixel -> projected map, the projected ->
geodetic -> ECEF -> local chain and the corner rule run in the CUDA library
(``ss_scene_vertices``, ``ss_facets_from_vertices``). The reference takes
the CRS step from pyproj; here the projections the reference's synthetic
scenes and the ice-sheet DEMs use are built in: ``"EPSG:3413"`` and
``"EPSG:3031"`` (WGS84 polar stereographic), and ``None`` for coordinates
that already are ECEF (any other CRS raises ``ValueError``).

``LocalFrame`` is the reference's ENU frame with the WGS84 conversions
written out (no pyproj); ``frame`` arguments accept it or any object with
``origin_ecef`` and ``R``.
"""

import ctypes as C
from dataclasses import dataclass

import numpy as np
import torch

from . import _lib
from .coherent import to_host

WGS84_A = 6378137.0
WGS84_F = 1.0 / 298.257223563
WGS84_E2 = WGS84_F * (2.0 - WGS84_F)


@dataclass
class Facets:
    """The reference's Facets fields (scene.py:85-101); arrays are NumPy,
    or device tensors when built with ``as_tensors=True``."""

    centers: object
    normals: object
    areas: object
    e1: object
    e2: object
    cell: object
    grid_shape: tuple
    phase_keys: object = None

    def index_map(self):
        n = self.grid_shape[0] * self.grid_shape[1]
        return np.arange(n).reshape(self.grid_shape)


class LocalFrame:
    """East-North-Up frame anchored at (lat0, lon0, h0) on WGS84
    (scene.py:24-82): R's rows are E, N, U in ECEF."""

    def __init__(self, lat0, lon0, h0=0.0):
        self.lat0, self.lon0, self.h0 = float(lat0), float(lon0), float(h0)
        self.origin_ecef = np.array(geodetic_to_ecef(lat0, lon0, h0))
        lat, lon = np.deg2rad(self.lat0), np.deg2rad(self.lon0)
        sl, cl, so, co = np.sin(lat), np.cos(lat), np.sin(lon), np.cos(lon)
        self.R = np.array([[-so, co, 0.0], [-sl * co, -sl * so, cl],
                           [cl * co, cl * so, sl]], dtype=np.float64)

    def ecef_to_local(self, xyz):
        return (np.atleast_2d(np.asarray(xyz, np.float64)) -
                self.origin_ecef) @ self.R.T

    def local_to_ecef(self, enu):
        return np.atleast_2d(np.asarray(enu, np.float64)) @ self.R + \
            self.origin_ecef


def geodetic_to_ecef(lat_deg, lon_deg, h):
    lat, lon = np.radians(lat_deg), np.radians(lon_deg)
    sl = np.sin(lat)
    n = WGS84_A / np.sqrt(1.0 - WGS84_E2 * sl * sl)
    return ((n + h) * np.cos(lat) * np.cos(lon),
            (n + h) * np.cos(lat) * np.sin(lon),
            (n * (1.0 - WGS84_E2) + h) * sl)


def _frame_struct(frame):
    fr = _lib.Frame()
    fr.origin[:] = [float(v) for v in np.asarray(frame.origin_ecef).ravel()]
    fr.R[:] = [float(v) for v in np.asarray(frame.R, np.float64).ravel()]
    return fr


def _stream(device):
    return C.c_void_p(torch.cuda.current_stream(device).cuda_stream)


def lattice_axis(n, step, origin):
    """Crop-local sample coordinates and their parent-lattice keys
    (scene.py:115-123)."""
    eps = 1e-10
    first = int(np.ceil((origin - eps) / step))
    last = int(np.floor((origin + n - 1 + eps) / step))
    keys = np.arange(first, last + 1, dtype=np.int64)
    if len(keys) < 2:
        raise ValueError("DEM crop is too small for the requested facet "
                         "spacing")
    return keys.astype(np.float64) * step - origin, keys


def _transform6(transform):
    if hasattr(transform, "a"):
        return tuple(float(getattr(transform, k)) for k in "abcdef")
    t = tuple(float(v) for v in transform)
    if len(t) < 6:
        raise ValueError("transform needs six coefficients (a, b, c, d, e, f)")
    return t[:6]


def build_facets(dem, transform, crs, frame, spacing=None, grid_origin=(0, 0),
                 *, device=None, as_tensors=False):
    """Tessellate a projected DEM window into upward-oriented mean-plane
    facets in ``frame`` (scene.py:126-176). ``transform``: an affine
    transform (attributes a..f) or the six coefficients."""
    if crs not in _lib.PROJ:
        raise ValueError(f"unsupported CRS {crs!r} (supported: EPSG:3413, "
                         "EPSG:3031, or None for ECEF coordinates)")
    device = torch.device(device or "cuda")
    t6 = _transform6(transform)
    dem = np.asarray(dem, dtype=np.float64)
    ny, nx = dem.shape
    px = 0.5 * (abs(t6[0]) + abs(t6[4]))
    if spacing is None or abs(spacing - px) < 1e-9:
        step = 1.0
    elif spacing > px:
        step = float(max(1, int(round(spacing / px))))
    else:
        step = float(spacing / px)
    orow, ocol = map(float, grid_origin)
    rows, row_keys = lattice_axis(ny, step, orow)
    cols, col_keys = lattice_axis(nx, step, ocol)
    H, W = len(rows), len(cols)

    def up(a):
        return torch.from_numpy(np.ascontiguousarray(a)).to(device)
    dem_t, rows_t, cols_t = up(dem), up(rows), up(cols)
    rk_t, ck_t = up(row_keys), up(col_keys)
    V = torch.empty((H, W, 3), dtype=torch.float64, device=device)
    g = _lib.DemGrid(dem_t.data_ptr(), ny, nx, rows_t.data_ptr(),
                     cols_t.data_ptr(), H, W)
    g.transform[:] = list(t6)
    g.projection = _lib.PROJ[crs]
    g.frame = _frame_struct(frame)
    L = _lib.lib()
    _lib.check(L.ss_scene_vertices(C.byref(g), C.c_void_p(V.data_ptr()),
                                   _stream(device)), "ss_scene_vertices")
    n = (H - 1) * (W - 1)
    f64 = dict(dtype=torch.float64, device=device)
    out = dict(centers=torch.empty((n, 3), **f64),
               normals=torch.empty((n, 3), **f64),
               areas=torch.empty(n, **f64), e1=torch.empty((n, 3), **f64),
               e2=torch.empty((n, 3), **f64),
               cell=torch.empty((n, 2), dtype=torch.int64, device=device),
               phase_keys=torch.empty((n, 2), dtype=torch.int64,
                                      device=device))
    fo = _lib.FacetOut(*[out[k].data_ptr() for k in (
        "centers", "normals", "areas", "e1", "e2", "cell", "phase_keys")])
    _lib.check(L.ss_facets_from_vertices(
        C.c_void_p(V.data_ptr()), H, W, C.c_void_p(rk_t.data_ptr()),
        C.c_void_p(ck_t.data_ptr()), C.byref(fo), _stream(device)),
        "ss_facets_from_vertices")
    if not as_tensors:
        out = {k: to_host(v) for k, v in out.items()}
    return Facets(out["centers"], out["normals"], out["areas"], out["e1"],
                  out["e2"], out["cell"], (H - 1, W - 1), out["phase_keys"])


def seed_base(seed):
    """The 64-bit word the reference derives from a seed
    (roughness.py:212: SeedSequence state)."""
    return int(np.random.SeedSequence(seed).generate_state(
        1, dtype=np.uint64)[0])


def speckle_phasors_tensor(keys, seed):
    """Keyed phasors of a device (n, 2) int64 key tensor, as a device
    complex64 tensor (n,)."""
    if keys.dim() != 2 or keys.shape[1] != 2:
        raise ValueError("speckle keys must have shape (n, 2)")
    keys = keys.to(torch.int64).contiguous()
    n = keys.shape[0]
    out = torch.empty(n, dtype=torch.complex64, device=keys.device)
    _lib.check(_lib.lib().ss_speckle_phasors_keyed(
        C.c_void_p(keys.data_ptr()), n, seed_base(seed),
        C.c_void_p(out.data_ptr()), _stream(keys.device)),
        "ss_speckle_phasors_keyed")
    return out


def speckle_phasors_for_keys(keys, seed, *, device=None):
    """Stateless Gaussian phasors keyed by parent-grid cells
    (roughness.py:207-233): complex64 (n,) NumPy array."""
    keys = np.asarray(keys, dtype=np.int64)
    if keys.ndim != 2 or keys.shape[1] != 2:
        raise ValueError("speckle keys must have shape (n, 2)")
    device = torch.device(device or "cuda")
    return to_host(speckle_phasors_tensor(
        torch.from_numpy(np.ascontiguousarray(keys)).to(device), seed))


def offset_facets(facets, frame, offset, *, device=None):
    """Facets with centres moved ``offset`` metres along local ellipsoidal
    up (layered.py:38-53); normals, areas, edges and cells are copies."""
    device = torch.device(device or "cuda")
    cen = np.ascontiguousarray(facets.centers, np.float64)
    c_t = torch.from_numpy(cen).to(device)
    out = torch.empty_like(c_t)
    fr = _frame_struct(frame)
    _lib.check(_lib.lib().ss_offset_centers(
        C.c_void_p(c_t.data_ptr()), len(cen), C.byref(fr), float(offset),
        C.c_void_p(out.data_ptr()), _stream(device)), "ss_offset_centers")
    keys = facets.phase_keys
    return Facets(to_host(out), np.array(facets.normals, copy=True),
                  np.array(facets.areas, copy=True),
                  np.array(facets.e1, copy=True),
                  np.array(facets.e2, copy=True),
                  np.array(facets.cell, copy=True), facets.grid_shape,
                  None if keys is None else np.array(keys, copy=True))
