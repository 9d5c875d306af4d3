"""Scene assembly in float64 NumPy (oracle).

Test infrastructure only: the GPU path never imports this module.

Restates soundersim ``scene.py`` and ``roughness.py`` pieces that turn a
projected DEM window into facets and per-facet random fields:

* ``speckle_phasors_for_keys`` (roughness.py:207-233): stateless Gaussian
  phasors from a 64-bit mixing hash of parent-grid keys (Box-Muller);
* ``lattice_axis`` / ``bilinear`` (scene.py:104-124): crop-local sample
  positions on the parent lattice and bilinear DEM sampling;
* ``facets_from_vertices`` (scene.py:158-176): the mean-plane corner rule,
  cells and phase keys;
* ``build_facets`` (scene.py:126-176) with the projected -> ECEF step given
  as a callable (the reference takes it from pyproj);
* WGS84 geodetic <-> ECEF, the ellipsoidal polar stereographic projection
  (EPSG:3413 north, EPSG:3031 south; Snyder 1987, "Map Projections -- A
  Working Manual", USGS PP 1395, section 21), the ENU ``LocalFrame``
  (scene.py:24-82) and ``offset_facets`` (layered.py:38-53).

Parity: the hash, lattice, bilinear sampling and corner rule are pinned to
the reference's own outputs (tests/golden/scene.npz, made through a pyproj
stand-in whose transform is the identity). The geodetic and projection
formulas have no reference run here (pyproj is absent): they are checked
by round trips and closed-form properties only.
"""

import numpy as np

WGS84_A = 6378137.0
WGS84_F = 1.0 / 298.257223563
WGS84_E2 = WGS84_F * (2.0 - WGS84_F)

_GOLDEN = np.uint64(0x9E3779B97F4A7C15)
_M1 = np.uint64(0xBF58476D1CE4E5B9)
_M2 = np.uint64(0x94D049BB133111EB)
_KEY_MUL = np.uint64(0xD2B74407B1CE6E93)
_SALT = np.uint64(0xCA5A826395121157)


def _mix(x):
    """64-bit finaliser (roughness.py:214-219)."""
    with np.errstate(over="ignore"):
        x = x + _GOLDEN
        x = (x ^ (x >> np.uint64(30))) * _M1
        x = (x ^ (x >> np.uint64(27))) * _M2
    return x ^ (x >> np.uint64(31))


def seed_base(seed):
    """The 64-bit base word of a seed (roughness.py:212)."""
    return np.random.SeedSequence(seed).generate_state(1, dtype=np.uint64)[0]


def speckle_phasors_for_keys(keys, seed):
    keys = np.asarray(keys, np.int64)
    if keys.ndim != 2 or keys.shape[1] != 2:
        raise ValueError("speckle keys must have shape (n, 2)")
    base = seed_base(seed)
    with np.errstate(over="ignore"):
        keyed = (base ^ keys[:, 0].astype(np.uint64)
                 ^ (keys[:, 1].astype(np.uint64) * _KEY_MUL))
    h1 = _mix(keyed)
    h2 = _mix(keyed ^ _SALT)
    scale = 1.0 / (1 << 53)
    u1 = ((h1 >> np.uint64(11)).astype(np.float64) + 0.5) * scale
    u2 = ((h2 >> np.uint64(11)).astype(np.float64) + 0.5) * scale
    radius = np.sqrt(-2.0 * np.log(u1))
    angle = 2.0 * np.pi * u2
    ph = radius * (np.cos(angle) + 1j * np.sin(angle)) / np.sqrt(2.0)
    return ph.astype(np.complex64)


def lattice_axis(n, step, origin):
    """Crop-local sample coordinates and parent-lattice keys
    (scene.py:115-123)."""
    eps = 1e-10
    first = int(np.ceil((origin - eps) / step))
    last = int(np.floor((origin + n - 1 + eps) / step))
    keys = np.arange(first, last + 1, dtype=np.int64)
    if len(keys) < 2:
        raise ValueError("DEM crop is too small for the requested facet "
                         "spacing")
    return keys.astype(np.float64) * step - origin, keys


def facet_step(transform_a, transform_e, spacing):
    """Sampling step in DEM pixels (scene.py:142-148)."""
    px = 0.5 * (abs(transform_a) + abs(transform_e))
    if spacing is None or abs(spacing - px) < 1e-9:
        return 1.0
    if spacing > px:
        return float(max(1, int(round(spacing / px))))
    return float(spacing / px)


def bilinear(dem, rows, cols):
    """scene.py:104-112."""
    r0 = np.clip(np.floor(rows).astype(int), 0, dem.shape[0] - 2)
    c0 = np.clip(np.floor(cols).astype(int), 0, dem.shape[1] - 2)
    fr, fc = (rows - r0)[:, None], (cols - c0)[None, :]
    d00, d01 = dem[np.ix_(r0, c0)], dem[np.ix_(r0, c0 + 1)]
    d10, d11 = dem[np.ix_(r0 + 1, c0)], dem[np.ix_(r0 + 1, c0 + 1)]
    return (d00 * (1 - fr) * (1 - fc) + d01 * (1 - fr) * fc
            + d10 * fr * (1 - fc) + d11 * fr * fc)


def affine_apply(t, x, y):
    """(a x + b y + c, d x + e y + f) for t = (a, b, c, d, e, f)."""
    a, b, c, d, e, f = t
    return x * a + y * b + c, x * d + y * e + f


def facets_from_vertices(V, row_keys=None, col_keys=None):
    """Corner rule (scene.py:158-176): V (H, W, 3) vertices -> centers,
    normals, areas, e1, e2, cell, grid_shape, phase_keys."""
    v00, v01 = V[:-1, :-1], V[:-1, 1:]
    v10, v11 = V[1:, :-1], V[1:, 1:]
    e1 = ((v01 + v11) - (v00 + v10)) / 2.0
    e2 = ((v10 + v11) - (v00 + v01)) / 2.0
    centers = ((v00 + v01 + v10 + v11) / 4.0).reshape(-1, 3)
    raw = np.cross(e1, e2).reshape(-1, 3)
    mag = np.linalg.norm(raw, axis=1)
    normals = raw / mag[:, None]
    normals *= np.where(normals[:, 2] < 0.0, -1.0, 1.0)[:, None]
    hc, wc = V.shape[0] - 1, V.shape[1] - 1
    ci, cj = np.meshgrid(np.arange(hc), np.arange(wc), indexing="ij")
    cell = np.stack([ci.ravel(), cj.ravel()], axis=1)
    keys = None
    if row_keys is not None:
        ki, kj = np.meshgrid(row_keys[:-1], col_keys[:-1], indexing="ij")
        keys = np.stack([ki.ravel(), kj.ravel()], axis=1)
    return dict(centers=centers, normals=normals, areas=mag,
                e1=e1.reshape(-1, 3), e2=e2.reshape(-1, 3), cell=cell,
                grid_shape=(hc, wc), phase_keys=keys)


def build_facets(dem, transform, to_ecef, ecef_to_local, spacing=None,
                 grid_origin=(0, 0)):
    """scene.py:126-176 with the CRS step as ``to_ecef(E, N, h)`` and the
    frame as ``ecef_to_local(xyz)``; ``transform`` = (a, b, c, d, e, f)."""
    dem = np.asarray(dem, np.float64)
    ny, nx = dem.shape
    step = facet_step(transform[0], transform[4], spacing)
    orow, ocol = map(float, grid_origin)
    rows, row_keys = lattice_axis(ny, step, orow)
    cols, col_keys = lattice_axis(nx, step, ocol)
    dem = bilinear(dem, rows, cols)
    J, I = np.meshgrid(cols + 0.5, rows + 0.5)
    E, N = affine_apply(transform, J, I)
    ecef = np.column_stack(to_ecef(E.ravel(), N.ravel(), dem.ravel()))
    V = ecef_to_local(ecef).reshape(*dem.shape, 3)
    return facets_from_vertices(V, row_keys, col_keys)


# ---------------------------------------------------------------- WGS84

def geodetic_to_ecef(lat_deg, lon_deg, h):
    lat, lon = np.radians(lat_deg), np.radians(lon_deg)
    sl = np.sin(lat)
    n = WGS84_A / np.sqrt(1.0 - WGS84_E2 * sl * sl)
    return ((n + h) * np.cos(lat) * np.cos(lon),
            (n + h) * np.cos(lat) * np.sin(lon),
            (n * (1.0 - WGS84_E2) + h) * sl)


def ecef_to_geodetic(x, y, z, iters=6):
    """Latitude by fixed-point iteration on tan(lat) (converges to 1e-15
    rad in a few steps away from the geocentre); degrees, degrees, metres."""
    p = np.hypot(x, y)
    lat = np.arctan2(z, p * (1.0 - WGS84_E2))
    for _ in range(iters):
        sl = np.sin(lat)
        n = WGS84_A / np.sqrt(1.0 - WGS84_E2 * sl * sl)
        lat = np.arctan2(z + WGS84_E2 * n * sl, p)
    sl = np.sin(lat)
    n = WGS84_A / np.sqrt(1.0 - WGS84_E2 * sl * sl)
    cl = np.cos(lat)
    h = np.where(np.abs(cl) > 1e-10, p / np.where(cl == 0, 1, cl) - n,
                 np.abs(z) - n * (1.0 - WGS84_E2))
    return np.degrees(lat), np.degrees(np.arctan2(y, x)), h


class LocalFrame:
    """ENU frame at (lat0, lon0, h0) on WGS84 (scene.py:24-82)."""

    def __init__(self, lat0, lon0, h0=0.0):
        self.lat0, self.lon0, self.h0 = float(lat0), float(lon0), float(h0)
        self.origin_ecef = np.array(geodetic_to_ecef(lat0, lon0, h0))
        lat, lon = np.radians(lat0), np.radians(lon0)
        sl, cl, so, co = np.sin(lat), np.cos(lat), np.sin(lon), np.cos(lon)
        self.R = np.array([[-so, co, 0.0], [-sl * co, -sl * so, cl],
                           [cl * co, cl * so, sl]])

    def ecef_to_local(self, xyz):
        return (np.atleast_2d(xyz) - self.origin_ecef) @ self.R.T

    def local_to_ecef(self, enu):
        return np.atleast_2d(enu) @ self.R + self.origin_ecef

    def up_at(self, enu):
        x = self.local_to_ecef(enu)
        lat, lon, _ = ecef_to_geodetic(x[:, 0], x[:, 1], x[:, 2])
        lat, lon = np.radians(lat), np.radians(lon)
        up = np.column_stack([np.cos(lat) * np.cos(lon),
                              np.cos(lat) * np.sin(lon), np.sin(lat)])
        return up @ self.R.T


def offset_centers(centers, frame, offset):
    """layered.py:38-53: centres moved ``offset`` metres along local
    ellipsoidal up."""
    up = frame.up_at(centers)
    up = up / np.linalg.norm(up, axis=1, keepdims=True)
    return centers + offset * up


# ------------------------------------------------- polar stereographic

POLAR = {"EPSG:3413": (70.0, -45.0, 1.0), "EPSG:3031": (-71.0, 0.0, -1.0)}


def _tfun(phi, e):
    es = e * np.sin(phi)
    return np.tan(np.pi / 4 - phi / 2) / ((1 - es) / (1 + es)) ** (e / 2)


def polar_stereo_inverse(x, y, crs):
    """(lon, lat) degrees of projected (x, y) metres (Snyder 1987, eqs.
    21-33 to 21-41, ellipsoid, standard parallel, no false origin)."""
    lat_c, lon0, sgn = POLAR[crs]
    e = np.sqrt(WGS84_E2)
    x, y = sgn * np.asarray(x, np.float64), sgn * np.asarray(y, np.float64)
    pc = np.radians(sgn * lat_c)
    mc = np.cos(pc) / np.sqrt(1 - WGS84_E2 * np.sin(pc) ** 2)
    tc = _tfun(pc, e)
    rho = np.hypot(x, y)
    t = rho * tc / (WGS84_A * mc)
    phi = np.pi / 2 - 2 * np.arctan(t)
    for _ in range(8):
        es = e * np.sin(phi)
        phi = np.pi / 2 - 2 * np.arctan(t * ((1 - es) / (1 + es)) ** (e / 2))
    lam = np.radians(sgn * lon0) + np.arctan2(x, -y)
    lon = np.degrees(lam) * sgn
    lon = (lon + 180.0) % 360.0 - 180.0
    return lon, sgn * np.degrees(phi)


def polar_stereo_forward(lon, lat, crs):
    lat_c, lon0, sgn = POLAR[crs]
    e = np.sqrt(WGS84_E2)
    phi = np.radians(sgn * np.asarray(lat, np.float64))
    lam = np.radians(sgn * np.asarray(lon, np.float64))
    pc = np.radians(sgn * lat_c)
    mc = np.cos(pc) / np.sqrt(1 - WGS84_E2 * np.sin(pc) ** 2)
    rho = WGS84_A * mc * _tfun(phi, e) / _tfun(pc, e)
    dl = lam - np.radians(sgn * lon0)
    return sgn * rho * np.sin(dl), -sgn * rho * np.cos(dl)
