// Scene assembly on the device: DEM window -> local-frame vertices ->
// mean-plane facets, keyed speckle phasors, and vertical offsets of an
// interface.
//
// Replaces the host NumPy/pyproj work of soundersim scene.py:104-176
// (`_bilinear`, `build_facets`), roughness.py:207-233
// (`speckle_phasors_for_keys`) and layered.py:38-53 (`offset_facets`).
// Everything is float64. The lattice positions come from the host (a few
// hundred numbers per axis); every per-vertex and per-facet operation runs
// here, one thread per vertex / facet / key, written with round-to-nearest
// intrinsics in the reference's operation order where the reference's
// result is a plain arithmetic chain (bilinear weights, affine map, corner
// rule, hash), so those outputs are bit-identical to it.
#include <algorithm>

#include "ss_internal.cuh"

namespace ss {

__device__ __forceinline__ double dm(double a, double b) {
  return __dmul_rn(a, b);
}
__device__ __forceinline__ double da(double a, double b) {
  return __dadd_rn(a, b);
}
__device__ __forceinline__ double ds(double a, double b) {
  return __dsub_rn(a, b);
}

// ------------------------------------------------------------ WGS84 ----
constexpr double kA = 6378137.0;
constexpr double kF = 1.0 / 298.257223563;
constexpr double kE2 = kF * (2.0 - kF);

__device__ void geodetic_to_ecef(double lat, double lon, double h,
                                 double &x, double &y, double &z) {
  double sl, cl, so, co;
  sincos(lat, &sl, &cl);
  sincos(lon, &so, &co);
  const double n = kA / sqrt(1.0 - kE2 * sl * sl);
  x = (n + h) * cl * co;
  y = (n + h) * cl * so;
  z = (n * (1.0 - kE2) + h) * sl;
}

// Latitude of an ECEF point by fixed-point iteration on tan(lat)
// (converges to ~1e-15 rad in a few steps away from the geocentre).
__device__ double ecef_latitude(double x, double y, double z) {
  const double p = hypot(x, y);
  double lat = atan2(z, p * (1.0 - kE2));
  for (int it = 0; it < 6; ++it) {
    const double sl = sin(lat);
    const double n = kA / sqrt(1.0 - kE2 * sl * sl);
    lat = atan2(z + kE2 * n * sl, p);
  }
  return lat;
}

// Ellipsoidal polar stereographic inverse (Snyder 1987, USGS PP 1395,
// eqs. 21-33..21-41): the south aspect negates x, y, lat, lon, lat_c,
// lon_0 around the north formulas. Returns radians.
__device__ void polar_inverse(double x, double y, double lat_c_deg,
                              double lon0_deg, double sgn, double &lat,
                              double &lon) {
  const double e = sqrt(kE2);
  x *= sgn;
  y *= sgn;
  const double pc = sgn * lat_c_deg * (kPi / 180.0);
  const double spc = sin(pc);
  const double mc = cos(pc) / sqrt(1.0 - kE2 * spc * spc);
  const double tc = tan(kPi / 4 - pc / 2) /
                    pow((1.0 - e * spc) / (1.0 + e * spc), e / 2);
  const double rho = hypot(x, y);
  const double t = rho * tc / (kA * mc);
  double phi = kPi / 2 - 2.0 * atan(t);
  for (int it = 0; it < 8; ++it) {
    const double es = e * sin(phi);
    phi = kPi / 2 - 2.0 * atan(t * pow((1.0 - es) / (1.0 + es), e / 2));
  }
  lat = sgn * phi;
  lon = sgn * (sgn * lon0_deg * (kPi / 180.0) + atan2(x, -y));
}

// ----------------------------------------------------- vertices -------
__global__ void scene_vertices_kernel(ss_dem_grid g, double *V) {
  const long n = (long)g.n_rows * g.n_cols;
  for (long v = blockIdx.x * (long)blockDim.x + threadIdx.x; v < n;
       v += (long)gridDim.x * blockDim.x) {
    const int i = (int)(v / g.n_cols), j = (int)(v % g.n_cols);
    const double rows = g.rows[i], cols = g.cols[j];
    // bilinear sample (scene.py:104-112), the reference's operation order
    const int r0 = min(max((int)floor(rows), 0), g.ny - 2);
    const int c0 = min(max((int)floor(cols), 0), g.nx - 2);
    const double fr = ds(rows, (double)r0), fc = ds(cols, (double)c0);
    const double *d = g.dem;
    const double d00 = d[(long)r0 * g.nx + c0];
    const double d01 = d[(long)r0 * g.nx + c0 + 1];
    const double d10 = d[(long)(r0 + 1) * g.nx + c0];
    const double d11 = d[(long)(r0 + 1) * g.nx + c0 + 1];
    const double ofr = ds(1.0, fr), ofc = ds(1.0, fc);
    const double h = da(da(da(dm(dm(d00, ofr), ofc), dm(dm(d01, ofr), fc)),
                          dm(dm(d10, fr), ofc)),
                       dm(dm(d11, fr), fc));
    // pixel centre -> projected (x a + y b + c, x d + y e + f)
    const double J = da(cols, 0.5), I = da(rows, 0.5);
    const double *t = g.transform;
    const double E = da(da(dm(J, t[0]), dm(I, t[1])), t[2]);
    const double N = da(da(dm(J, t[3]), dm(I, t[4])), t[5]);
    double x = E, y = N, z = h;
    if (g.projection == SS_PROJ_POLAR_NORTH ||
        g.projection == SS_PROJ_POLAR_SOUTH) {
      double lat, lon;
      if (g.projection == SS_PROJ_POLAR_NORTH)
        polar_inverse(E, N, 70.0, -45.0, 1.0, lat, lon);    // EPSG:3413
      else
        polar_inverse(E, N, -71.0, 0.0, -1.0, lat, lon);    // EPSG:3031
      geodetic_to_ecef(lat, lon, h, x, y, z);
    }
    // ECEF -> local: R (rows E, N, U) applied to (xyz - origin)
    const double *o = g.frame.origin, *R = g.frame.R;
    const double qx = ds(x, o[0]), qy = ds(y, o[1]), qz = ds(z, o[2]);
    double *out = V + 3 * v;
    for (int r = 0; r < 3; ++r)
      out[r] = da(da(dm(qx, R[3 * r]), dm(qy, R[3 * r + 1])),
                  dm(qz, R[3 * r + 2]));
  }
}

// ------------------------------------------------------ corner rule ---
__global__ void facets_from_vertices_kernel(const double *V, int H, int W,
                                            const int64_t *row_keys,
                                            const int64_t *col_keys,
                                            ss_facet_out o) {
  const int hc = H - 1, wc = W - 1;
  const long n = (long)hc * wc;
  for (long f = blockIdx.x * (long)blockDim.x + threadIdx.x; f < n;
       f += (long)gridDim.x * blockDim.x) {
    const int i = (int)(f / wc), j = (int)(f % wc);
    const double *v00 = V + 3 * ((long)i * W + j);
    const double *v01 = v00 + 3;
    const double *v10 = V + 3 * ((long)(i + 1) * W + j);
    const double *v11 = v10 + 3;
    double e1[3], e2[3];
    for (int k = 0; k < 3; ++k) {
      e1[k] = ds(da(v01[k], v11[k]), da(v00[k], v10[k])) * 0.5;
      e2[k] = ds(da(v10[k], v11[k]), da(v00[k], v01[k])) * 0.5;
      if (o.centers)
        o.centers[3 * f + k] =
            da(da(da(v00[k], v01[k]), v10[k]), v11[k]) * 0.25;
      if (o.e1) o.e1[3 * f + k] = e1[k];
      if (o.e2) o.e2[3 * f + k] = e2[k];
    }
    // np.cross, then |.| and the upward orientation (scene.py:167-171)
    const double rx = ds(dm(e1[1], e2[2]), dm(e1[2], e2[1]));
    const double ry = ds(dm(e1[2], e2[0]), dm(e1[0], e2[2]));
    const double rz = ds(dm(e1[0], e2[1]), dm(e1[1], e2[0]));
    const double mag = __dsqrt_rn(da(da(dm(rx, rx), dm(ry, ry)), dm(rz, rz)));
    double nx = __ddiv_rn(rx, mag), ny = __ddiv_rn(ry, mag),
           nz = __ddiv_rn(rz, mag);
    if (nz < 0.0) {
      nx = -nx;
      ny = -ny;
      nz = -nz;
    }
    if (o.normals) {
      o.normals[3 * f] = nx;
      o.normals[3 * f + 1] = ny;
      o.normals[3 * f + 2] = nz;
    }
    if (o.areas) o.areas[f] = mag;
    if (o.cell) {
      o.cell[2 * f] = i;
      o.cell[2 * f + 1] = j;
    }
    if (o.phase_keys && row_keys && col_keys) {
      o.phase_keys[2 * f] = row_keys[i];
      o.phase_keys[2 * f + 1] = col_keys[j];
    }
  }
}

// ------------------------------------------------- keyed phasors ------
__device__ __forceinline__ uint64_t mix64(uint64_t x) {
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}

__global__ void speckle_keyed_kernel(const int64_t *keys, long n,
                                     uint64_t base, float2 *out) {
  for (long q = blockIdx.x * (long)blockDim.x + threadIdx.x; q < n;
       q += (long)gridDim.x * blockDim.x) {
    const uint64_t keyed = base ^ (uint64_t)keys[2 * q] ^
                           ((uint64_t)keys[2 * q + 1] * 0xD2B74407B1CE6E93ull);
    const uint64_t h1 = mix64(keyed);
    const uint64_t h2 = mix64(keyed ^ 0xCA5A826395121157ull);
    const double scale = 1.0 / 9007199254740992.0;  // 2^-53
    const double u1 = dm(da((double)(h1 >> 11), 0.5), scale);
    const double u2 = dm(da((double)(h2 >> 11), 0.5), scale);
    // Box-Muller (roughness.py:230-233)
    const double radius = __dsqrt_rn(dm(-2.0, log(u1)));
    double sn, cs;
    sincos(dm(2.0 * kPi, u2), &sn, &cs);
    // NumPy divides a complex by the real sqrt(2) as a multiplication by
    // the rounded reciprocal 1/sqrt(2)
    const double inv_r2 = __drcp_rn(1.4142135623730951);
    out[q] = make_float2((float)dm(dm(radius, cs), inv_r2),
                         (float)dm(dm(radius, sn), inv_r2));
  }
}

// ------------------------------------------------------ offsets -------
__global__ void offset_centers_kernel(const double *c, long n, ss_frame fr,
                                      double offset, double *out) {
  const double *o = fr.origin, *R = fr.R;
  for (long f = blockIdx.x * (long)blockDim.x + threadIdx.x; f < n;
       f += (long)gridDim.x * blockDim.x) {
    const double e = c[3 * f], nn = c[3 * f + 1], u = c[3 * f + 2];
    // local -> ECEF: enu @ R + origin
    const double x = e * R[0] + nn * R[3] + u * R[6] + o[0];
    const double y = e * R[1] + nn * R[4] + u * R[7] + o[1];
    const double z = e * R[2] + nn * R[5] + u * R[8] + o[2];
    const double lat = ecef_latitude(x, y, z);
    const double lon = atan2(y, x);
    double sl, cl, so, co;
    sincos(lat, &sl, &cl);
    sincos(lon, &so, &co);
    const double ux = cl * co, uy = cl * so, uz = sl;
    double up[3];
    for (int r = 0; r < 3; ++r)
      up[r] = ux * R[3 * r] + uy * R[3 * r + 1] + uz * R[3 * r + 2];
    const double m = sqrt(up[0] * up[0] + up[1] * up[1] + up[2] * up[2]);
    for (int r = 0; r < 3; ++r) out[3 * f + r] = c[3 * f + r] + offset * up[r] / m;
  }
}

static int grid_for(long n) {
  return (int)std::min<long>((n + 255) / 256, 64L * sm_count());
}

}  // namespace ss

using namespace ss;

extern "C" int ss_scene_vertices(const ss_dem_grid *g, double *V,
                                 void *stream) {
  if (!g || !V || !g->dem || !g->rows || !g->cols || g->ny < 2 ||
      g->nx < 2 || g->n_rows < 1 || g->n_cols < 1 ||
      g->projection < SS_PROJ_IDENTITY || g->projection > SS_PROJ_POLAR_SOUTH) {
    set_error("ss_scene_vertices: bad argument");
    return SS_ERR_ARG;
  }
  const long n = (long)g->n_rows * g->n_cols;
  scene_vertices_kernel<<<grid_for(n), 256, 0,
                          reinterpret_cast<cudaStream_t>(stream)>>>(*g, V);
  return cuda_status(cudaGetLastError(), "scene vertices launch");
}

extern "C" int ss_facets_from_vertices(const double *V, int32_t H, int32_t W,
                                       const int64_t *row_keys,
                                       const int64_t *col_keys,
                                       const ss_facet_out *out,
                                       void *stream) {
  if (!V || !out || H < 2 || W < 2) {
    set_error("ss_facets_from_vertices: bad argument");
    return SS_ERR_ARG;
  }
  const long n = (long)(H - 1) * (W - 1);
  facets_from_vertices_kernel<<<grid_for(n), 256, 0,
                                reinterpret_cast<cudaStream_t>(stream)>>>(
      V, H, W, row_keys, col_keys, *out);
  return cuda_status(cudaGetLastError(), "facets launch");
}

extern "C" int ss_speckle_phasors_keyed(const int64_t *keys, int64_t n,
                                        uint64_t base, float *out,
                                        void *stream) {
  if (n < 0 || (n > 0 && (!keys || !out))) {
    set_error("ss_speckle_phasors_keyed: bad argument");
    return SS_ERR_ARG;
  }
  if (n == 0) return SS_OK;
  speckle_keyed_kernel<<<grid_for(n), 256, 0,
                         reinterpret_cast<cudaStream_t>(stream)>>>(
      keys, n, base, reinterpret_cast<float2 *>(out));
  return cuda_status(cudaGetLastError(), "speckle launch");
}

extern "C" int ss_offset_centers(const double *centers, int64_t n,
                                 const ss_frame *frame, double offset,
                                 double *out, void *stream) {
  if (n < 0 || !frame || (n > 0 && (!centers || !out))) {
    set_error("ss_offset_centers: bad argument");
    return SS_ERR_ARG;
  }
  if (n == 0) return SS_OK;
  offset_centers_kernel<<<grid_for(n), 256, 0,
                          reinterpret_cast<cudaStream_t>(stream)>>>(
      centers, n, *frame, offset, out);
  return cuda_status(cudaGetLastError(), "offset launch");
}
