// Internal helpers shared by the GB300 facet kernels (not part of the ABI).
#pragma once

#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include "soundersim_gb300.h"

#define SS_MAX_TB 8          // traces per CTA (trace block) upper bound
#define SS_MAX_TERMS 4096    // D_Phi series length the kernels accept
#define SS_FAD_N 32          // Weideman terms (roughness.py:67-80 default)

namespace ss {

constexpr double kPi = 3.141592653589793238462643383279502884;
constexpr double kTwoPi = 6.283185307179586476925286766559005768;

// Record the last CUDA error for ss_last_error().
void set_error(const char *msg);
int cuda_status(cudaError_t e, const char *where);

// Weideman (1994) Faddeeva constants for N = 32, computed on the host once.
struct FadCoeffs {
  double L;
  double a[SS_FAD_N];  // a[0] multiplies Z^(N-1) ... a[N-1] multiplies Z^0
};
const FadCoeffs &faddeeva_coeffs();

// Host-side decomposition of a trace-block x facet-chunk grid.
struct Plan {
  int tb;          // traces per CTA
  int n_groups;    // ceil(T / tb)
  int n_chunks;    // facet chunks per trace block
  int threads;     // CTA size
  size_t smem;     // dynamic shared memory bytes
};

// Ordered sum of per-CTA partial histograms (n_chunks, T, n_seg) into the
// output layout, plus the dropped-power partials (n_chunks, T).
struct ReduceArgs {
  int T, n_seg, n_samples, split, n_chunks;
  const void *part;
  const double *part_drop;
};
int launch_reduce(const ReduceArgs &r, bool f64_parts, const ss_output *out,
                  cudaStream_t st);
int sm_count();

// ---------------------------------------------------------------------
// float64 device math shared by the FP64 forms
// ---------------------------------------------------------------------
__device__ __forceinline__ double dot3(double ax, double ay, double az,
                                       double bx, double by, double bz) {
  return (ax * bx + ay * by) + az * bz;
}

// numpy's normalised sinc evaluated at y = x / pi: sin(pi y) / (pi y).
__device__ __forceinline__ double sinc_np(double y) {
  if (y == 0.0) return 1.0;
  return sinpi(y) / (kPi * y);
}

// Forward-hemisphere cos^(q/2) element field (antenna.py:138-143).
__device__ __forceinline__ double element_field64(double cb, double q,
                                                  double enabled) {
  if (enabled == 0.0) return 1.0;
  if (!(cb >= 0.0)) return 0.0;
  double c = fmin(fmax(cb, 0.0), 1.0);
  return pow(c, q / 2.0);
}

// One-way field gain for a departure direction (antenna.py:204-258).
__device__ __forceinline__ double gain64(int kind, int n, const double *pa, const double *pb,
                         const double *pv, double dx, double dy, double dz) {
  switch (kind) {
    case SS_PAT_DIPOLE: {
      double ca = dot3(dx, dy, dz, pv[0], pv[1], pv[2]);
      double s = sqrt(fmax(1.0 - ca * ca, 1e-12));
      return cos((kPi / 2.0) * ca) / s;
    }
    case SS_PAT_ARRAY: {
      double ne = pa[0];
      double u = dot3(dx, dy, dz, pv[0], pv[1], pv[2]);
      double ct = dot3(dx, dy, dz, pv[3], pv[4], pv[5]);
      double x = kPi * pb[0] * u;
      double sx = sin(x);
      double af = fabs(sx) < 1e-5 ? cos(ne * x) / cos(x)
                                  : sin(ne * x) / (ne * sx);
      return pb[1] * element_field64(ct, pb[2], pb[3]) * fabs(af);
    }
    case SS_PAT_ARRAY_TAPERED: {
      double u = dot3(dx, dy, dz, pv[0], pv[1], pv[2]);
      double ct = dot3(dx, dy, dz, pv[3], pv[4], pv[5]);
      double ctx = 0, stx = 0, crx = 0, srx = 0, wt = 0, wr = 0;
      for (int j = 0; j < n; ++j) {
        double mj = (double)j - (double)(n - 1) / 2.0;
        double ph = (2.0 * kPi * pb[0]) * u * mj;
        double s, c;
        sincos(ph, &s, &c);
        ctx += pa[j] * c;
        stx += pa[j] * s;
        crx += pa[n + j] * c;
        srx += pa[n + j] * s;
        wt += pa[j];
        wr += pa[n + j];
      }
      double aft = sqrt(ctx * ctx + stx * stx) / wt;
      double afr = sqrt(crx * crx + srx * srx) / wr;
      return pb[1] * element_field64(ct, pb[2], pb[3]) * sqrt(aft * afr);
    }
    case SS_PAT_FINITE_DIPOLE: {
      double kh = kPi * pa[0];
      double ca = dot3(dx, dy, dz, pv[0], pv[1], pv[2]);
      double s = sqrt(fmax(1.0 - ca * ca, 1e-12));
      return fabs(cos(kh * ca) - cos(kh)) / (s * (1.0 - cos(kh)));
    }
    case SS_PAT_TABULATED: {
      double ct = fmin(fmax(dot3(dx, dy, dz, pv[0], pv[1], pv[2]), -1.0), 1.0);
      double th = acos(ct);
      if (th <= pa[0]) return pb[0];
      if (th >= pa[n - 1]) return pb[n - 1];
      int lo = 0, hi = n - 1;  // pa[lo] <= th < pa[hi]
      while (hi - lo > 1) {
        int mid = (lo + hi) >> 1;
        if (pa[mid] <= th) lo = mid; else hi = mid;
      }
      double slope = (pb[hi] - pb[lo]) / (pa[hi] - pa[lo]);
      return slope * (th - pa[lo]) + pb[lo];
    }
    default:
      return 1.0;
  }
}

// Weideman rational approximation of w(z), Im z >= 0 (roughness.py:67-80).
__device__ __forceinline__ void faddeeva64(const double *a, double L, double zr,
                                           double zi, double &wr, double &wi) {
  // iz = i z = (-zi, zr); den = L - iz; Z = (L + iz) / den
  double dr = L + zi, di = -zr;            // den
  double nr = L - zi, ni = zr;             // L + iz
  double inv = 1.0 / (dr * dr + di * di);
  double Zr = (nr * dr + ni * di) * inv;   // (n * conj(d)) / |d|^2
  double Zi = (ni * dr - nr * di) * inv;
  double pr = a[0], pi = 0.0;              // Horner
  for (int j = 1; j < SS_FAD_N; ++j) {
    double tr = pr * Zr - pi * Zi + a[j];
    pi = pr * Zi + pi * Zr;
    pr = tr;
  }
  // 1/den and 1/den^2
  double ir = dr * inv, ii = -di * inv;
  double i2r = ir * ir - ii * ii, i2i = 2.0 * ir * ii;
  const double inv_sqrt_pi = 0.56418958354775628694807945156077259;
  wr = 2.0 * (pr * i2r - pi * i2i) + inv_sqrt_pi * ir;
  wi = 2.0 * (pr * i2i + pi * i2r) + inv_sqrt_pi * ii;
}

// One Eq 22-24 factor F(m) (roughness.py:92-107).
__device__ __forceinline__ double f_factor64(const double *fa, double L,
                                             double m, double a0, double edge,
                                             double l) {
  double sq = sqrt(m);
  double x = a0 * l / (2.0 * sq);
  double y = edge * sq / l;
  double ex2 = exp(-x * x), ey2 = exp(-y * y);
  double wzr, wzi, wxr, wxi;
  faddeeva64(fa, L, x, y, wzr, wzi);
  faddeeva64(fa, L, x, 0.0, wxr, wxi);
  double sr, cr;
  sincos(a0 * edge, &sr, &cr);
  // q = (x + i y) * rot * w(z); Re(i q) = -Im(q)
  double ar_ = x * cr - y * sr, ai_ = x * sr + y * cr;
  double qi = ar_ * wzi + ai_ * wzr;
  double t1 = -y * ex2 - ey2 * (-qi);
  double t2 = x * wxi;
  const double sqrt_pi = 1.7724538509055160272981674833411452;
  return 1.0 - ey2 * cos(edge * a0) + sqrt_pi * (t1 - t2);
}

// D_Phi series summed in order m = 1..n_terms (roughness.py:127-186).
__device__ __forceinline__ double d_phi64(int kind, int n_terms,
                                          const double *lgam, const double *fa,
                                          double fL, double sigma, double l,
                                          double K, double A0, double B0,
                                          double Lx, double Ly) {
  double sk = sigma * K;
  double x = sk * sk;
  double logx = x > 0.0 ? log(x) : -INFINITY;
  double kb2 = A0 * A0 + B0 * B0;
  double kb = sqrt(kb2);
  double acc = 0.0;
  for (int m = 1; m <= n_terms; ++m) {
    double mf = (double)m;
    double logp = (mf * logx - lgam[m]) - x;
    double term;
    if (kind == SS_ROUGH_EXP_AREA) {
      double q = (l / mf) * (l / mf);
      term = exp(logp) * (2.0 * kPi * q * pow(1.0 + (kb * kb) * q, -1.5)) *
             Lx * Ly;
    } else if (kind == SS_ROUGH_GAUSS_AREA) {
      term = exp(logp - kb2 * (l * l) / (4.0 * mf)) * (kPi * (l * l) / mf) *
             Lx * Ly;
    } else {
      double l4 = (l * l) * (l * l);
      term = exp(logp) * (l4 / (mf * mf)) *
             f_factor64(fa, fL, mf, A0, Lx, l) *
             f_factor64(fa, fL, mf, B0, Ly, l);
    }
    acc = acc + term;
  }
  return fmax(acc, 0.0);
}

}  // namespace ss
