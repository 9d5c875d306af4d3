// float32 device math shared by the split-precision kernels (internal).
#pragma once

#include "ss_internal.cuh"

#define SS_PAT_MAX 256

namespace ss {


// Antenna table lengths (pa, pb) of a pattern kind (antenna.py:76-118
// packing), staged as floats in shared memory by the split kernels.
__host__ __device__ __forceinline__ void pattern_lengths(int kind, int n,
                                                         int &pa_len,
                                                         int &pb_len) {
  pa_len = pb_len = 0;
  if (kind == SS_PAT_ARRAY) { pa_len = 1; pb_len = 4; }
  if (kind == SS_PAT_FINITE_DIPOLE) pa_len = 1;
  if (kind == SS_PAT_ARRAY_TAPERED) { pa_len = 2 * n; pb_len = 4; }
  if (kind == SS_PAT_TABULATED) { pa_len = n; pb_len = n; }
}

__device__ __forceinline__ float reduce_2pi(float x) {
  const float n = rintf(x * 0.159154943091895336f);
  float r = __fmaf_rn(-n, 6.28318548202514648f, x);
  return __fmaf_rn(-n, -1.74845553146951e-07f, r);
}

__device__ __forceinline__ float sin_red(float x) {
  return __sinf(reduce_2pi(x));
}

__device__ __forceinline__ float cos_red(float x) {
  return __cosf(reduce_2pi(x));
}

// sin(x)/x. MUFU sin has an ABSOLUTE error of a few 1e-7, which is a large
// RELATIVE error of sin(x)/x for small x (near-nadir facets), so |x| < 0.5
// uses the even Taylor series through x^8 (truncation < 3e-11 there).
__device__ __forceinline__ float sinc32(float x) {
  const float x2 = x * x;
  if (x2 < 0.25f)
    return __fmaf_rn(x2, __fmaf_rn(x2, __fmaf_rn(x2, __fmaf_rn(
               x2, 2.7557319e-06f, -1.9841270e-04f), 8.3333333e-03f),
               -1.6666667e-01f), 1.0f);
  return __fdividef(sin_red(x), x);
}

__device__ __forceinline__ float dot3f(float ax, float ay, float az, float bx,
                                       float by, float bz) {
  return __fmaf_rn(az, bz, __fmaf_rn(ay, by, ax * bx));
}

__device__ __forceinline__ float element_field32(float cb, float q,
                                                 float enabled) {
  if (enabled == 0.0f) return 1.0f;
  if (!(cb >= 0.0f)) return 0.0f;
  float c = fminf(fmaxf(cb, 0.0f), 1.0f);
  return c > 0.0f ? __powf(c, 0.5f * q) : (q == 0.0f ? 1.0f : 0.0f);
}

// float32 twin of gain64 (antenna.py:204-258); pa then pb staged in `tab`.
__device__ __forceinline__ float gain32(int kind, int n, int pa_len,
                                        const float *tab, const float *pv,
                                        float dx, float dy, float dz) {
  const float *pa = tab, *pb = tab + pa_len;
  switch (kind) {
    case SS_PAT_DIPOLE: {
      float ca = dot3f(dx, dy, dz, pv[0], pv[1], pv[2]);
      float s = sqrtf(fmaxf(1.0f - ca * ca, 1e-12f));
      return __fdividef(__cosf(1.57079632679f * ca), s);
    }
    case SS_PAT_ARRAY: {
      // sin(n x) / (n sin x) near the main lobe divides two small sines:
      // MUFU's absolute error (~1e-6) would be a relative error of 1e-4 in
      // g^4 there, so this kind uses the accurate sinf/cosf
      float ne = pa[0];
      float u = dot3f(dx, dy, dz, pv[0], pv[1], pv[2]);
      float ct = dot3f(dx, dy, dz, pv[3], pv[4], pv[5]);
      float x = 3.14159265359f * pb[0] * u;
      float sx = sinf(x);
      float af = fabsf(sx) < 1e-5f ? __fdividef(cosf(ne * x), cosf(x))
                                   : __fdividef(sinf(ne * x), ne * sx);
      return pb[1] * element_field32(ct, pb[2], pb[3]) * fabsf(af);
    }
    case SS_PAT_ARRAY_TAPERED: {
      float u = dot3f(dx, dy, dz, pv[0], pv[1], pv[2]);
      float ct = dot3f(dx, dy, dz, pv[3], pv[4], pv[5]);
      float ctx = 0, stx = 0, crx = 0, srx = 0, wt = 0, wr = 0;
      for (int j = 0; j < n; ++j) {
        float mj = (float)j - 0.5f * (float)(n - 1);
        float ph = reduce_2pi(6.28318530718f * pb[0] * u * mj);
        float s, c;
        __sincosf(ph, &s, &c);
        ctx += pa[j] * c;
        stx += pa[j] * s;
        crx += pa[n + j] * c;
        srx += pa[n + j] * s;
        wt += pa[j];
        wr += pa[n + j];
      }
      float aft = sqrtf(ctx * ctx + stx * stx) / wt;
      float afr = sqrtf(crx * crx + srx * srx) / wr;
      return pb[1] * element_field32(ct, pb[2], pb[3]) * sqrtf(aft * afr);
    }
    case SS_PAT_FINITE_DIPOLE: {
      float kh = 3.14159265359f * pa[0];
      float ca = dot3f(dx, dy, dz, pv[0], pv[1], pv[2]);
      float s = sqrtf(fmaxf(1.0f - ca * ca, 1e-12f));
      // cos(kh ca) - cos(kh) cancels near the axis: accurate cosf
      float ck = cosf(kh);
      return __fdividef(fabsf(cosf(kh * ca) - ck), s * (1.0f - ck));
    }
    case SS_PAT_TABULATED: {
      float ct = fminf(fmaxf(dot3f(dx, dy, dz, pv[0], pv[1], pv[2]), -1.0f),
                       1.0f);
      float th = acosf(ct);
      if (th <= pa[0]) return pb[0];
      if (th >= pa[n - 1]) return pb[n - 1];
      // segment with pa[lo] <= th < pa[lo + 1]: guessed from the mean
      // spacing (exact for the usual evenly sampled tables), then walked;
      // the same segment a binary search finds, for any ascending table
      const float span = pa[n - 1] - pa[0];
      int lo = (int)((th - pa[0]) * __fdividef((float)(n - 1), span));
      lo = min(max(lo, 0), n - 2);
      while (lo < n - 2 && pa[lo + 1] <= th) ++lo;
      while (lo > 0 && pa[lo] > th) --lo;
      const int hi = lo + 1;
      float slope = __fdividef(pb[hi] - pb[lo], pa[hi] - pa[lo]);
      return __fmaf_rn(slope, th - pa[lo], pb[lo]);
    }
    default:
      return 1.0f;
  }
}

// The tabulated kind of gain32 with its per-segment slopes and index scale
// staged once per CTA (`slope[j]` = the same quotient gain32 forms for
// segment j, `inv` = (n - 1) / span): the same operations on the same
// values, so the same gain bit for bit.
__device__ __forceinline__ void tab_slopes(int n, const float *pa,
                                           const float *pb, float *slope,
                                           float *inv, int tid, int nthr) {
  for (int j = tid; j < n - 1; j += nthr)
    slope[j] = __fdividef(pb[j + 1] - pb[j], pa[j + 1] - pa[j]);
  if (tid == 0) *inv = __fdividef((float)(n - 1), pa[n - 1] - pa[0]);
}

__device__ __forceinline__ float gain_tab32(int n, const float *pa,
                                            const float *pb,
                                            const float *slope, float inv,
                                            const float *pv, float dx,
                                            float dy, float dz) {
  float ct = fminf(fmaxf(dot3f(dx, dy, dz, pv[0], pv[1], pv[2]), -1.0f),
                   1.0f);
  float th = acosf(ct);
  if (th <= pa[0]) return pb[0];
  if (th >= pa[n - 1]) return pb[n - 1];
  int lo = (int)((th - pa[0]) * inv);
  lo = min(max(lo, 0), n - 2);
  while (lo < n - 2 && pa[lo + 1] <= th) ++lo;
  while (lo > 0 && pa[lo] > th) --lo;
  return __fmaf_rn(slope[lo], th - pa[lo], pb[lo]);
}

// Weideman w(z) in float32 (roughness.py:67-80).
__device__ __forceinline__ void faddeeva32(const float *a, float L, float zr,
                                           float zi, float &wr, float &wi) {
  float dr = L + zi, di = -zr;
  float nr = L - zi, ni = zr;
  float inv = __fdividef(1.0f, dr * dr + di * di);
  float Zr = (nr * dr + ni * di) * inv;
  float Zi = (ni * dr - nr * di) * inv;
  float pr = a[0], pi = 0.0f;
#pragma unroll 8
  for (int j = 1; j < SS_FAD_N; ++j) {
    float tr = __fmaf_rn(pr, Zr, __fmaf_rn(-pi, Zi, a[j]));
    pi = __fmaf_rn(pr, Zi, pi * Zr);
    pr = tr;
  }
  float ir = dr * inv, ii = -di * inv;
  float i2r = ir * ir - ii * ii, i2i = 2.0f * ir * ii;
  wr = 2.0f * (pr * i2r - pi * i2i) + 0.564189583548f * ir;
  wi = 2.0f * (pr * i2i + pi * i2r) + 0.564189583548f * ii;
}

__device__ __forceinline__ float f_factor32(const float *fa, float L, float m,
                                            float a0, float edge, float l) {
  float sq = sqrtf(m);
  float x = a0 * l / (2.0f * sq);
  float y = edge * sq / l;
  float ex2 = __expf(-x * x), ey2 = __expf(-y * y);
  float wzr, wzi, wxr, wxi;
  faddeeva32(fa, L, x, y, wzr, wzi);
  faddeeva32(fa, L, x, 0.0f, wxr, wxi);
  float ae = reduce_2pi(a0 * edge);
  float sr, cr;
  __sincosf(ae, &sr, &cr);
  float ar_ = x * cr - y * sr, ai_ = x * sr + y * cr;
  float qi = ar_ * wzi + ai_ * wzr;
  float t1 = -y * ex2 + ey2 * qi;
  float t2 = x * wxi;
  return 1.0f - ey2 * cr + 1.77245385091f * (t1 - t2);
}

// Terms of the D_Phi series that can matter in float32. The Poisson weight
// x^m e^-x / m! of term m peaks at m ~ x with width sqrt(x). Outside
// [x - t, x + t], t = 8 sqrt(x) + 8, the exact Poisson tails, weighted by
// a W_m growing like m^-2 towards small m (the steepest the weights grow),
// hold under 1e-15 of the sum for every x from 1e-3 to 3000 -- far below
// float32 resolution -- so the low terms are skipped for all kinds. Above
// the peak only the exponential-ACF
// weight W_m = 2 pi l^2 m (m^2 + (k_B l)^2)^(-3/2) Lx Ly is known to stay
// algebraic (the Gaussian weights carry exp(-c/m), which grows with m), so
// the high terms are skipped for that kind only; the reference's fixed
// length n_terms caps the range.
template <int KIND>
__device__ __forceinline__ void d_phi_range(float x, int n_terms, int &m_lo,
                                            int &m_hi) {
  const float half = 8.0f * sqrtf(x) + 8.0f;
  m_lo = max(1, (int)floorf(x - half));
  m_hi = KIND == SS_ROUGH_EXP_AREA ? min(n_terms, (int)ceilf(x + half))
                                   : n_terms;
}

// Poisson weight P_m(x) = e^-x x^m / m! in float32 to a few ulp, for the
// anchor of a run of terms. The direct form m ln x - ln m! - x cancels
// terms of several hundred (1e-4 absolute at float32 rounding, i.e. 1e-4
// relative in P near the 300-term cap), so for m >= 10 the anchor uses
// Stirling's series for ln m! (Abramowitz & Stegun 6.1.41):
//   ln P_m = m (log1p(-u) + u) - ln(2 pi m) / 2 - 1/(12 m) + 1/(360 m^3),
// u = (m - x) / m, whose terms are small; the omitted 1/(1260 m^5) is
// below 1e-8 at m = 10. Below m = 10, e^-x x^m / m! by products.
__device__ __forceinline__ float poisson_anchor(int m, float x) {
  const float mf = (float)m;
  if (m < 10) {
    float p = expf(-x);
    for (int j = 1; j <= m; ++j) p *= x / (float)j;
    return p;
  }
  const float u = (mf - x) / mf;
  const float im = 1.0f / mf;
  const float lp = mf * (log1pf(-u) + u) -
                   0.5f * logf(6.28318530718f * mf) -
                   im * (0.0833333333f - 0.00277777778f * im * im);
  return expf(lp);
}

// 1/m for m = 1..n (t[0] = 0), correctly rounded, staged by the CTA for the
// series: the reciprocal per term is then a shared-memory load instead of
// a MUFU operation (the rough kernels are bound by that pipe).
__device__ __forceinline__ void fill_inv_table(float *t, int n, int tid,
                                               int nthr) {
  for (int m = tid; m <= n; m += nthr)
    t[m] = m ? __frcp_rn((float)m) : 0.0f;
}

// D_Phi in float32. Poisson weights are exact (poisson_anchor) at the start
// of every run of 64 terms and follow the recursion P_m = P_(m-1) x / m
// inside it (a few roundings per step, ~1e-6 relative at a run's end).
// `inv`: the CTA's 1/m table (fill_inv_table) up to n_terms, or null.
template <int KIND>
__device__ __forceinline__ float d_phi32(int n_terms, const float *inv,
                                         const float *fa, float fL,
                                         float sigma, float l, float K,
                                         float A0, float B0, float Lx,
                                         float Ly) {
  const float sk = sigma * K;
  const float x = sk * sk;
  if (!(x > 0.0f)) return 0.0f;
  const float kb2 = A0 * A0 + B0 * B0;
  int m_lo, m_hi;
  d_phi_range<KIND>(x, n_terms, m_lo, m_hi);
  float acc = 0.0f;
  if (KIND == SS_ROUGH_EXP_AREA) {
    // W_m = 2 pi l^2 m^-2 (1 + (k_B l / m)^2)^(-3/2) Lx Ly: one reciprocal
    // and one reciprocal square root per term, the prefactor outside
    const float kl2 = kb2 * l * l;
    for (int m0 = m_lo; m0 <= m_hi; m0 += 64) {
      float mf = (float)m0;
      float P = poisson_anchor(m0, x);
      float im = inv ? inv[m0] : __fdividef(1.0f, mf);
      float im2 = im * im;
      float rs = rsqrtf(__fmaf_rn(kl2, im2, 1.0f));
      acc = __fmaf_rn(P * im2, rs * rs * rs, acc);
      const int m_end = min(m_hi, m0 + 63);
      for (int m = m0 + 1; m <= m_end; ++m) {
        mf += 1.0f;
        im = inv ? inv[m] : __fdividef(1.0f, mf);
        P *= x * im;
        im2 = im * im;
        rs = rsqrtf(__fmaf_rn(kl2, im2, 1.0f));
        acc = __fmaf_rn(P * im2, rs * rs * rs, acc);
      }
    }
    acc *= 6.28318530718f * l * l * Lx * Ly;
  } else if (KIND == SS_ROUGH_GAUSS_AREA) {
    // W_m = pi l^2 / m exp(-kB^2 l^2 / (4 m)) Lx Ly
    const float c = 0.25f * kb2 * l * l;
    for (int m0 = m_lo; m0 <= m_hi; m0 += 64) {
      float P = poisson_anchor(m0, x);
      const int m_end = min(m_hi, m0 + 63);
      for (int m = m0; m <= m_end; ++m) {
        const float mf = (float)m;
        const float im = inv ? inv[m] : __fdividef(1.0f, mf);
        if (m > m0) P *= x * im;
        acc = __fmaf_rn(P * __expf(-c * im), im, acc);
      }
    }
    acc *= 3.14159265359f * l * l * Lx * Ly;
  } else {
    const float l4 = (l * l) * (l * l);
    for (int m0 = m_lo; m0 <= m_hi; m0 += 64) {
      float P = poisson_anchor(m0, x);
      const int m_end = min(m_hi, m0 + 63);
      for (int m = m0; m <= m_end; ++m) {
        const float mf = (float)m;
        if (m > m0) P *= x / mf;
        if (P == 0.0f) continue;
        acc += P * (l4 / (mf * mf)) * f_factor32(fa, fL, mf, A0, Lx, l) *
               f_factor32(fa, fL, mf, B0, Ly, l);
      }
    }
  }
  return fmaxf(acc, 0.0f);
}

// D_Phi and its derivative with respect to x = (sigma K)^2 (adjoint): each
// series term P_m(x) W_m has d/dx = P_m W_m (m / x - 1), so
// dD/dx = sum_m (m - x) P_m W_m / x, accumulated with the factor (m - x)
// itself (the form sum m P W / x - D cancels to ~1/sqrt(x) of its terms
// near the Poisson peak). Same anchored Poisson weights as d_phi32.
template <int KIND>
__device__ __forceinline__ float d_phi32_dx(int n_terms, const float *inv,
                                            const float *fa, float fL,
                                            float sigma, float l, float K,
                                            float A0, float B0, float Lx,
                                            float Ly, float &dDdx) {
  dDdx = 0.0f;
  const float sk = sigma * K;
  const float x = sk * sk;
  if (!(x > 0.0f)) return 0.0f;
  const float kb2 = A0 * A0 + B0 * B0;
  int m_lo, m_hi;
  d_phi_range<KIND>(x, n_terms, m_lo, m_hi);
  float acc = 0.0f, accd = 0.0f;
  if (KIND == SS_ROUGH_EXP_AREA) {
    const float kl2 = kb2 * l * l;
    for (int m0 = m_lo; m0 <= m_hi; m0 += 64) {
      float mf = (float)m0;
      float P = poisson_anchor(m0, x);
      const int m_end = min(m_hi, m0 + 63);
      for (int m = m0; m <= m_end; ++m) {
        const float im = inv ? inv[m] : __fdividef(1.0f, mf);
        if (m > m0) P *= x * im;
        const float im2 = im * im;
        const float rs = rsqrtf(__fmaf_rn(kl2, im2, 1.0f));
        const float t = P * im2 * (rs * rs * rs);
        acc += t;
        accd = __fmaf_rn(mf - x, t, accd);
        mf += 1.0f;
      }
    }
    const float pref = 6.28318530718f * l * l * Lx * Ly;
    acc *= pref;
    accd *= pref;
  } else {
    for (int m0 = m_lo; m0 <= m_hi; m0 += 64) {
      float P = poisson_anchor(m0, x);
      const int m_end = min(m_hi, m0 + 63);
      for (int m = m0; m <= m_end; ++m) {
        const float mf = (float)m;
        const float im = inv ? inv[m] : __fdividef(1.0f, mf);
        if (m > m0) P *= x * im;
        float t;
        if (KIND == SS_ROUGH_GAUSS_AREA) {
          t = P * __expf(-0.25f * kb2 * l * l * im) *
              (3.14159265359f * l * l * Lx * Ly * im);
        } else {
          t = P == 0.0f ? 0.0f
                        : P * ((l * l) * (l * l) * im * im) *
                              f_factor32(fa, fL, mf, A0, Lx, l) *
                              f_factor32(fa, fL, mf, B0, Ly, l);
        }
        acc += t;
        accd = __fmaf_rn(mf - x, t, accd);
      }
    }
  }
  if (!(acc > 0.0f)) return 0.0f;
  dDdx = accd / x;
  return acc;
}

}  // namespace ss
