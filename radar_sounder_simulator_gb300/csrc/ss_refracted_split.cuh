// Split-precision refracted multilayer kernel.
//
// On GB300 the FP64 pipe runs at a small fraction of the FP32 rate, and the
// float64 form of this kernel is bound by it: fixed-budget Newton solves on
// 20 km geometry. This form runs every solve in float32 and carries the few
// quantities that need more than 24 bits as double-floats (hi + lo float
// pairs on the FP32 pipe):
//
//   * geometry relative to the local facet centres. Each two-point and joint
//     solve is posed in coordinates measured from the plane points (mean
//     point for the lookup pass, local facet centre for the crossing), with
//     the long platform offset p - o formed exactly as a double-float and
//     rounded once. The crossing is rebuilt from the short side of the ray
//     (the target's foot for a downward ray), so the float32 root places the
//     crossing to micrometres near the facet centre (to ~3e-5 m where a
//     steep facet's plane meets the ray hundreds of metres from its
//     centre), which keeps the facet's arrival direction -- and the sinc
//     arguments k_j (r_hat . e) -- accurate to ~1e-8 rad;
//   * facet lookups: the float32 mean-plane crossing gives the affine cell
//     coordinate (formed as a double-float; the crossing itself carries up
//     to ~5e-5 cells of float32 error through three interfaces); within
//     1.5e-4 cells of a rounding boundary the float64 mean-plane chain of
//     the reference is re-run for that pair, so the lookups are the
//     reference's integer decisions;
//   * leg lengths, optical path, carrier phase (2 k0 opl mod 2 pi) and the
//     fast-time bin in double-float. The optical path is stationary in the
//     crossing positions along the interface (Fermat), so that float32
//     error enters at second order. The crossings' float32 offsets from the
//     facet planes (up to ~1e-5 m for crossings far from the facet centre)
//     enter at first order, and both paths add them back (height from
//     exact products times the legs' index-weighted cosines): the optical
//     path then agrees with the float64 form's to ~1e-9 m. A sequential
//     chain through two or more interfaces is not stationary in its upper
//     crossings, so their float32 in-plane error also enters at first order
//     (~1e-5 m). A pair whose bin position lies within 1e-6 bins of a bin
//     edge (for such chains, within 5e-5 m of optical path) is re-evaluated
//     with the complete float64 path, so bins equal the float64 form's;
//   * radiometry (Fresnel, spreading, attenuation, antenna gain, sinc,
//     roughness series, diffuse channel) in float32.
//
// Validity: same-side tests in float32 on plane-relative heights; Newton
// convergence by the float32 Snell residual with tolerance 1e-4 (the float32
// floor is ~1e-6; failed solves sit at O(0.1)).
#pragma once

#include <algorithm>

#include "ss_df.cuh"
#include "ss_f32.cuh"
#include "ss_refracted_fp64.cuh"

namespace ss {

constexpr float kTiny32 = 1e-30f;
constexpr float kEps32 = 1.1920929e-07f;
constexpr float kTol32 = 1e-4f;
// Lookup guard band (cells): 3.3x the largest float32 cell-coordinate error
// measured through three interfaces (4.5e-5 cells).
constexpr float kLookupGuard = 1.5e-4f;
// Bin-edge band: kBinGuard bins; for sequential chains through two or more
// interfaces, the larger of that and kOplGuardChain metres of optical path
// (~6x their largest float32 optical-path error, 8.6e-6 m).
constexpr float kBinGuard = 1e-6f;
constexpr double kOplGuardChain = 5e-5;

// Per-interface constants of the float32 lookup pass.
struct MeanPlane32 {
  float mp[3];    // mean point (rounded)
  float mn[3];    // unit mean normal
  float dmp[3];   // mean point of the interface above minus this one
  float coef[4];  // affine fit: row = c0 x + c2 y + rb0, col = c1 x + c3 y + rb1
  float coefl[4]; // low parts of the coefficients (double-float)
  float rb[2];    // affine value at the mean point (double-float hi)
  float rbl[2];   // ... and lo
};

struct RefSplitConsts {
  float k0, amp_pref_j, kj, taper_inv, sigma, corr, fadL, n_exp;
  float K2h, K2l;             // 2 k0 as double-float
  float Ah, Al, Bh, Bl;       // u = opl A - B, A = 2/(c dt), B = t0/dt
  float bin_guard;            // bin-edge band in bins (kBinGuard, kOplGuardChain)
  float n_leg[SS_MAX_IFACE + 1], n_leg_lo[SS_MAX_IFACE + 1],
      eps_leg[SS_MAX_IFACE + 1], att_leg[SS_MAX_IFACE + 1],
      sig_c[SS_MAX_IFACE];
  // d att_leg / d alpha per leg (adjoint only): the legs whose attenuation
  // rate is the differentiated parameter
  float att_mask[SS_MAX_IFACE + 1];
  MeanPlane32 mean[SS_MAX_IFACE];
};

__device__ __forceinline__ float dot3a(const float *a, const float *b) {
  return __fmaf_rn(a[2], b[2], __fmaf_rn(a[1], b[1], a[0] * b[0]));
}

// float32 safeguarded Newton on sigma = sin(theta_rare) (the reference's
// update, refraction.py:120-144), stopping once the step is below float32
// resolution.
__device__ __forceinline__ float sigma32(float ar, float bd, float Lh,
                                         float ah, float bh, float ratio,
                                         int n_iter, float sig0 = -1.0f) {
  const float hi0 = 1.0f - 8.0f * kEps32;
  float sig = sig0 >= 0.0f
                  ? fminf(sig0, hi0)
                  : fminf(Lh / fmaxf(sqrtf(Lh * Lh + (ah + bh) * (ah + bh)),
                                     kTiny32), hi0);
  float lo = 0.0f, hi = hi0;
  for (int it = 0; it < n_iter; ++it) {
    const float v = ratio * sig;
    const float c1 = fmaxf((1.0f - sig) * (1.0f + sig), kTiny32);
    const float c2 = fmaxf((1.0f - v) * (1.0f + v), kTiny32);
    const float r1 = rsqrtf(c1), r2 = rsqrtf(c2);
    const float F = (ar * sig * r1 + bd * v * r2) - Lh;
    if (F <= 0.0f) lo = sig; else hi = sig;
    const float Fp = ar * r1 * r1 * r1 + bd * ratio * r2 * r2 * r2;
    const float sn = sig - F / fmaxf(Fp, kTiny32);
    const bool ok = (sn >= lo) && (sn <= hi) && isfinite(sn);
    const float nxt = ok ? sn : 0.5f * (lo + hi);
    const bool done = fabsf(nxt - sig) <= 2.0f * kEps32 * fmaxf(sig, 1e-6f);
    sig = nxt;
    if (done) break;
  }
  return sig;
}

// Two-point solve with both end points relative to the plane point.
struct Solve32 {
  float y[3];    // crossing relative to the plane point
  float sig;     // the root sigma = sin(theta) on the rare side
  float c1, c2;  // cos(theta) on the p side and on the q side
  float res;     // Snell residual (closure form, like refraction.py:155)
  bool sides;    // end points strictly on opposite sides of the plane
};

// `x0` (optional, relative to the plane point): a point near the crossing
// whose offset along the plane starts the Newton iteration on sigma in
// place of the straight-line guess (the root is the same).
__device__ __forceinline__ void snell_rel32(const float *P, const float *Q,
                                            const float *nrm, float n1,
                                            float n2, int n_iter,
                                            Solve32 &S,
                                            const float *x0 = nullptr) {
  const float h1 = dot3a(P, nrm), h2 = dot3a(Q, nrm);
  const float a = fabsf(h1), b = fabsf(h2);
  float fp[3], fq[3], w[3];
  for (int j = 0; j < 3; ++j) {
    fp[j] = P[j] - h1 * nrm[j];
    fq[j] = Q[j] - h2 * nrm[j];
    w[j] = fq[j] - fp[j];
  }
  const float L = sqrtf(dot3a(w, w));
  const float iL = 1.0f / fmaxf(L, kTiny32);
  const float s = fmaxf(a + b + L, kTiny32);
  const float inv_s = 1.0f / s;
  const float ah = a * inv_s, bh = b * inv_s, Lh = L * inv_s;
  const bool swap = n1 > n2;
  const float ratio = fminf(n1, n2) / fmaxf(n1, n2);
  const float ar = swap ? bh : ah, bd = swap ? ah : bh;
  float sig0 = -1.0f;
  if (x0) {
    // x0's offset from p's foot along w, normalised like tp, then the
    // rare-side offset tr and sigma = tr / sqrt(ar^2 + tr^2)
    const float tp0 = fminf(fmaxf(((x0[0] - fp[0]) * w[0] +
                                   (x0[1] - fp[1]) * w[1] +
                                   (x0[2] - fp[2]) * w[2]) * iL * inv_s,
                                  0.0f), Lh);
    const float tr0 = swap ? Lh - tp0 : tp0;
    sig0 = tr0 * rsqrtf(fmaxf(ar * ar + tr0 * tr0, kTiny32));
  }
  const float sig = sigma32(ar, bd, Lh, ah, bh, ratio, n_iter, sig0);
  S.sig = sig;
  const float v = ratio * sig;
  const float tr = ar * sig * rsqrtf(fmaxf((1.0f - sig) * (1.0f + sig),
                                           kTiny32));
  const float td = bd * v * rsqrtf(fmaxf((1.0f - v) * (1.0f + v), kTiny32));
  // offsets from the feet of p and q along w (t_p + t_q = Lh at the root)
  const float tp = fminf(fmaxf(swap ? td : tr, 0.0f), Lh);
  const float tq = fminf(fmaxf(swap ? tr : td, 0.0f), Lh);
  if (tq <= tp) {
    const float st = s * tq * iL;
    for (int j = 0; j < 3; ++j) S.y[j] = fq[j] - st * w[j];
  } else {
    const float st = s * tp * iL;
    for (int j = 0; j < 3; ++j) S.y[j] = fp[j] + st * w[j];
  }
  // back onto the plane: the foot of a 20 km distant point is off the plane
  // by (1 - |n|^2) x 20 km, and an off-plane crossing is a first-order
  // optical-path error (in-plane errors are second order)
  const float yn = dot3a(S.y, nrm);
  for (int j = 0; j < 3; ++j) S.y[j] -= yn * nrm[j];
  const float r1 = sqrtf(ah * ah + tp * tp), r2 = sqrtf(bh * bh + tq * tq);
  S.c1 = ah / fmaxf(r1, kTiny32);
  S.c2 = bh / fmaxf(r2, kTiny32);
  const float d2 = Lh - tp;
  S.res = n1 * tp / fmaxf(r1, kTiny32) -
          n2 * d2 / fmaxf(sqrtf(bh * bh + d2 * d2), kTiny32);
  S.sides = h1 * h2 < 0.0f;
}

// Affine cell of a float32 mean-plane crossing (offset y from the mean
// point); false when either coordinate is within the guard band of a
// rounding boundary.
__device__ __forceinline__ bool cell_of(const MeanPlane32 &M,
                                        const ss_interface &I, const float *y,
                                        int &row, int &col) {
  // rc = rb + y . coef as a double-float (the float32 sum of ~500-cell
  // terms would carry ~3e-5 cells of rounding)
  float f[2];
  int idx[2];
  for (int c = 0; c < 2; ++c) {
    float p0, e0, p1, e1, s0, es, s1, es1;
    two_prod(y[0], M.coef[c], p0, e0);
    two_prod(y[1], M.coef[2 + c], p1, e1);
    two_sum(p0, p1, s0, es);
    two_sum(M.rb[c], s0, s1, es1);
    const float lo = (es1 + es) + (e0 + e1) + M.rbl[c] +
                     (y[0] * M.coefl[c] + y[1] * M.coefl[2 + c]);
    const float fl = floorf(s1);
    float fr = (s1 - fl) + lo;  // in [-small, 1 + small)
    float base = fl;
    if (fr < 0.0f) { base -= 1.0f; fr += 1.0f; }
    else if (fr >= 1.0f) { base += 1.0f; fr -= 1.0f; }
    f[c] = fr;
    idx[c] = (int)(base + (fr >= 0.5f ? 1.0f : 0.0f));
  }
  row = min(max(idx[0], 0), I.ny - 1);
  col = min(max(idx[1], 0), I.nx - 1);
  return fabsf(f[0] - 0.5f) > kLookupGuard && fabsf(f[1] - 0.5f) > kLookupGuard;
}

// Exact reference cell from a float64 mean-plane solve (multilayer.py
// :375-381 for comp = true, refraction_joint sequential chain for false).
static __device__ __noinline__ void cell64(const ss_interface &I, const double *cur,
                                    const double *q, double n1, double n2,
                                    bool comp, double *x_out, int &row,
                                    int &col) {
  Snell64 R;
  snell64(cur, q, I.mean_point, I.mean_normal, n1, n2, 10, comp, R, true,
          true);
  const double rc0 = __dadd_rn(__dadd_rn(__dmul_rn(R.x[0], I.coef[0]),
                                         __dmul_rn(R.x[1], I.coef[2])),
                               I.coef[4]);
  const double rc1 = __dadd_rn(__dadd_rn(__dmul_rn(R.x[0], I.coef[1]),
                                         __dmul_rn(R.x[1], I.coef[3])),
                               I.coef[5]);
  row = (int)fmin(fmax(rint(rc0), 0.0), (double)(I.ny - 1));
  col = (int)fmin(fmax(rint(rc1), 0.0), (double)(I.nx - 1));
  for (int j = 0; j < 3; ++j) x_out[j] = R.x[j];
}

// The float64 mean-plane solve of cell64 restated in double-float on the
// FP32 pipe (GB300 runs float64 at 1/64 of the float32 rate): the same
// projections, the same safeguarded Newton on sigma = sin(theta) from the
// same start, ~2^-46 relative per operation, so the crossing agrees with
// the float64 one to ~1e-10 m. Returns false if the last Newton step has
// not settled below 1e-12 of sigma (the float64 chain then decides).
// Out of line: only the fix-up runs it, and one copy of its long body keeps
// that kernel's instruction footprint small.
static __device__ __noinline__ bool snell_df(const df *p, const df *q,
                                         const df *o, const df *nrm,
                                         double n1, double n2, int n_iter,
                                         df *x, float sig0) {
  const df tiny = df_make(1e-30f, 0.0f);
  df po[3], qo[3];
  for (int j = 0; j < 3; ++j) {
    po[j] = df_sub(p[j], o[j]);
    qo[j] = df_sub(q[j], o[j]);
  }
  const df h1 = df_dot3(po, nrm), h2 = df_dot3(qo, nrm);
  const df a = df_abs(h1), b = df_abs(h2);
  df fp[3], w[3];
  for (int j = 0; j < 3; ++j) {
    fp[j] = df_sub(p[j], df_mul(h1, nrm[j]));
    w[j] = df_sub(df_sub(q[j], df_mul(h2, nrm[j])), fp[j]);
  }
  const df L = df_sqrt(df_dot3(w, w));
  const df Lm = df_max(L, tiny);
  df u[3];
  for (int j = 0; j < 3; ++j) u[j] = df_div(w[j], Lm);
  const df s = df_max(df_add(df_add(a, b), L), tiny);
  const df ah = df_div(a, s), bh = df_div(b, s), Lh = df_div(L, s);
  const bool swap = n1 > n2;
  const df ratio = df_from_double(fmin(n1, n2) / fmax(n1, n2));
  const df ar = swap ? bh : ah, bd = swap ? ah : bh;
  const df one = df_make(1.0f, 0.0f);
  const df hi0 = df_from_double(1.0 - 8.0 * kEps64);
  const df abh = df_add(ah, bh);
  // start: the float32 pass's root when given (within ~1e-7 of this one:
  // two or three steps), else the float64 chain's straight-line start
  df sig = sig0 >= 0.0f
               ? df_min(df_make(sig0, 0.0f), hi0)
               : df_min(df_div(Lh, df_max(df_sqrt(df_add(df_mul(Lh, Lh),
                                                         df_mul(abh, abh))),
                                          tiny)),
                        hi0);
  df lo = df_make(0.0f, 0.0f), hi = hi0;
  float step = 1.0f;
  for (int it = 0; it < n_iter; ++it) {
    const df v = df_mul(ratio, sig);
    const df c1 = df_max(df_mul(df_sub(one, sig), df_add(one, sig)), tiny);
    const df c2 = df_max(df_mul(df_sub(one, v), df_add(one, v)), tiny);
    const df sc1 = df_sqrt(c1), sc2 = df_sqrt(c2);
    const df F = df_sub(df_add(df_div(df_mul(ar, sig), sc1),
                               df_div(df_mul(bd, v), sc2)),
                        Lh);
    if (!(F.hi > 0.0f)) lo = sig; else hi = sig;
    const df Fp = df_add(df_div(ar, df_mul(c1, sc1)),
                         df_div(df_mul(bd, ratio), df_mul(c2, sc2)));
    const df sn = df_sub(sig, df_div(F, df_max(Fp, tiny)));
    const bool ok = !df_lt(sn, lo) && !df_lt(hi, sn) && isfinite(sn.hi);
    const df nxt = ok ? sn : df_mul_f(df_add(lo, hi), 0.5f);
    step = fabsf(df_sub(nxt, sig).hi);
    sig = nxt;
    if (step <= 1e-14f * fmaxf(sig.hi, 1e-12f)) break;
  }
  const df c1 = df_max(df_mul(df_sub(one, sig), df_add(one, sig)), tiny);
  const df tr = df_div(df_mul(ar, sig), df_sqrt(c1));
  const df t = df_min(df_max(swap ? df_sub(Lh, tr) : tr,
                             df_make(0.0f, 0.0f)),
                      Lh);
  const df st = df_mul(s, t);
  for (int j = 0; j < 3; ++j) x[j] = df_add(fp[j], df_mul(st, u[j]));
  return step <= 1e-12f * fmaxf(sig.hi, 1e-12f);
}

// The reference's cell of a crossing from the double-float mean-plane solve
// when its affine coordinates lie more than 1e-8 cells from a rounding
// boundary (the two solves differ by ~1e-11 cells); false otherwise, and
// the float64 chain (cell64) decides.
__device__ __forceinline__ bool cell_df(const ss_interface &I, const df *cur,
                                        const df *q, double n1, double n2,
                                        df *x_out, int &row, int &col,
                                        float sig0 = -1.0f) {
  df o[3], nrm[3], x[3];
  for (int j = 0; j < 3; ++j) {
    o[j] = df_from_double(I.mean_point[j]);
    nrm[j] = df_from_double(I.mean_normal[j]);
  }
  if (!snell_df(cur, q, o, nrm, n1, n2, 10, x, sig0)) return false;
  int idx[2];
  for (int c = 0; c < 2; ++c) {
    const df rc = df_add(df_add(df_mul(x[0], df_from_double(I.coef[c])),
                                df_mul(x[1], df_from_double(I.coef[2 + c]))),
                         df_from_double(I.coef[4 + c]));
    // signed distance from the half between fl and fl + 1: the first
    // difference is exact, so d carries rounding relative to itself only
    const float fl = floorf(rc.hi);
    const float d = (rc.hi - (fl + 0.5f)) + rc.lo;
    if (fabsf(d) < 1e-8f) return false;
    idx[c] = (int)(fl + (d > 0.0f ? 1.0f : 0.0f));
  }
  row = min(max(idx[0], 0), I.ny - 1);
  col = min(max(idx[1], 0), I.nx - 1);
  for (int j = 0; j < 3; ++j) x_out[j] = x[j];
  return true;
}

// Plane point o and unit normal n of a table cell; t (optional) receives
// the normal as stored, whose direction the float64 form uses.
__device__ __forceinline__ void cell_plane32(const ss_interface &I, int row,
                                             int col, float *o, float *n,
                                             float *t = nullptr) {
  const float *g = I.table + ((size_t)row * I.nx + col) * 6;
  for (int j = 0; j < 3; ++j) {
    o[j] = g[j];
    n[j] = g[3 + j];
    if (t) t[j] = n[j];
  }
  // unit length to float32 rounding (rsqrt seed + one Newton step)
  const float nn = dot3a(n, n);
  float in = rsqrtf(nn);
  in = in * __fmaf_rn(-0.5f * nn * in, in, 1.5f);
  for (int j = 0; j < 3; ++j) n[j] *= in;
}

// t . y from exact products (two_prod) and a compensated sum: the height of
// a float32 point y (relative to the plane point) over the plane of normal
// t, to float32 precision of the height itself.
__device__ __forceinline__ float plane_height(const float *y, const float *t) {
  float p0, e0, p1, e1, p2, e2, s, f1, f2;
  two_prod(y[0], t[0], p0, e0);
  two_prod(y[1], t[1], p1, e1);
  two_prod(y[2], t[2], p2, e2);
  two_sum(p0, p1, s, f1);
  two_sum(s, p2, s, f2);
  return s + ((f1 + f2) + (e0 + e1 + e2));
}

__device__ __forceinline__ float fresnel_gamma32(float e1, float e2,
                                                 float c1) {
  const float n1 = sqrtf(e1), n2 = sqrtf(e2);
  const float s2 = (e1 / e2) * (1.0f - c1 * c1);
  const float c2 = sqrtf(fmaxf(1.0f - s2, 0.0f));
  return (n1 * c1 - n2 * c2) / (n1 * c1 + n2 * c2);
}

// Per-trace platform data staged in shared memory.
struct TraceS {
  float ph[3], pl[3];  // position as double-float
  float pm0[3];        // p - mean point of the first interface (rounded)
};

struct PathS {
  df opl;              // optical path over the legs above the final one
  df s_last;           // final-leg length
  float rh[3];         // unit vector facet -> last crossing
  float d0[3];         // platform -> first crossing
  float loss_db, sum_par, sum_perp, tau2, c0, c_last;
  float dloss;         // d loss_db / d alpha over these legs (GRAD only)
  bool valid;
  bool defer;          // needs the float64 lookup chain (EXACT = false only)
};

// p - o as a double-float vector (o a float point).
__device__ __forceinline__ void p_minus(const TraceS &T, const float *o,
                                        df *out) {
  for (int j = 0; j < 3; ++j) {
    float s, e;
    two_sum(T.ph[j], -o[j], s, e);
    out[j] = df_make(s, e + T.pl[j]);
  }
}

// ---------------------------------------------------------------------
// sequential chain (multilayer.py:352-406)
// ---------------------------------------------------------------------
template <bool EXACT, bool GRAD = false>
__device__ __forceinline__ void path_sequential_split(const RefArgs &a,
                                      const RefSplitConsts &k,
                                      const TraceS &T, const double *p64,
                                      const float *q, PathS &P) {
  float o_prev[3] = {0, 0, 0}, y_prev[3] = {0, 0, 0};
  df Pd[3], Qd[3];
  float y[3] = {0, 0, 0};
  P.valid = true;
  P.defer = false;
  P.opl = df_make(0.0f, 0.0f);
  P.loss_db = P.sum_par = P.sum_perp = 0.0f;
  P.dloss = 0.0f;
  P.tau2 = 1.0f;
  P.c0 = P.c_last = 1.0f;
  for (int i = 0; i < a.ni; ++i) {
    const ss_interface &I = a.ifc[i];
    const MeanPlane32 &M = k.mean[i];
    // facet lookup from the mean-plane crossing
    float Pm[3], Qm[3];
    for (int j = 0; j < 3; ++j) {
      Pm[j] = i == 0 ? T.pm0[j] : (o_prev[j] - M.mp[j]) + y_prev[j];
      Qm[j] = q[j] - M.mp[j];
    }
    Solve32 Sm;
    snell_rel32(Pm, Qm, M.mn, k.n_leg[i], k.n_leg[i + 1], 10, Sm);
    int row, col;
    if (!cell_of(M, I, Sm.y, row, col)) {
      if (!EXACT) {
        P.defer = true;
        return;
      }
      // the double-float solve decides unless the crossing is within
      // 1e-8 cells of a boundary; then the float64 chain of the reference
      df cdf[3], qdf[3], xdf[3];
      for (int j = 0; j < 3; ++j) {
        cdf[j] = i == 0 ? df_from_double(p64[j])
                        : df_make(o_prev[j], 0.0f);
        if (i > 0) cdf[j] = df_add_f(cdf[j], y_prev[j]);  // exact sum
        qdf[j] = df_make(q[j], 0.0f);
      }
      if (!cell_df(I, cdf, qdf, a.n_leg[i], a.n_leg[i + 1], xdf, row, col,
                   Sm.sig)) {
        double cur64[3], q64[3] = {q[0], q[1], q[2]}, x1[3];
        for (int j = 0; j < 3; ++j)
          cur64[j] = i == 0 ? p64[j] : (double)o_prev[j] + (double)y_prev[j];
        cell64(I, cur64, q64, a.n_leg[i], a.n_leg[i + 1], true, x1, row,
               col);
      }
    }
    float o[3], n[3], tn[3];
    cell_plane32(I, row, col, o, n, tn);
    // local-plane solve relative to the facet centre o
    if (i == 0) {
      p_minus(T, o, Pd);
    } else {
      for (int j = 0; j < 3; ++j)
        Pd[j] = df_add_f(df_diff(o_prev[j], o[j]), y_prev[j]);
    }
    for (int j = 0; j < 3; ++j) Qd[j] = df_diff(q[j], o[j]);
    const float Ph[3] = {Pd[0].hi, Pd[1].hi, Pd[2].hi};
    const float Qh[3] = {Qd[0].hi, Qd[1].hi, Qd[2].hi};
    // the mean-plane crossing relative to this facet's plane point starts
    // the local solve
    const float x0[3] = {(M.mp[0] - o[0]) + Sm.y[0],
                         (M.mp[1] - o[1]) + Sm.y[1],
                         (M.mp[2] - o[2]) + Sm.y[2]};
    Solve32 S;
    snell_rel32(Ph, Qh, n, k.n_leg[i], k.n_leg[i + 1], 25, S, x0);
    P.valid = P.valid && S.sides && fabsf(S.res) <= kTol32;
    for (int j = 0; j < 3; ++j) y[j] = S.y[j];
    // upper leg |cur - x| = |(cur - o) - y|
    const df s1 = df_norm3(df_add_f(Pd[0], -y[0]), df_add_f(Pd[1], -y[1]),
                           df_add_f(Pd[2], -y[2]));
    P.opl = df_add(P.opl, df_mul(s1, df_make(k.n_leg[i], k.n_leg_lo[i])));
    // A crossing hundreds of metres from its facet centre carries ~3e-5 m
    // of float32 rounding, ~1e-5 m of it off the facet plane, which the
    // optical path takes at first order (the in-plane part is second
    // order). Moving the crossing onto the plane of the table's own normal
    // changes the two legs by hp c1 and -hp c2, hp its height over that
    // plane towards the upper point. c2 is the two-point solve's cosine
    // towards the target: exact for the last crossing; for an upper
    // crossing of a chain the next leg bends at the next interface, so
    // that half of the correction is approximate there.
    {
      const float hp = dot3a(Ph, n) >= 0.0f ? plane_height(y, tn)
                                            : -plane_height(y, tn);
      P.opl = df_add_f(P.opl, hp * (k.n_leg[i] * S.c1 -
                                    k.n_leg[i + 1] * S.c2));
    }
    const float c_inc = fmaxf(S.c1, (float)kCMin);
    if (i == 0) {
      P.c0 = c_inc;
      for (int j = 0; j < 3; ++j) P.d0[j] = y[j] - Ph[j];
    }
    const float g = fresnel_gamma32(k.eps_leg[i], k.eps_leg[i + 1], c_inc);
    P.tau2 *= (1.0f - g * g);
    if (a.rough_cross) {
      const float kt = k.k0 * (k.n_leg[i] * c_inc - k.n_leg[i + 1] * S.c2);
      const float sk = k.sig_c[i] * kt;
      P.tau2 *= __expf(-2.0f * sk * sk);
    }
    const float s1f = s1.hi;
    P.loss_db += s1f * (k.att_leg[i] * 1e-3f);
    if (GRAD) P.dloss += s1f * (k.att_mask[i] * 1e-3f);
    P.sum_perp += s1f / k.n_leg[i];
    P.sum_par += s1f / (k.n_leg[i] * c_inc * c_inc);
    P.c_last = fmaxf(S.c2, (float)kCMin);
    for (int j = 0; j < 3; ++j) {
      o_prev[j] = o[j];
      y_prev[j] = y[j];
    }
  }
  // final leg: q - x = (q - o) - y
  const df fx = df_add_f(Qd[0], -y[0]), fy = df_add_f(Qd[1], -y[1]),
           fz = df_add_f(Qd[2], -y[2]);
  P.s_last = df_norm3(fx, fy, fz);
  const float is = 1.0f / fmaxf(P.s_last.hi, 1e-30f);
  P.rh[0] = -fx.hi * is;
  P.rh[1] = -fy.hi * is;
  P.rh[2] = -fz.hi * is;
}

// ---------------------------------------------------------------------
// joint solve (multilayer.py:408-457, refraction_joint.py:249-322)
// ---------------------------------------------------------------------
template <int NI, bool EXACT, bool GRAD = false>
__device__ __forceinline__ void path_joint_split(const RefArgs &a, const RefSplitConsts &k,
                                 const TraceS &T, const double *p64,
                                 const float *q, PathS &P) {
  // a deep stack (NI == kDeepNI) holds up to NI interfaces in its arrays
  // and crosses a.ni of them; the other instantiations fold ni to NI
  const int ni = NI == kDeepNI ? a.ni : NI;
  const float *nm = k.n_leg;
  P.defer = false;
  // pass 1: mean-plane chain anchors the lookups; its crossings (relative
  // to each mean point) also seed the joint solve
  int rows[NI], cols[NI];
  float Xm[NI][3], Sg[NI];
  {
    float Pm[3] = {T.pm0[0], T.pm0[1], T.pm0[2]};
    int last_unsafe = -1;
    for (int i = 0; i < ni; ++i) {
      const MeanPlane32 &M = k.mean[i];
      if (i > 0)
        for (int j = 0; j < 3; ++j) Pm[j] += M.dmp[j];
      const float Qm[3] = {q[0] - M.mp[0], q[1] - M.mp[1], q[2] - M.mp[2]};
      Solve32 S;
      snell_rel32(Pm, Qm, M.mn, nm[i], nm[i + 1], 10, S);
      if (!cell_of(M, a.ifc[i], S.y, rows[i], cols[i])) last_unsafe = i;
      for (int j = 0; j < 3; ++j) Pm[j] = Xm[i][j] = S.y[j];
      Sg[i] = S.sig;
    }
    if (last_unsafe >= 0) {  // the reference's float64 chain for this pair
      if (!EXACT) {
        P.defer = true;
        return;
      }
      // the double-float chain decides the cells up to the last one the
      // float32 chain left undecided (the mean-plane chain does not depend
      // on the cells, so the later float32 decisions stand) unless a
      // crossing is within 1e-8 cells of a boundary; then the float64
      // chain of the reference decides them all
      df cdf[3], qdf[3];
      for (int j = 0; j < 3; ++j) {
        cdf[j] = df_from_double(p64[j]);
        qdf[j] = df_make(q[j], 0.0f);
      }
      bool dfok = true;
      for (int i = 0; i <= last_unsafe && dfok; ++i)
        dfok = cell_df(a.ifc[i], cdf, qdf, a.n_leg[i], a.n_leg[i + 1], cdf,
                       rows[i], cols[i], Sg[i]);
      if (!dfok) {
        double c64[3] = {p64[0], p64[1], p64[2]};
        const double q64[3] = {q[0], q[1], q[2]};
        for (int i = 0; i < ni; ++i)
          cell64(a.ifc[i], c64, q64, a.n_leg[i], a.n_leg[i + 1], false, c64,
                 rows[i], cols[i]);
      }
    }
  }
  // local planes and exact segment bases D_0 = o_0 - p, D_k = o_k - o_k-1,
  // D_NI = q - o_NI-1
  float O[NI][3], Nn[NI][3];
  for (int i = 0; i < ni; ++i) cell_plane32(a.ifc[i], rows[i], cols[i], O[i],
                                            Nn[i]);
  df D[NI + 1][3];
  p_minus(T, O[0], D[0]);
  for (int j = 0; j < 3; ++j) {
    D[0][j].hi = -D[0][j].hi;
    D[0][j].lo = -D[0][j].lo;
    for (int i = 1; i < ni; ++i) D[i][j] = df_diff(O[i][j], O[i - 1][j]);
    D[ni][j] = df_diff(q[j], O[ni - 1][j]);
  }
  float tot[3] = {0, 0, 0};
  for (int i = 0; i <= ni; ++i)
    for (int j = 0; j < 3; ++j) tot[j] += D[i][j].hi;
  const float scale = fmaxf(sqrtf(dot3a(tot, tot)), kTiny32);
  const float inv = 1.0f / scale;
  float Ds[NI + 1][3];
  for (int i = 0; i <= ni; ++i)
    for (int j = 0; j < 3; ++j) Ds[i][j] = D[i][j].hi * inv;
  // Start of the joint solve: the mean-plane crossings of pass 1 moved onto
  // the looked-up facet planes (offsets y_i from o_i, scaled). They lie
  // within the facets' height and tilt from the mean planes -- tens of
  // metres, ~1e-3 of the path scale -- so Gauss-Newton converges in the
  // same few steps as from the reference's chain of two-point solves,
  // whose three float32 solves it saves; the root is the same.
  float Y[NI][3];
  for (int i = 0; i < ni; ++i) {
    const float *mp = k.mean[i].mp;
    for (int j = 0; j < 3; ++j)
      Y[i][j] = ((mp[j] - O[i][j]) + Xm[i][j]) * inv;
    const float yn = dot3a(Y[i], Nn[i]);
    for (int j = 0; j < 3; ++j) Y[i][j] -= yn * Nn[i][j];
  }
  // in-plane bases and offsets
  float B[NI][3][2], ab[NI][2];
  for (int i = 0; i < ni; ++i) {
    const float *n = Nn[i];
    const bool use_z = fabsf(n[2]) < 0.9f;
    const float a0 = use_z ? 0.0f : 1.0f, a2 = use_z ? 1.0f : 0.0f;
    float u[3] = {-a2 * n[1], a2 * n[0] - a0 * n[2], a0 * n[1]};
    const float un = rsqrtf(fmaxf(dot3a(u, u), 1e-30f));
    for (int j = 0; j < 3; ++j) u[j] *= un;
    const float v[3] = {n[1] * u[2] - n[2] * u[1], n[2] * u[0] - n[0] * u[2],
                        n[0] * u[1] - n[1] * u[0]};
    for (int j = 0; j < 3; ++j) {
      B[i][j][0] = u[j];
      B[i][j][1] = v[j];
    }
    for (int c = 0; c < 2; ++c)
      ab[i][c] = B[i][0][c] * Y[i][0] + B[i][1][c] * Y[i][1] +
                 B[i][2][c] * Y[i][2];
  }
  // B_i^T B_{i+1}: constant over the Newton steps
  float G[NI > 1 ? NI - 1 : 1][2][2];
  for (int i = 0; i + 1 < ni; ++i)
    for (int r = 0; r < 2; ++r)
      for (int c = 0; c < 2; ++c)
        G[i][r][c] = B[i][0][r] * B[i + 1][0][c] +
                     B[i][1][r] * B[i + 1][1][c] +
                     B[i][2][r] * B[i + 1][2][c];
  const float mu = 6.4e-6f;  // Levenberg shift, float32 eps^0.75
  float s[NI + 1], dh[NI + 1][3], f[NI][2], pp[NI][2], qq[NI][2];
  // geometry of the polyline for in-plane offsets abv: segment lengths sv,
  // unit directions dv, the in-plane projections pv_i = B_i^T d_i (incoming)
  // and qv_i = B_i^T d_i+1 (outgoing), and the stationarity residual
  // fv_i = B_i^T (n_i d_i - n_i+1 d_i+1) = n_i pv_i - n_i+1 qv_i
  auto geom = [&](const float (&abv)[NI][2], float (&sv)[NI + 1],
                  float (&dv)[NI + 1][3], float (&pv)[NI][2],
                  float (&qv)[NI][2], float (&fv)[NI][2]) {
    float y[NI][3];
    for (int i = 0; i < ni; ++i)
      for (int j = 0; j < 3; ++j)
        y[i][j] = B[i][j][0] * abv[i][0] + B[i][j][1] * abv[i][1];
    for (int kk = 0; kk <= ni; ++kk) {
      float d[3];
      for (int j = 0; j < 3; ++j)
        d[j] = Ds[kk][j] + (kk < ni ? y[kk][j] : 0.0f) -
               (kk > 0 ? y[kk - 1][j] : 0.0f);
      const float ss = fmaxf(sqrtf(dot3a(d, d)), kTiny32);
      sv[kk] = ss;
      const float is = 1.0f / ss;
      for (int j = 0; j < 3; ++j) dv[kk][j] = d[j] * is;
    }
    for (int i = 0; i < ni; ++i)
      for (int c = 0; c < 2; ++c) {
        pv[i][c] = B[i][0][c] * dv[i][0] + B[i][1][c] * dv[i][1] +
                   B[i][2][c] * dv[i][2];
        qv[i][c] = B[i][0][c] * dv[i + 1][0] + B[i][1][c] * dv[i + 1][1] +
                   B[i][2][c] * dv[i + 1][2];
        fv[i][c] = nm[i] * pv[i][c] - nm[i + 1] * qv[i][c];
      }
  };
  for (int it = 0; it < a.n_newton; ++it) {
    geom(ab, s, dh, pp, qq, f);
    // Gauss-Newton blocks. With orthonormal in-plane bases,
    // B_i^T (n/s)(I - d d^T) B_j = (n/s)(B_i^T B_j - (B_i^T d)(B_j^T d)^T),
    // so every block is a 2x2 from the projections (refraction_joint.py
    // :296-303 forms the same blocks through 3x3 products).
    float A[NI][2][2], Cm[NI > 1 ? NI - 1 : 1][2][2];
    for (int i = 0; i < ni; ++i) {
      const float sa = nm[i] / s[i], sb = nm[i + 1] / s[i + 1];
      for (int r = 0; r < 2; ++r)
        for (int c = 0; c < 2; ++c)
          A[i][r][c] = sa * ((r == c ? 1.0f : 0.0f) - pp[i][r] * pp[i][c]) +
                       sb * ((r == c ? 1.0f : 0.0f) - qq[i][r] * qq[i][c]) +
                       (r == c ? mu : 0.0f);
    }
    for (int i = 0; i + 1 < ni; ++i) {
      const float sb = nm[i + 1] / s[i + 1];
      for (int r = 0; r < 2; ++r)
        for (int c = 0; c < 2; ++c)
          Cm[i][r][c] = -sb * (G[i][r][c] - qq[i][r] * pp[i + 1][c]);
    }
    // block Thomas (refraction_joint.py:218-246)
    float dinv[NI][2][2], yv[NI][2], delta[NI][2];
    for (int i = 0; i < ni; ++i) {
      float M[2][2] = {{A[i][0][0], A[i][0][1]}, {A[i][1][0], A[i][1][1]}};
      float rhs[2] = {-f[i][0], -f[i][1]};
      if (i > 0) {
        float cpt[2][2];
        for (int r = 0; r < 2; ++r)
          for (int c = 0; c < 2; ++c)
            cpt[r][c] = Cm[i - 1][0][r] * dinv[i - 1][0][c] +
                        Cm[i - 1][1][r] * dinv[i - 1][1][c];
        for (int r = 0; r < 2; ++r) {
          for (int c = 0; c < 2; ++c)
            M[r][c] -= cpt[r][0] * Cm[i - 1][0][c] + cpt[r][1] * Cm[i - 1][1][c];
          rhs[r] -= cpt[r][0] * yv[i - 1][0] + cpt[r][1] * yv[i - 1][1];
        }
      }
      float det = M[0][0] * M[1][1] - M[0][1] * M[1][0];
      if (fabsf(det) < kTiny32) det = kTiny32;
      const float idt = 1.0f / det;
      dinv[i][0][0] = M[1][1] * idt;
      dinv[i][0][1] = -M[0][1] * idt;
      dinv[i][1][0] = -M[1][0] * idt;
      dinv[i][1][1] = M[0][0] * idt;
      yv[i][0] = rhs[0];
      yv[i][1] = rhs[1];
    }
    for (int i = ni - 1; i >= 0; --i) {
      float rr[2] = {yv[i][0], yv[i][1]};
      if (i < ni - 1)
        for (int r = 0; r < 2; ++r)
          rr[r] -= Cm[i][r][0] * delta[i + 1][0] + Cm[i][r][1] * delta[i + 1][1];
      for (int r = 0; r < 2; ++r)
        delta[i][r] = dinv[i][r][0] * rr[0] + dinv[i][r][1] * rr[1];
    }
    // converged to float32 resolution: take the step and stop
    float dmax = 0.0f;
    for (int i = 0; i < ni; ++i)
      dmax = fmaxf(dmax, fmaxf(fabsf(delta[i][0]), fabsf(delta[i][1])));
    if (dmax < 1e-7f) {
      for (int i = 0; i < ni; ++i)
        for (int r = 0; r < 2; ++r) ab[i][r] += delta[i][r];
      break;
    }
    // quadratic-convergence region: a full Newton step of at most 1e-2 of
    // the path scale decreases |F|^2 (step halving accepted lambda = 1 for
    // every such step measured on the benchmark scenes), so the merit
    // evaluation is skipped there; after a step below 1e-5 the remaining
    // error (~C d^2) is below the float32 resolution of the solve, so the
    // confirming Newton system is skipped too (a threshold of 3e-4 already
    // shows in the bed's phase, 3e-5 and 1e-5 do not)
    if (dmax < 1e-2f) {
      for (int i = 0; i < ni; ++i)
        for (int r = 0; r < 2; ++r) ab[i][r] += delta[i][r];
      if (dmax < 1e-5f) break;
      continue;
    }
    float m0 = 0.0f;
    for (int i = 0; i < ni; ++i) m0 += f[i][0] * f[i][0] + f[i][1] * f[i][1];
    float lam_sel = 0.0f, lam = 1.0f;
    for (int j = 0; j < a.n_backtrack; ++j, lam *= 0.5f) {
      float cand[NI][2], sc[NI + 1], dc[NI + 1][3], pc[NI][2], qc[NI][2],
          fc[NI][2];
      for (int i = 0; i < ni; ++i)
        for (int r = 0; r < 2; ++r) cand[i][r] = ab[i][r] + lam * delta[i][r];
      geom(cand, sc, dc, pc, qc, fc);
      float mc = 0.0f;
      for (int i = 0; i < ni; ++i) mc += fc[i][0] * fc[i][0] + fc[i][1] * fc[i][1];
      if (mc < m0) {
        lam_sel = lam;
        break;
      }
    }
    for (int i = 0; i < ni; ++i)
      for (int r = 0; r < 2; ++r) ab[i][r] += lam_sel * delta[i][r];
  }
  geom(ab, s, dh, pp, qq, f);
  // crossings in metres from their facet centres; exact segment lengths
  float Ym[NI][3];
  for (int i = 0; i < ni; ++i)
    for (int j = 0; j < 3; ++j)
      Ym[i][j] = scale * (B[i][j][0] * ab[i][0] + B[i][j][1] * ab[i][1]);
  df S[NI + 1];
  df seg_last[3];
  for (int kk = 0; kk <= ni; ++kk) {
    df v[3];
    for (int j = 0; j < 3; ++j) {
      v[j] = D[kk][j];
      if (kk < ni) v[j] = df_add_f(v[j], Ym[kk][j]);
      if (kk > 0) v[j] = df_add_f(v[j], -Ym[kk - 1][j]);
    }
    S[kk] = df_norm3(v[0], v[1], v[2]);
    if (kk == 0)
      for (int j = 0; j < 3; ++j) P.d0[j] = v[j].hi;
    if (kk == ni)
      for (int j = 0; j < 3; ++j) seg_last[j] = v[j];
  }
  // validity: residual, straddling, evanescence (refraction_joint:143-176)
  float residual = 0.0f;
  bool sides = true, evan = false;
  float cinc[NI], cout_[NI];
  for (int i = 0; i < ni; ++i) {
    const float *n = Nn[i];
    const float ct1 = dot3a(n, dh[i]), ct2 = dot3a(n, dh[i + 1]);
    float t1[3], t2[3], dG[3];
    for (int j = 0; j < 3; ++j) {
      t1[j] = dh[i][j] - ct1 * n[j];
      t2[j] = dh[i + 1][j] - ct2 * n[j];
      dG[j] = nm[i] * dh[i][j] - nm[i + 1] * dh[i + 1][j];
    }
    const float st1 = sqrtf(dot3a(t1, t1)), st2 = sqrtf(dot3a(t2, t2));
    cinc[i] = fabsf(ct1) * rsqrtf(fmaxf(ct1 * ct1 + st1 * st1, 1e-30f));
    cout_[i] = fabsf(ct2) * rsqrtf(fmaxf(ct2 * ct2 + st2 * st2, 1e-30f));
    const float nd = dot3a(n, dG);
    const float rt[3] = {dG[0] - nd * n[0], dG[1] - nd * n[1], dG[2] - nd * n[2]};
    const float res = sqrtf(dot3a(rt, rt));
    if (res > residual || isnan(res)) residual = res;
    sides = sides && (-dot3a(n, dh[i]) * dot3a(n, dh[i + 1]) < 0.0f);
    evan = evan || (nm[i] * st1 > nm[i + 1] * (1.0f + 64.0f * kEps32));
  }
  P.valid = (residual <= kTol32) && isfinite(residual) && sides && !evan;
  // The crossings lie in the planes of the float32-normalised normals,
  // up to ~1e-7 of their distance from the facet centre off the plane of
  // the table's normal as stored, which the float64 form uses; the
  // optical path takes that offset at first order (the in-plane error is
  // second order: the joint path is stationary in every crossing). Moving
  // crossing i onto the stored plane changes its two legs by hp c_in and
  // -hp c_out, hp its height over that plane towards the upper point.
  float dopl = 0.0f;
  for (int i = 0; i < ni; ++i) {
    const float *g =
        a.ifc[i].table + ((size_t)rows[i] * a.ifc[i].nx + cols[i]) * 6;
    const float tn[3] = {g[3], g[4], g[5]};
    const float h = plane_height(Ym[i], tn);
    const float hp = dot3a(Nn[i], dh[i]) <= 0.0f ? h : -h;
    dopl += hp * (nm[i] * cinc[i] - nm[i + 1] * cout_[i]);
  }
  // radiometry sums and optical path (multilayer.py:436-457)
  float c_inc[NI];
  for (int i = 0; i < ni; ++i) c_inc[i] = fmaxf(cinc[i], (float)kCMin);
  const float c_surf = c_inc[a.k_pad];
  float tau2 = 1.0f, loss = 0.0f, sperp = 0.0f, spar = 0.0f, dloss = 0.0f;
  df opl = df_make(0.0f, 0.0f);
  for (int i = 0; i < ni; ++i) {
    const float g = fresnel_gamma32(k.eps_leg[i], k.eps_leg[i + 1], c_inc[i]);
    tau2 *= (1.0f - g * g);
    if (a.rough_cross) {
      const float kt = k.k0 * (nm[i] * cinc[i] - nm[i + 1] * cout_[i]);
      const float sk = k.sig_c[i] * kt;
      tau2 *= __expf(-2.0f * sk * sk);
    }
    const float cp = i < a.k_pad ? c_surf : c_inc[i];
    const float si = S[i].hi;
    opl = df_add(opl, df_mul(S[i], df_make(k.n_leg[i], k.n_leg_lo[i])));
    loss += si * (k.att_leg[i] * 1e-3f);
    if (GRAD) dloss += si * (k.att_mask[i] * 1e-3f);
    sperp += si / nm[i];
    spar += si / (nm[i] * cp * cp);
  }
  P.tau2 = tau2;
  P.opl = df_add_f(opl, dopl);
  P.loss_db = loss;
  P.dloss = dloss;
  P.sum_perp = sperp;
  P.sum_par = spar;
  P.c0 = c_surf;
  P.c_last = fmaxf(cout_[ni - 1], (float)kCMin);
  P.s_last = S[ni];
  const float is = 1.0f / fmaxf(S[ni].hi, 1e-30f);
  for (int j = 0; j < 3; ++j) P.rh[j] = -seg_last[j].hi * is;
}

// Platform data of trace t in the split kernels' form.
__device__ __forceinline__ void load_trace(const RefArgs &a, int t, TraceS &T,
                                           double *p64, float *u, float *pv) {
  for (int j = 0; j < 3; ++j) {
    const double pj = a.pos[3 * t + j];
    p64[j] = pj;
    const df v = df_from_double(pj);
    T.ph[j] = v.hi;
    T.pl[j] = v.lo;
    T.pm0[j] = (float)(pj - a.ifc[0].mean_point[j]);
    u[j] = a.uct ? (float)a.uct[3 * t + j] : 0.0f;
  }
  for (int j = 0; j < 6; ++j)
    pv[j] = (a.pv && j < a.pv_len) ? (float)a.pv[a.pv_len * t + j] : 0.0f;
}

// Result of one (trace, facet) pair.
struct PairOut {
  float re, im, pwr;
  int bin;  // segment index, or -1 when the pair is dropped
};

// One (trace, facet) pair of the split form (multilayer.py:459-588 per
// pair). With EXACT = false the pair returns false, without a result, when
// it needs a float64 decision: a facet lookup or a fast-time bin within the
// guard band of a rounding boundary. The fast kernel holds no float64 code
// (which halves its registers) and leaves those pairs -- a few per thousand
// -- to the fix-up kernel, which evaluates them with EXACT = true.
// Partial derivatives of one pair's contribution (adjoint only): the part
// proportional to the facet's reflection coefficient, its derivative with
// respect to the facet's rms height, and d loss_db / d alpha.
struct PairGrad {
  float gre, gim;  // contribution of the gamma-proportional terms
  float sre, sim;  // d contribution / d sigma
  float dloss;
};

template <int NI, int ROUGH, bool EXACT, bool GRAD = false,
          bool PLAIN = false>
__device__ __forceinline__ bool pair_eval(
    const RefArgs &a, const RefSplitConsts &k, const TraceS &T,
    const double *p64, const float *u, const float *pv, const float *pat,
    int pa_len, const float *lg, const float *fad, int i, const float *q,
    PairOut &o, PairGrad *pg = nullptr) {
  PathS P;
  if (NI == 0)
    path_sequential_split<EXACT, GRAD>(a, k, T, p64, q, P);
  else
    path_joint_split<NI == 0 ? 1 : NI, EXACT, GRAD>(a, k, T, p64, q, P);
  if (!EXACT && P.defer) return false;
  const int nj = a.leg_last;
  const float n0 = k.n_leg[0], njn = k.n_leg[nj];
  const float nsf = (float)a.n_samples;
  const float fn[3] = {a.F.nx[i], a.F.ny[i], a.F.nz[i]};
  const float fa = a.F.area[i];
  // final leg (medium j)
  const df opl = df_add(P.opl, df_mul(P.s_last, df_make(k.n_leg[nj],
                                                        k.n_leg_lo[nj])));
  const float s_j = P.s_last.hi;
  const float *rh = P.rh;
  const float loss = P.loss_db + s_j * (k.att_leg[nj] * 1e-3f);
  const float sperp = P.sum_perp + s_j / njn;
  const float spar = P.sum_par + s_j / (njn * P.c_last * P.c_last);
  const float l_perp = n0 * sperp;
  const float l_par = n0 * P.c0 * P.c0 * spar;
  const float flux = (n0 * P.c0) / (njn * P.c_last);
  const float att_f = exp2f(-loss * 0.33219280949f);  // 10^(-loss/10)
  const float cos_t = dot3a(rh, fn);
  float spread = P.tau2 * flux / (l_par * l_perp);
  if (!PLAIN && a.pat_kind != SS_PAT_ISOTROPIC) {
    const float dm = rsqrtf(fmaxf(dot3a(P.d0, P.d0), 1e-30f));
    const float g = gain32(a.pat_kind, a.pat_n, pa_len, pat, pv,
                           P.d0[0] * dm, P.d0[1] * dm, P.d0[2] * dm);
    spread *= g * g;
  }
  float re, im, pwr;
  if (a.coherent) {
    const float gam = a.F.gamma_f64 ? (float)a.F.gamma_f64[i]
                                    : (float)a.gamma;
    const float f1[3] = {a.F.e1x[i], a.F.e1y[i], a.F.e1z[i]};
    const float f2[3] = {a.F.e2x[i], a.F.e2y[i], a.F.e2z[i]};
    const float d1 = dot3a(rh, f1), d2 = dot3a(rh, f2);
    const float base = k.amp_pref_j * gam * cos_t * spread * att_f;
    float amp = base * fa * sinc32(k.kj * d1) * sinc32(k.kj * d2);
    if (!PLAIN && a.taper) {
      const float ct = fminf(fmaxf(cos_t, (float)kCMin), 1.0f);
      const float ct2 = ct * ct;
      amp *= __expf(-__fdividef(1.0f - ct2, ct2) * k.taper_inv);
    }
    float cr = amp, ci = 0.0f;
    float dcr = 0.0f, dci = 0.0f;  // d (cr, ci) / d sigma (GRAD)
    if (ROUGH != SS_ROUGH_NONE) {
      const float sg = a.F.sigma ? a.F.sigma[i] : k.sigma;
      const float lc = a.F.corr ? a.F.corr[i] : k.corr;
      const float l1 = sqrtf(dot3a(f1, f1)), l2 = sqrtf(dot3a(f2, f2));
      const float kk = 2.0f * k.kj * cos_t;
      float dpdx = 0.0f;
      const float dp =
          GRAD ? d_phi32_dx<ROUGH>(a.n_terms, lg, fad, k.fadL, sg, lc, kk,
                                   2.0f * k.kj * d1 / l1,
                                   2.0f * k.kj * d2 / l2, l1, l2, dpdx)
               : d_phi32<ROUGH>(a.n_terms, lg, fad, k.fadL, sg, lc, kk,
                                2.0f * k.kj * d1 / l1, 2.0f * k.kj * d2 / l2,
                                l1, l2);
      const float sk = sg * kk;
      const float att_r = __expf(-0.5f * sk * sk);
      cr = amp * att_r;
      if (GRAD) dcr = -amp * att_r * sg * kk * kk;
      if (fa > 0.0f) {
        const float sq = sqrtf(dp);
        const float ai = base * sq;
        cr += ai * a.F.phasor[2 * i];
        ci += ai * a.F.phasor[2 * i + 1];
        if (GRAD && sq > 0.0f) {
          // d sqrt(D) / d sigma = D'(x) 2 sigma K^2 / (2 sqrt(D))
          const float dai = base * dpdx * sg * kk * kk / sq;
          dcr += dai * a.F.phasor[2 * i];
          dci = dai * a.F.phasor[2 * i + 1];
        }
      }
    }
    const float gcr = cr, gci = ci;  // gamma-proportional part
    if (!PLAIN && a.F.diffuse_amp && fa > 0.0f) {
      const float ct = fmaxf(cos_t, 0.0f);
      const float ad = sqrtf(fa * 0.15915494309f) *
                       (float)a.F.diffuse_amp[i] * ct *
                       (ct > 0.0f ? __powf(ct, 0.5f * k.n_exp)
                                  : (k.n_exp == 0.0f ? 1.0f : 0.0f)) *
                       spread * att_f;
      cr += ad * a.F.diffuse_phasor[2 * i];
      ci += ad * a.F.diffuse_phasor[2 * i + 1];
    }
    // carrier phase 2 k0 opl mod 2 pi (double-float, Cody-Waite)
    float ph, pe;
    two_prod(k.K2h, opl.hi, ph, pe);
    const float pl = pe + __fmaf_rn(k.K2h, opl.lo, k.K2l * opl.hi);
    const float n2 = rintf(ph * 0.159154943091895336f);
    float red = __fmaf_rn(-n2, 6.28318548202514648f, ph);  // exact
    red = __fmaf_rn(-n2, -1.74845553146951e-07f, red) + pl;
    float sn, cs;
    __sincosf(red, &sn, &cs);
    re = cr * sn - ci * cs;
    im = cr * cs + ci * sn;
    pwr = re * re + im * im;
    if (GRAD) {
      pg->gre = gcr * sn - gci * cs;
      pg->gim = gcr * cs + gci * sn;
      pg->sre = dcr * sn - dci * cs;
      pg->sim = dcr * cs + dci * sn;
      pg->dloss = P.dloss + s_j * (k.att_mask[nj] * 1e-3f);
    }
  } else {
    const float aa = fa * cos_t * spread;
    re = aa * aa * att_f * att_f;
    im = 0.0f;
    pwr = re;
  }
  // fast-time bin u = opl A - B (double-float), float64 path near edges
  float up, ue, us, ue2;
  two_prod(opl.hi, k.Ah, up, ue);
  two_sum(up, -k.Bh, us, ue2);
  const float ul = (ue2 + ue) + __fmaf_rn(opl.hi, k.Al, opl.lo * k.Ah) - k.Bl;
  float fb = floorf(us);
  float frac = (us - fb) + ul;
  if (frac < 0.0f) { fb -= 1.0f; frac += 1.0f; }
  else if (frac >= 1.0f) { fb += 1.0f; frac -= 1.0f; }
  if ((frac < k.bin_guard || frac > 1.0f - k.bin_guard) && us > -4.0f &&
      us < nsf + 4.0f) {
    if (!EXACT) return false;
    bool v64;
    const double q64[3] = {q[0], q[1], q[2]};
    const double o64 = full_opl64<NI>(a, p64, q64, v64);
    const double twtt = __ddiv_rn(__dmul_rn(2.0, o64), a.c);
    fb = (float)floor(__ddiv_rn(__dsub_rn(twtt, a.t0), a.dt));
  }
  o.re = re;
  o.im = im;
  o.pwr = pwr;
  o.bin = -1;
  if (P.valid && fb >= 0.0f && fb < nsf) {
    int b = (int)fb;
    if (!PLAIN && a.split) {
      const float v[3] = {q[0] - T.ph[0], q[1] - T.ph[1], q[2] - T.ph[2]};
      if (dot3a(v, u) > 0.0f) b += a.n_samples;
    }
    o.bin = b;
  }
  return true;
}

// One CTA's work item of the fast kernel: facet chunk `chunk` of trace
// block `group`; thread <-> facet; per-trace histograms in shared memory;
// pairs that need a float64 decision are marked in the deferral bitmask
// (bit t * defer_w + (i - lo_t)). Shared by the one-call kernel (item =
// block index) and the batched persistent kernel (item from a work queue).
template <int NI, int ROUGH, bool PLAIN>
__device__ __forceinline__ void refracted_split_cta(const RefArgs &a,
                                                    const RefSplitConsts &k,
                                                    int chunk, int group,
                                                    unsigned char *smem_raw) {
  float2 *hist = reinterpret_cast<float2 *>(smem_raw);
  float *lg = reinterpret_cast<float *>(hist + (size_t)a.tb * a.n_seg);
  __shared__ double s_p64[SS_MAX_TB][3];
  __shared__ TraceS s_tr[SS_MAX_TB];
  __shared__ float s_u[SS_MAX_TB][3], s_pv[SS_MAX_TB][6];
  __shared__ int s_lo[SS_MAX_TB], s_hi[SS_MAX_TB];
  __shared__ float s_drop[SS_MAX_TB];
  __shared__ float s_pat[SS_PAT_MAX];
  __shared__ float s_fad[SS_FAD_N];
  __shared__ int s_rng[2];
  __shared__ int s_next;
  const int t_base = group * a.tb;
  const int nt = min(a.tb, a.T - t_base);
  const int tid = threadIdx.x;
  int pa_len, pb_len;
  pattern_lengths(a.pat_kind, a.pat_n, pa_len, pb_len);
  if (tid < nt) {
    const int t = t_base + tid;
    load_trace(a, t, s_tr[tid], s_p64[tid], s_u[tid], s_pv[tid]);
    long lo = (long)a.off[t] * a.bs;
    long hi = min((long)(a.off[t] + a.n_win) * a.bs, (long)a.N);
    s_lo[tid] = (int)min(lo, (long)a.N);
    s_hi[tid] = (int)hi;
    s_drop[tid] = 0.0f;
  }
  for (int j = tid; j < pa_len; j += blockDim.x) s_pat[j] = (float)a.pa[j];
  for (int j = tid; j < pb_len; j += blockDim.x)
    s_pat[pa_len + j] = (float)a.pb[j];
  if (ROUGH == SS_ROUGH_GAUSS_FULL && tid < SS_FAD_N)
    s_fad[tid] = (float)a.fad.a[tid];
  for (int j = tid; j < a.tb * a.n_seg; j += blockDim.x)
    hist[j] = make_float2(0.0f, 0.0f);
  if (ROUGH != SS_ROUGH_NONE) fill_inv_table(lg, a.n_terms, tid, blockDim.x);
  __syncthreads();
  if (tid == 0) {
    int lo = s_lo[0], hi = s_hi[0];
    for (int j = 1; j < nt; ++j) {
      lo = min(lo, s_lo[j]);
      hi = max(hi, s_hi[j]);
    }
    long len = max(hi - lo, 0);
    s_rng[0] = lo + (int)(len * chunk / a.n_chunks);
    s_rng[1] = lo + (int)(len * (chunk + 1) / a.n_chunks);
    s_next = s_rng[0];
  }
  __syncthreads();

  // warps take 32 consecutive facets at a time from a shared counter, so a
  // warp whose pairs iterate longer (solver steps, series terms, deferred
  // decisions) does not hold the others at the write-out barrier
  const int lane = tid & 31;
  const int i_end = s_rng[1];
  for (;;) {
    int base = 0;
    if (lane == 0) base = atomicAdd(&s_next, 32);
    base = __shfl_sync(0xffffffffu, base, 0);
    if (base >= i_end) break;
    const int i = base + lane;
    if (i >= i_end) continue;
    const float q[3] = {a.F.cx[i], a.F.cy[i], a.F.cz[i]};
    for (int tt = 0; tt < nt; ++tt) {
      if (i < s_lo[tt] || i >= s_hi[tt]) continue;
      PairOut o;
      if (!pair_eval<NI, ROUGH, false, false, PLAIN>(
              a, k, s_tr[tt], s_p64[tt], s_u[tt], s_pv[tt], s_pat, pa_len,
              lg, s_fad, i, q, o)) {
        const unsigned long long bit =
            (unsigned long long)(t_base + tt) * a.defer_w + (i - s_lo[tt]);
        atomicOr(&a.defer_mask[bit >> 5], 1u << (bit & 31));
        continue;
      }
      if (o.bin >= 0) {
        float2 *h = hist + (size_t)tt * a.n_seg + o.bin;
        atomicAdd(&h->x, o.re);
        if (a.coherent) atomicAdd(&h->y, o.im);
      } else {
        atomicAdd(&s_drop[tt], o.pwr);
      }
    }
  }
  __syncthreads();
  float2 *part = reinterpret_cast<float2 *>(a.part);
  for (int tt = 0; tt < nt; ++tt) {
    const size_t base = ((size_t)chunk * a.T + t_base + tt) * a.n_seg;
    for (int j = tid; j < a.n_seg; j += blockDim.x)
      part[base + j] = hist[(size_t)tt * a.n_seg + j];
  }
  if (tid < nt)
    a.part_drop[(size_t)chunk * a.T + t_base + tid] = (double)s_drop[tid];
}

// Fast kernel: one CTA per (facet chunk, trace block).
// Up to two crossings the solve fits 64 registers, so two 512-thread CTAs
// share an SM (32 warps; the joint solve through two interfaces spills a
// few words at that budget and still gains 8%); through three or more it
// keeps ~125 registers and one CTA.
template <int NI, int ROUGH, bool PLAIN>
__global__ void __launch_bounds__(kSplitThreads, NI >= 3 ? 1 : 2)
refracted_split_kernel(RefArgs a, RefSplitConsts k) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  refracted_split_cta<NI, ROUGH, PLAIN>(a, k, blockIdx.x, blockIdx.y,
                                        smem_raw);
}

// Fix-up kernel: evaluates the deferred pairs with the float64 decisions
// and adds them to facet chunk 0's partials, which the fast kernel has
// written in full. Deferred pairs are sparse (a few per thousand bits), so
// each warp scans 32 mask words at a time and queues their set bits in
// shared memory, then evaluates them 32 at a time with every lane busy.
// 4 CTAs per SM (128 registers, a few hundred bytes of spills): the
// fix-up is bound by instruction fetch over its long exact path, and twice
// the resident warps (from 246 registers and two CTAs) hide more of it.
constexpr int kFixWarps = 4;
constexpr int kFixQueue = 32 * 32 + 32;  // one scan round plus a partial batch

template <int NI, int ROUGH>
__device__ __forceinline__ void fixup_pair(const RefArgs &a,
                                           const RefSplitConsts &k,
                                           unsigned long long bit,
                                           const float *pat, int pa_len,
                                           const float *lg, const float *fad) {
  const int t = (int)(bit / a.defer_w);
  const long lo = min((long)a.off[t] * a.bs, (long)a.N);
  const int i = (int)(lo + (long)(bit % a.defer_w));
  TraceS T;
  double p64[3];
  float u[3], pv[6];
  load_trace(a, t, T, p64, u, pv);
  const float q[3] = {a.F.cx[i], a.F.cy[i], a.F.cz[i]};
  PairOut o;
  pair_eval<NI, ROUGH, true>(a, k, T, p64, u, pv, pat, pa_len, lg, fad, i, q,
                             o);
  if (o.bin >= 0) {
    float2 *h = reinterpret_cast<float2 *>(a.part) + (size_t)t * a.n_seg +
                o.bin;
    atomicAdd(&h->x, o.re);
    if (a.coherent) atomicAdd(&h->y, o.im);
  } else {
    atomicAdd(&a.part_drop[t], (double)o.pwr);
  }
}

template <int NI, int ROUGH>
__global__ void __launch_bounds__(32 * kFixWarps, 4)
refracted_split_fixup(RefArgs a, RefSplitConsts k) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float *lg = reinterpret_cast<float *>(smem_raw);
  __shared__ float s_pat[SS_PAT_MAX];
  __shared__ float s_fad[SS_FAD_N];
  __shared__ unsigned long long s_q[kFixWarps][kFixQueue];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  int pa_len, pb_len;
  pattern_lengths(a.pat_kind, a.pat_n, pa_len, pb_len);
  for (int j = tid; j < pa_len; j += blockDim.x) s_pat[j] = (float)a.pa[j];
  for (int j = tid; j < pb_len; j += blockDim.x)
    s_pat[pa_len + j] = (float)a.pb[j];
  if (ROUGH == SS_ROUGH_GAUSS_FULL && tid < SS_FAD_N)
    s_fad[tid] = (float)a.fad.a[tid];
  if (ROUGH != SS_ROUGH_NONE) fill_inv_table(lg, a.n_terms, tid, blockDim.x);
  __syncthreads();
  const unsigned long long n_words =
      ((unsigned long long)a.T * a.defer_w + 31) >> 5;
  const unsigned long long n_warps =
      (unsigned long long)gridDim.x * kFixWarps;
  unsigned long long *q = s_q[warp];
  int qn = 0;  // queued bits (warp-uniform)
  for (unsigned long long base =
           ((unsigned long long)blockIdx.x * kFixWarps + warp) * 32;
       base < n_words; base += n_warps * 32) {
    const unsigned long long w = base + lane;
    unsigned int m = w < n_words ? a.defer_mask[w] : 0u;
    const int c = __popc(m);
    int incl = c;
    for (int d = 1; d < 32; d <<= 1) {
      const int v = __shfl_up_sync(0xffffffffu, incl, d);
      if (lane >= d) incl += v;
    }
    const int total = __shfl_sync(0xffffffffu, incl, 31);
    int pos = qn + incl - c;
    while (m) {
      const int b = __ffs(m) - 1;
      m &= m - 1;
      q[pos++] = (w << 5) + b;
    }
    __syncwarp();
    qn += total;
    while (qn >= 32) {
      const unsigned long long bit = q[qn - 32 + lane];
      __syncwarp();
      fixup_pair<NI, ROUGH>(a, k, bit, s_pat, pa_len, lg, s_fad);
      qn -= 32;
    }
    __syncwarp();
  }
  if (lane < qn) fixup_pair<NI, ROUGH>(a, k, q[lane], s_pat, pa_len, lg, s_fad);
}

template <int NI, int ROUGH, bool PLAIN>
inline cudaError_t launch_fast(RefArgs &a, const RefSplitConsts &k,
                               const Plan &p, size_t smem, cudaStream_t st) {
  cudaError_t e = cudaFuncSetAttribute(
      refracted_split_kernel<NI, ROUGH, PLAIN>,
      cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  dim3 grid(p.n_chunks, p.n_groups);
  refracted_split_kernel<NI, ROUGH, PLAIN><<<grid, p.threads, smem, st>>>(a,
                                                                         k);
  return cudaGetLastError();
}

template <int NI, int ROUGH>
inline int launch_split(RefArgs &a, const RefSplitConsts &k, const Plan &p,
                        size_t smem, cudaStream_t st) {
  const unsigned long long n_words =
      ((unsigned long long)a.T * a.defer_w + 31) >> 5;
  cudaError_t e =
      cudaMemsetAsync(a.defer_mask, 0, n_words * sizeof(uint32_t), st);
  if (e != cudaSuccess) return cuda_status(e, "deferral mask clear");
  // compile-time plain form (isotropic antenna, no taper, no diffuse
  // channel, no side split) for smooth targets: less code, fewer registers
  const bool plain = ROUGH == SS_ROUGH_NONE &&
                     a.pat_kind == SS_PAT_ISOTROPIC && !a.taper &&
                     !a.F.diffuse_amp && !a.split;
  e = plain ? launch_fast<NI, ROUGH, ROUGH == SS_ROUGH_NONE>(a, k, p, smem,
                                                              st)
            : launch_fast<NI, ROUGH, false>(a, k, p, smem, st);
  if (e != cudaSuccess) return cuda_status(e, "refracted_split launch");
  const size_t fsmem =
      a.rough_kind ? (size_t)(a.n_terms + 1) * sizeof(float) : 0;
  const unsigned long long want = (n_words + 32 * kFixWarps - 1) /
                                  (32 * kFixWarps);
  const int blocks =
      (int)std::max<unsigned long long>(1, std::min<unsigned long long>(
                                               want, 8ull * sm_count()));
  refracted_split_fixup<NI, ROUGH><<<blocks, 32 * kFixWarps, fsmem, st>>>(a,
                                                                          k);
  return cuda_status(cudaGetLastError(), "refracted_split fix-up launch");
}

template <int NI>
inline int launch_split_r(RefArgs &a, const RefSplitConsts &k, const Plan &p,
                          size_t smem, cudaStream_t st) {
  switch (a.rough_kind) {
    case SS_ROUGH_NONE: return launch_split<NI, SS_ROUGH_NONE>(a, k, p, smem, st);
    case SS_ROUGH_GAUSS_FULL:
      return launch_split<NI, SS_ROUGH_GAUSS_FULL>(a, k, p, smem, st);
    case SS_ROUGH_GAUSS_AREA:
      return launch_split<NI, SS_ROUGH_GAUSS_AREA>(a, k, p, smem, st);
    default: return launch_split<NI, SS_ROUGH_EXP_AREA>(a, k, p, smem, st);
  }
}

// ---------------------------------------------------------------------
// batched refracted targets: one persistent work-queue launch for many
// jobs of one path class (crossed-interface count), roughness kind and
// form, then one batched fix-up and one batched reduce
// ---------------------------------------------------------------------
struct RefBatchJob {
  RefArgs a;
  RefSplitConsts k;
  long long item0;  // first work item (trace block x facet chunk)
  long long out0;   // first reduce element (trace x segment)
  long long word0;  // first deferral-mask word (multiple of 32)
  long long words;  // this job's mask words
  int n_chunks, n_groups;
  ss_output out;
};

// Index of the job owning position `x` of a prefix field (first <= x).
template <int FIELD>
__device__ __forceinline__ int ref_batch_find(const RefBatchJob *jobs,
                                              int n_jobs, long long x) {
  int lo = 0, hi = n_jobs - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    const long long f = FIELD == 0 ? jobs[mid].item0
                                   : FIELD == 1 ? jobs[mid].out0
                                                : jobs[mid].word0;
    if (f <= x) lo = mid; else hi = mid - 1;
  }
  return lo;
}

template <int NI, int ROUGH, bool PLAIN>
__global__ void __launch_bounds__(kSplitThreads, NI >= 3 ? 1 : 2)
refracted_batch_kernel(const RefBatchJob *jobs, int n_jobs,
                       long long n_items, unsigned long long *counter) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ long long s_item;
  __shared__ int s_job;
  for (;;) {
    __syncthreads();  // the previous item's shared memory is free
    if (threadIdx.x == 0) {
      const long long it = (long long)atomicAdd(counter, 1ull);
      s_item = it;
      s_job = it < n_items ? ref_batch_find<0>(jobs, n_jobs, it) : 0;
    }
    __syncthreads();
    const long long it = s_item;
    if (it >= n_items) break;
    const RefBatchJob &J = jobs[s_job];
    const long long local = it - J.item0;
    refracted_split_cta<NI, ROUGH, PLAIN>(J.a, J.k,
                                          (int)(local % J.n_chunks),
                                          (int)(local / J.n_chunks),
                                          smem_raw);
  }
}

// Batched fix-up: the jobs' masks are laid end to end in 32-word groups,
// so each warp's 32-word scan belongs to one job; queued bits carry their
// job. The jobs share one antenna table (staged once).
template <int NI, int ROUGH>
__global__ void __launch_bounds__(32 * kFixWarps, 4)
refracted_batch_fixup(const RefBatchJob *jobs, int n_jobs,
                      long long n_words) {
  // the jobs' series lengths differ: no 1/m table (the series divides)
  const float *lg = nullptr;
  __shared__ float s_pat[SS_PAT_MAX];
  __shared__ float s_fad[SS_FAD_N];
  __shared__ unsigned long long s_q[kFixWarps][kFixQueue];
  __shared__ int s_qj[kFixWarps][kFixQueue];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const RefArgs &a0 = jobs[0].a;
  int pa_len, pb_len;
  pattern_lengths(a0.pat_kind, a0.pat_n, pa_len, pb_len);
  for (int j = tid; j < pa_len; j += blockDim.x) s_pat[j] = (float)a0.pa[j];
  for (int j = tid; j < pb_len; j += blockDim.x)
    s_pat[pa_len + j] = (float)a0.pb[j];
  if (ROUGH == SS_ROUGH_GAUSS_FULL && tid < SS_FAD_N)
    s_fad[tid] = (float)a0.fad.a[tid];
  __syncthreads();
  const unsigned long long n_warps =
      (unsigned long long)gridDim.x * kFixWarps;
  unsigned long long *q = s_q[warp];
  int *qj = s_qj[warp];
  int qn = 0;
  auto eval = [&](unsigned long long bit, int jb) {
    const RefBatchJob &J = jobs[jb];
    fixup_pair<NI, ROUGH>(J.a, J.k, bit, s_pat, pa_len, lg, s_fad);
  };
  for (unsigned long long base =
           ((unsigned long long)blockIdx.x * kFixWarps + warp) * 32;
       base < (unsigned long long)n_words; base += n_warps * 32) {
    const int jb = ref_batch_find<2>(jobs, n_jobs, (long long)base);
    const RefBatchJob &J = jobs[jb];
    const long long lw = (long long)base - J.word0 + lane;
    unsigned int m = lw < J.words ? J.a.defer_mask[lw] : 0u;
    const int c = __popc(m);
    int incl = c;
    for (int d = 1; d < 32; d <<= 1) {
      const int v = __shfl_up_sync(0xffffffffu, incl, d);
      if (lane >= d) incl += v;
    }
    const int total = __shfl_sync(0xffffffffu, incl, 31);
    int pos = qn + incl - c;
    while (m) {
      const int b = __ffs(m) - 1;
      m &= m - 1;
      qj[pos] = jb;
      q[pos++] = ((unsigned long long)lw << 5) + b;
    }
    __syncwarp();
    qn += total;
    while (qn >= 32) {
      const unsigned long long bit = q[qn - 32 + lane];
      const int jq = qj[qn - 32 + lane];
      __syncwarp();
      eval(bit, jq);
      qn -= 32;
    }
    __syncwarp();
  }
  if (lane < qn) eval(q[lane], qj[lane]);
}

// Persistent pass and fix-up of one path class (NI = 0: sequential).
#define SS_REF_BATCH_DECL(N)                                                \
  int refracted_batch_launch_ni##N(                                         \
      const RefBatchJob *jobs, int n_jobs, long long n_items,              \
      long long n_words, unsigned long long *counter, int rough_kind,      \
      bool plain, int ctas, size_t smem, size_t fix_smem, cudaStream_t st); \
  int refracted_batch_occupancy_ni##N(int rough_kind, bool plain,          \
                                      size_t smem);
SS_REF_BATCH_DECL(0)
SS_REF_BATCH_DECL(1)
SS_REF_BATCH_DECL(2)
SS_REF_BATCH_DECL(3)
SS_REF_BATCH_DECL(4)
#undef SS_REF_BATCH_DECL

// Launch helpers instantiated in each path class's translation unit.
template <int NI, int ROUGH, bool PLAIN>
inline int ref_batch_launch_t(const RefBatchJob *jobs, int n_jobs,
                              long long n_items, long long n_words,
                              unsigned long long *counter, int ctas,
                              size_t smem, size_t fix_smem,
                              cudaStream_t st) {
  refracted_batch_kernel<NI, ROUGH, PLAIN><<<ctas, kSplitThreads, smem, st>>>(
      jobs, n_jobs, n_items, counter);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_status(e, "refracted batch launch");
  const unsigned long long want =
      ((unsigned long long)n_words + 32 * kFixWarps - 1) / (32 * kFixWarps);
  const int blocks = (int)std::max<unsigned long long>(
      1, std::min<unsigned long long>(want, 8ull * sm_count()));
  refracted_batch_fixup<NI, ROUGH><<<blocks, 32 * kFixWarps, fix_smem, st>>>(
      jobs, n_jobs, n_words);
  return cuda_status(cudaGetLastError(), "refracted batch fix-up launch");
}

template <int NI>
inline int ref_batch_launch_r(const RefBatchJob *jobs, int n_jobs,
                              long long n_items, long long n_words,
                              unsigned long long *counter, int rough_kind,
                              bool plain, int ctas, size_t smem,
                              size_t fix_smem, cudaStream_t st) {
  switch (rough_kind) {
    case SS_ROUGH_NONE:
      return plain ? ref_batch_launch_t<NI, SS_ROUGH_NONE, true>(
                         jobs, n_jobs, n_items, n_words, counter, ctas, smem,
                         fix_smem, st)
                   : ref_batch_launch_t<NI, SS_ROUGH_NONE, false>(
                         jobs, n_jobs, n_items, n_words, counter, ctas, smem,
                         fix_smem, st);
    case SS_ROUGH_GAUSS_FULL:
      return ref_batch_launch_t<NI, SS_ROUGH_GAUSS_FULL, false>(
          jobs, n_jobs, n_items, n_words, counter, ctas, smem, fix_smem, st);
    case SS_ROUGH_GAUSS_AREA:
      return ref_batch_launch_t<NI, SS_ROUGH_GAUSS_AREA, false>(
          jobs, n_jobs, n_items, n_words, counter, ctas, smem, fix_smem, st);
    default:
      return ref_batch_launch_t<NI, SS_ROUGH_EXP_AREA, false>(
          jobs, n_jobs, n_items, n_words, counter, ctas, smem, fix_smem, st);
  }
}

template <int NI>
inline int ref_batch_occupancy(int rough_kind, bool plain, size_t smem) {
  int n = 0;
  cudaError_t e = cudaSuccess;
  auto one = [&](auto kern) {
    e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)smem);
    if (e == cudaSuccess)
      e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, kern,
                                                        kSplitThreads, smem);
  };
  switch (rough_kind) {
    case SS_ROUGH_NONE:
      if (plain) one(refracted_batch_kernel<NI, SS_ROUGH_NONE, true>);
      else one(refracted_batch_kernel<NI, SS_ROUGH_NONE, false>);
      break;
    case SS_ROUGH_GAUSS_FULL:
      one(refracted_batch_kernel<NI, SS_ROUGH_GAUSS_FULL, false>);
      break;
    case SS_ROUGH_GAUSS_AREA:
      one(refracted_batch_kernel<NI, SS_ROUGH_GAUSS_AREA, false>);
      break;
    default:
      one(refracted_batch_kernel<NI, SS_ROUGH_EXP_AREA, false>);
  }
  return e == cudaSuccess ? n : 0;
}

// float32 / double-float constants of the split kernels.
RefSplitConsts split_consts(const RefArgs &a);
// Dynamic shared memory of the fast kernel for a trace block of tb.
size_t split_smem_bytes(const RefArgs &a, int tb);

// Fast + fix-up launches of one crossed-interface count (NI = 0: the
// sequential path), each instantiated in its own translation unit.
int split_launch_ni0(RefArgs &a, const RefSplitConsts &k, const Plan &p,
                     size_t smem, cudaStream_t st);
int split_launch_ni1(RefArgs &a, const RefSplitConsts &k, const Plan &p,
                     size_t smem, cudaStream_t st);
int split_launch_ni2(RefArgs &a, const RefSplitConsts &k, const Plan &p,
                     size_t smem, cudaStream_t st);
int split_launch_ni3(RefArgs &a, const RefSplitConsts &k, const Plan &p,
                     size_t smem, cudaStream_t st);
int split_launch_ni4(RefArgs &a, const RefSplitConsts &k, const Plan &p,
                     size_t smem, cudaStream_t st);
// Joint solve through 5..SS_MAX_IFACE interfaces: one instantiation whose
// arrays hold SS_MAX_IFACE interfaces (in local memory).
int split_launch_deep(RefArgs &a, const RefSplitConsts &k, const Plan &p,
                      size_t smem, cudaStream_t st);

}  // namespace ss
