// Split-precision refracted multilayer kernel.
//
// The float64 form spends nearly all its time in fixed-budget Newton
// iterations (10 + 25 per crossing, or the joint solve's 6 damped steps of
// block-Thomas plus step halving), on GB300 whose FP64 rate is a small
// fraction of its FP32 rate. This form keeps float64 only where the result
// needs it and runs the iterations in float32:
//
//   * facet lookups: the mean-plane crossing is solved in float32 in
//     plane-relative coordinates; if the affine cell coordinate lies within
//     1e-3 cells of a rounding boundary (the float32 crossing error is
//     ~4e-5 cells) the float64 mean-plane solve of the reference is re-run
//     for that pair, so lookups are the reference's integer decisions;
//   * the local-plane two-point solve: float64 geometry (heights, feet,
//     scale) around float32 Newton iterations; the crossing offset t comes
//     from the float32 root and the path lengths are evaluated in float64 at
//     that t -- the optical path is stationary in t (Fermat), so the float32
//     root error enters only at second order;
//   * the joint solve: float32 damped Newton on in-plane offsets measured
//     from each local plane's facet centre (segments are formed from float64
//     centre differences, so float32 keeps ~1e-7 of each segment), then
//     float64 segment lengths; again second order in the root error;
//   * optical path, carrier phase reduction and fast-time bin in float64; a
//     pair within 1e-6 of a bin edge is re-evaluated with the complete
//     float64 path, so bins equal the float64 form's;
//   * everything radiometric (Fresnel, spreading, attenuation, antenna gain,
//     sinc at k_j, roughness series, diffuse channel) in float32.
//
// Validity: same-side/shadow tests use the float64 heights; convergence uses
// the float32 Snell residual with tolerance 1e-4 (the float32 floor is
// ~1e-6; failed solves sit at O(0.1)).
#include "ss_df.cuh"
#include "ss_f32.cuh"
#include "ss_refracted_fp64.cuh"

namespace ss {

constexpr float kTiny32 = 1e-30f;
constexpr float kEps32 = 1.1920929e-07f;
constexpr float kTol32 = 1e-4f;
constexpr double kLookupGuard = 1e-3;
constexpr float kBinGuard = 1e-6f;

struct RefSplitConsts {
  float k0, amp_pref_j, kj, taper_inv, sigma, corr, fadL, n_exp;
  float n_leg[SS_MAX_IFACE + 1], eps_leg[SS_MAX_IFACE + 1],
      att_leg[SS_MAX_IFACE + 1], sig_c[SS_MAX_IFACE];
};

__device__ __forceinline__ float dot3a(const float *a, const float *b) {
  return __fmaf_rn(a[2], b[2], __fmaf_rn(a[1], b[1], a[0] * b[0]));
}

// float32 safeguarded Newton on sigma = sin(theta_rare) (the reference's
// update, refraction.py:120-144), stopping early once the step is below
// float32 resolution.
__device__ __forceinline__ float sigma32(float ar, float bd, float Lh,
                                         float ah, float bh, float ratio,
                                         int n_iter) {
  const float hi0 = 1.0f - 8.0f * kEps32;
  float sig = fminf(Lh / fmaxf(sqrtf(Lh * Lh + (ah + bh) * (ah + bh)),
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

// float32 two-point solve with both endpoints given relative to the plane
// point: returns the crossing offset from the plane point.
__device__ __forceinline__ void snell32_rel(const float *P, const float *Q,
                                            const float *nrm, float n1,
                                            float n2, int n_iter, float *y) {
  const float h1 = dot3a(P, nrm), h2 = dot3a(Q, nrm);
  const float a = fabsf(h1), b = fabsf(h2);
  float fp[3], w[3];
  for (int j = 0; j < 3; ++j) {
    fp[j] = P[j] - h1 * nrm[j];
    w[j] = (Q[j] - h2 * nrm[j]) - fp[j];
  }
  const float L = sqrtf(dot3a(w, w));
  const float Lm = fmaxf(L, kTiny32);
  const float s = fmaxf(a + b + L, kTiny32);
  const float inv_s = 1.0f / s;
  const float ah = a * inv_s, bh = b * inv_s, Lh = L * inv_s;
  const bool swap = n1 > n2;
  const float ratio = fminf(n1, n2) / fmaxf(n1, n2);
  const float ar = swap ? bh : ah, bd = swap ? ah : bh;
  const float sig = sigma32(ar, bd, Lh, ah, bh, ratio, n_iter);
  const float c1 = fmaxf((1.0f - sig) * (1.0f + sig), kTiny32);
  const float tr = ar * sig * rsqrtf(c1);
  const float t = fminf(fmaxf(swap ? Lh - tr : tr, 0.0f), Lh);
  const float st = s * t / Lm;
  for (int j = 0; j < 3; ++j) y[j] = fp[j] + st * w[j];
}

// Local-plane two-point solve: float64 heights/feet/scale, float32 root,
// float64 crossing and leg lengths at that root.
struct LocalSolve {
  double x[3];       // crossing (float64)
  double s1;         // |cur - x|
  double s2;         // |x - q|
  float c1, c2;      // cos(theta1), cos(theta2)
  bool valid;
};

__device__ __forceinline__ void snell_local(const double *cur, const double *q,
                                            const double *o, const double *nrm,
                                            double n1, double n2, int n_iter,
                                            LocalSolve &R) {
  double po[3] = {cur[0] - o[0], cur[1] - o[1], cur[2] - o[2]};
  double qo[3] = {q[0] - o[0], q[1] - o[1], q[2] - o[2]};
  const double h1 = dot3v(po, nrm), h2 = dot3v(qo, nrm);
  const double a = fabs(h1), b = fabs(h2);
  double fp[3], w[3];
  for (int j = 0; j < 3; ++j) {
    fp[j] = cur[j] - h1 * nrm[j];
    w[j] = (q[j] - h2 * nrm[j]) - fp[j];
  }
  const double L = sqrt(dot3v(w, w));
  const double s = fmax(a + b + L, kTiny);
  const double inv_s = 1.0 / s;
  const double ah = a * inv_s, bh = b * inv_s, Lh = L * inv_s;
  const bool swap = n1 > n2;
  const float ratio = (float)(fmin(n1, n2) / fmax(n1, n2));
  const float ah32 = (float)ah, bh32 = (float)bh, Lh32 = (float)Lh;
  const float ar32 = swap ? bh32 : ah32, bd32 = swap ? ah32 : bh32;
  const float sig32 = sigma32(ar32, bd32, Lh32, ah32, bh32, ratio, n_iter);
  // one float64 Newton step from the float32 root: the crossing enters the
  // facet's arrival direction (and so the sinc arguments) at first order
  const double ar = swap ? bh : ah, bd = swap ? ah : bh;
  const double ratio64 = fmin(n1, n2) / fmax(n1, n2);
  double sg = (double)sig32;
  {
    const double v = ratio64 * sg;
    const double r1i = rsqrt(fmax((1.0 - sg) * (1.0 + sg), kTiny));
    const double r2i = rsqrt(fmax((1.0 - v) * (1.0 + v), kTiny));
    const double F = (ar * sg * r1i + bd * v * r2i) - Lh;
    const double Fp = ar * r1i * r1i * r1i + bd * ratio64 * r2i * r2i * r2i;
    const double sn = sg - F / fmax(Fp, kTiny);
    if (isfinite(sn) && sn >= 0.0 && sn < 1.0) sg = sn;
  }
  const double tr = ar * sg * rsqrt(fmax((1.0 - sg) * (1.0 + sg), kTiny));
  const double t = fmin(fmax(swap ? Lh - tr : tr, 0.0), Lh);
  const double d2 = Lh - t;
  const double r1 = fmax(sqrt(ah * ah + t * t), kTiny);
  const double r2 = fmax(sqrt(bh * bh + d2 * d2), kTiny);
  R.s1 = s * r1;
  R.s2 = s * r2;
  const double stl = s * t / fmax(L, kTiny);
  for (int j = 0; j < 3; ++j) R.x[j] = fp[j] + stl * w[j];
  R.c1 = (float)(ah / r1);
  R.c2 = (float)(bh / r2);
  const float res = (float)n1 * (float)(t / r1) - (float)n2 * (float)(d2 / r2);
  R.valid = (h1 * h2 < 0.0) && (fabsf(res) <= kTol32);
}

// Mean-plane crossing in float32 relative to the mean point, then the
// affine cell coordinate; returns false when either coordinate is within
// the guard band of a rounding boundary.
__device__ __forceinline__ bool mean_lookup32(const ss_interface &I,
                                              const double *cur,
                                              const double *q, float n1,
                                              float n2, int n_iter, int &row,
                                              int &col) {
  const float P[3] = {(float)(cur[0] - I.mean_point[0]),
                      (float)(cur[1] - I.mean_point[1]),
                      (float)(cur[2] - I.mean_point[2])};
  const float Q[3] = {(float)(q[0] - I.mean_point[0]),
                      (float)(q[1] - I.mean_point[1]),
                      (float)(q[2] - I.mean_point[2])};
  const float nrm[3] = {(float)I.mean_normal[0], (float)I.mean_normal[1],
                        (float)I.mean_normal[2]};
  float y[3];
  snell32_rel(P, Q, nrm, n1, n2, n_iter, y);
  const double b0 = I.mean_point[0] * I.coef[0] + I.mean_point[1] * I.coef[2] +
                    I.coef[4];
  const double b1 = I.mean_point[0] * I.coef[1] + I.mean_point[1] * I.coef[3] +
                    I.coef[5];
  const double rc0 = b0 + (double)(y[0] * (float)I.coef[0] +
                                   y[1] * (float)I.coef[2]);
  const double rc1 = b1 + (double)(y[0] * (float)I.coef[1] +
                                   y[1] * (float)I.coef[3]);
  const double f0 = rc0 - floor(rc0), f1 = rc1 - floor(rc1);
  const bool safe = fabs(f0 - 0.5) > kLookupGuard &&
                    fabs(f1 - 0.5) > kLookupGuard;
  row = (int)fmin(fmax(rint(rc0), 0.0), (double)(I.ny - 1));
  col = (int)fmin(fmax(rint(rc1), 0.0), (double)(I.nx - 1));
  return safe;
}

__device__ __forceinline__ void cell_plane(const ss_interface &I, int row,
                                           int col, double *pt, double *nr) {
  const float *g = I.table + ((size_t)row * I.nx + col) * 6;
  for (int j = 0; j < 3; ++j) {
    pt[j] = (double)g[j];
    nr[j] = (double)g[3 + j];
  }
}

__device__ __forceinline__ float fresnel_gamma32(float e1, float e2,
                                                 float c1) {
  const float n1 = sqrtf(e1), n2 = sqrtf(e2);
  const float s2 = (e1 / e2) * (1.0f - c1 * c1);
  const float c2 = sqrtf(fmaxf(1.0f - s2, 0.0f));
  return (n1 * c1 - n2 * c2) / (n1 * c1 + n2 * c2);
}

struct PathS {
  double cur[3], xf[3];
  double opl;
  float loss_db, sum_par, sum_perp, tau2, c0, c_last;
  bool valid;
};

__device__ void path_sequential_split(const RefArgs &a,
                                      const RefSplitConsts &k,
                                      const double *p, const double *q,
                                      PathS &P) {
  double cur[3] = {p[0], p[1], p[2]};
  P.valid = true;
  P.opl = 0.0;
  P.loss_db = P.sum_par = P.sum_perp = 0.0f;
  P.tau2 = 1.0f;
  P.c0 = P.c_last = 1.0f;
  for (int i = 0; i < a.ni; ++i) {
    const ss_interface &I = a.ifc[i];
    int row, col;
    if (!mean_lookup32(I, cur, q, k.n_leg[i], k.n_leg[i + 1], 10, row,
                       col)) {
      Snell64 R1;  // exact reference decision near a rounding boundary
      snell64(cur, q, I.mean_point, I.mean_normal, a.n_leg[i],
              a.n_leg[i + 1], 10, true, R1);
      double pt[3], nr[3];
      lookup64(I, R1.x, pt, nr);
      const double rc0 = __dadd_rn(__dadd_rn(__dmul_rn(R1.x[0], I.coef[0]),
                                             __dmul_rn(R1.x[1], I.coef[2])),
                                   I.coef[4]);
      const double rc1 = __dadd_rn(__dadd_rn(__dmul_rn(R1.x[0], I.coef[1]),
                                             __dmul_rn(R1.x[1], I.coef[3])),
                                   I.coef[5]);
      row = (int)fmin(fmax(rint(rc0), 0.0), (double)(I.ny - 1));
      col = (int)fmin(fmax(rint(rc1), 0.0), (double)(I.nx - 1));
    }
    double pt[3], nr[3];
    cell_plane(I, row, col, pt, nr);
    const double inn = 1.0 / sqrt(dot3v(nr, nr));
    for (int j = 0; j < 3; ++j) nr[j] *= inn;
    LocalSolve R;
    snell_local(cur, q, pt, nr, a.n_leg[i], a.n_leg[i + 1], 25, R);
    P.valid = P.valid && R.valid;
    const float c_inc = fmaxf(R.c1, (float)kCMin);
    if (i == 0) {
      P.c0 = c_inc;
      for (int j = 0; j < 3; ++j) P.xf[j] = R.x[j];
    }
    const float g = fresnel_gamma32(k.eps_leg[i], k.eps_leg[i + 1], c_inc);
    P.tau2 *= (1.0f - g * g);
    if (a.rough_cross) {
      const float kt = k.k0 * (k.n_leg[i] * c_inc - k.n_leg[i + 1] * R.c2);
      const float sk = k.sig_c[i] * kt;
      P.tau2 *= __expf(-2.0f * sk * sk);
    }
    const float s1f = (float)R.s1;
    P.opl += a.n_leg[i] * R.s1;
    P.loss_db += s1f * (k.att_leg[i] * 1e-3f);
    P.sum_perp += s1f / k.n_leg[i];
    P.sum_par += s1f / (k.n_leg[i] * c_inc * c_inc);
    P.c_last = fmaxf(R.c2, (float)kCMin);
    for (int j = 0; j < 3; ++j) cur[j] = R.x[j];
  }
  for (int j = 0; j < 3; ++j) P.cur[j] = cur[j];
  double d[3] = {cur[0] - q[0], cur[1] - q[1], cur[2] - q[2]};
  (void)d;
}

// float32 joint solve on in-plane offsets from the local facet centres.
template <int NI>
__device__ void path_joint_split(const RefArgs &a, const RefSplitConsts &k,
                                 const double *p, const double *q,
                                 PathS &P) {
  // pass 1: mean-plane chain anchors the lookups (float32 + exact fallback)
  int rows[NI], cols[NI];
  {
    double cur[3] = {p[0], p[1], p[2]};
    bool safe = true;
    for (int i = 0; i < NI; ++i) {
      const ss_interface &I = a.ifc[i];
      const float Pr[3] = {(float)(cur[0] - I.mean_point[0]),
                           (float)(cur[1] - I.mean_point[1]),
                           (float)(cur[2] - I.mean_point[2])};
      const float Qr[3] = {(float)(q[0] - I.mean_point[0]),
                           (float)(q[1] - I.mean_point[1]),
                           (float)(q[2] - I.mean_point[2])};
      const float nrm[3] = {(float)I.mean_normal[0], (float)I.mean_normal[1],
                            (float)I.mean_normal[2]};
      float y[3];
      snell32_rel(Pr, Qr, nrm, k.n_leg[i], k.n_leg[i + 1], 10, y);
      for (int j = 0; j < 3; ++j) cur[j] = I.mean_point[j] + (double)y[j];
      const double rc0 = cur[0] * I.coef[0] + cur[1] * I.coef[2] + I.coef[4];
      const double rc1 = cur[0] * I.coef[1] + cur[1] * I.coef[3] + I.coef[5];
      const double f0 = rc0 - floor(rc0), f1 = rc1 - floor(rc1);
      safe = safe && fabs(f0 - 0.5) > kLookupGuard &&
             fabs(f1 - 0.5) > kLookupGuard;
      rows[i] = (int)fmin(fmax(rint(rc0), 0.0), (double)(I.ny - 1));
      cols[i] = (int)fmin(fmax(rint(rc1), 0.0), (double)(I.nx - 1));
    }
    if (!safe) {  // exact reference chain for this pair
      double c64[3] = {p[0], p[1], p[2]};
      for (int i = 0; i < NI; ++i) {
        const ss_interface &I = a.ifc[i];
        Snell64 R;
        snell64(c64, q, I.mean_point, I.mean_normal, a.n_leg[i],
                a.n_leg[i + 1], 10, false, R);
        for (int j = 0; j < 3; ++j) c64[j] = R.x[j];
        const double rc0 = __dadd_rn(__dadd_rn(__dmul_rn(R.x[0], I.coef[0]),
                                               __dmul_rn(R.x[1], I.coef[2])),
                                     I.coef[4]);
        const double rc1 = __dadd_rn(__dadd_rn(__dmul_rn(R.x[0], I.coef[1]),
                                               __dmul_rn(R.x[1], I.coef[3])),
                                     I.coef[5]);
        rows[i] = (int)fmin(fmax(rint(rc0), 0.0), (double)(I.ny - 1));
        cols[i] = (int)fmin(fmax(rint(rc1), 0.0), (double)(I.nx - 1));
      }
    }
  }
  // local planes: float64 centres, float32 unit normals
  double O[NI][3], N64[NI][3];
  float Nn[NI][3];
  for (int i = 0; i < NI; ++i) {
    double nr[3];
    cell_plane(a.ifc[i], rows[i], cols[i], O[i], nr);
    const double nn = sqrt(dot3v(nr, nr));
    for (int j = 0; j < 3; ++j) {
      N64[i][j] = nr[j] / nn;
      Nn[i][j] = (float)N64[i][j];
    }
  }
  // segment bases: D_0 = o_0 - p, D_k = o_k - o_{k-1}, D_NI = q - o_{NI-1}
  double D64[NI + 1][3];
  for (int j = 0; j < 3; ++j) {
    D64[0][j] = O[0][j] - p[j];
    for (int i = 1; i < NI; ++i) D64[i][j] = O[i][j] - O[i - 1][j];
    D64[NI][j] = q[j] - O[NI - 1][j];
  }
  double pq[3] = {p[0] - q[0], p[1] - q[1], p[2] - q[2]};
  const float scale = (float)fmax(sqrt(dot3v(pq, pq)), kTiny);
  const float inv = 1.0f / scale;
  float Ds[NI + 1][3];
  for (int i = 0; i <= NI; ++i)
    for (int j = 0; j < 3; ++j) Ds[i][j] = (float)D64[i][j] * inv;
  const float *nm = k.n_leg;
  // chain initialiser (25 iterations), offsets y_i from o_i (scaled units)
  float Y[NI][3];
  {
    float Qrel[NI][3];  // q - o_i = sum_{j > i} D_j
    for (int j = 0; j < 3; ++j) {
      float acc = Ds[NI][j];
      for (int i = NI - 1; i >= 0; --i) {
        Qrel[i][j] = acc;
        acc += Ds[i][j];
      }
    }
    for (int i = 0; i < NI; ++i) {
      float Pr[3];
      for (int j = 0; j < 3; ++j)
        Pr[j] = i == 0 ? -Ds[0][j] : Y[i - 1][j] - Ds[i][j];
      snell32_rel(Pr, Qrel[i], Nn[i], nm[i], nm[i + 1], 25, Y[i]);
    }
  }
  // in-plane bases and offsets
  float B[NI][3][2], ab[NI][2];
  for (int i = 0; i < NI; ++i) {
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
  const float mu = 6.4e-6f;  // Levenberg shift, float32 eps^0.75
  float s[NI + 1], dh[NI + 1][3], f[NI][2];
  auto geom = [&](const float (&abv)[NI][2], float (&sv)[NI + 1],
                  float (&dv)[NI + 1][3], float (&fv)[NI][2]) {
    float y[NI][3];
    for (int i = 0; i < NI; ++i)
      for (int j = 0; j < 3; ++j)
        y[i][j] = B[i][j][0] * abv[i][0] + B[i][j][1] * abv[i][1];
    float g[NI + 1][3];
    for (int kk = 0; kk <= NI; ++kk) {
      float d[3];
      for (int j = 0; j < 3; ++j)
        d[j] = Ds[kk][j] + (kk < NI ? y[kk][j] : 0.0f) -
               (kk > 0 ? y[kk - 1][j] : 0.0f);
      const float ss = fmaxf(sqrtf(dot3a(d, d)), kTiny32);
      sv[kk] = ss;
      const float is = 1.0f / ss;
      for (int j = 0; j < 3; ++j) {
        dv[kk][j] = d[j] * is;
        g[kk][j] = nm[kk] * dv[kk][j];
      }
    }
    for (int i = 0; i < NI; ++i)
      for (int c = 0; c < 2; ++c)
        fv[i][c] = B[i][0][c] * (g[i][0] - g[i + 1][0]) +
                   B[i][1][c] * (g[i][1] - g[i + 1][1]) +
                   B[i][2][c] * (g[i][2] - g[i + 1][2]);
  };
  float dinv[NI][2][2], Cm[NI > 1 ? NI - 1 : 1][2][2];
  // block-Thomas solve with the current factorisation (dinv, Cm)
  auto thomas = [&](const float (&rhs_in)[NI][2], float (&delta)[NI][2]) {
    float yv[NI][2];
    for (int i = 0; i < NI; ++i) {
      float rhs[2] = {rhs_in[i][0], rhs_in[i][1]};
      if (i > 0) {
        float cpt[2][2];
        for (int r = 0; r < 2; ++r)
          for (int c = 0; c < 2; ++c)
            cpt[r][c] = Cm[i - 1][0][r] * dinv[i - 1][0][c] +
                        Cm[i - 1][1][r] * dinv[i - 1][1][c];
        for (int r = 0; r < 2; ++r)
          rhs[r] -= cpt[r][0] * yv[i - 1][0] + cpt[r][1] * yv[i - 1][1];
      }
      yv[i][0] = rhs[0];
      yv[i][1] = rhs[1];
    }
    for (int i = NI - 1; i >= 0; --i) {
      float rr[2] = {yv[i][0], yv[i][1]};
      if (i < NI - 1)
        for (int r = 0; r < 2; ++r)
          rr[r] -= Cm[i][r][0] * delta[i + 1][0] + Cm[i][r][1] * delta[i + 1][1];
      for (int r = 0; r < 2; ++r)
        delta[i][r] = dinv[i][r][0] * rr[0] + dinv[i][r][1] * rr[1];
    }
  };
  for (int it = 0; it < a.n_newton; ++it) {
    geom(ab, s, dh, f);
    float W[NI + 1][3][3];
    for (int kk = 0; kk <= NI; ++kk) {
      const float sc = nm[kk] / s[kk];
      for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c)
          W[kk][r][c] = sc * ((r == c ? 1.0f : 0.0f) - dh[kk][r] * dh[kk][c]);
    }
    float A[NI][2][2];
    for (int i = 0; i < NI; ++i) {
      float BW[2][3];
      for (int r = 0; r < 2; ++r)
        for (int l = 0; l < 3; ++l)
          BW[r][l] = B[i][0][r] * (W[i][0][l] + W[i + 1][0][l]) +
                     B[i][1][r] * (W[i][1][l] + W[i + 1][1][l]) +
                     B[i][2][r] * (W[i][2][l] + W[i + 1][2][l]);
      for (int r = 0; r < 2; ++r)
        for (int c = 0; c < 2; ++c)
          A[i][r][c] = BW[r][0] * B[i][0][c] + BW[r][1] * B[i][1][c] +
                       BW[r][2] * B[i][2][c] + (r == c ? mu : 0.0f);
    }
    for (int i = 0; i + 1 < NI; ++i) {
      float BW[2][3];
      for (int r = 0; r < 2; ++r)
        for (int l = 0; l < 3; ++l)
          BW[r][l] = B[i][0][r] * W[i + 1][0][l] + B[i][1][r] * W[i + 1][1][l] +
                     B[i][2][r] * W[i + 1][2][l];
      for (int r = 0; r < 2; ++r)
        for (int c = 0; c < 2; ++c)
          Cm[i][r][c] = -(BW[r][0] * B[i + 1][0][c] +
                          BW[r][1] * B[i + 1][1][c] +
                          BW[r][2] * B[i + 1][2][c]);
    }
    // factor: dinv_i = (A_i - C_{i-1}^T dinv_{i-1} C_{i-1})^-1
    for (int i = 0; i < NI; ++i) {
      float M[2][2] = {{A[i][0][0], A[i][0][1]}, {A[i][1][0], A[i][1][1]}};
      if (i > 0) {
        float cpt[2][2];
        for (int r = 0; r < 2; ++r)
          for (int c = 0; c < 2; ++c)
            cpt[r][c] = Cm[i - 1][0][r] * dinv[i - 1][0][c] +
                        Cm[i - 1][1][r] * dinv[i - 1][1][c];
        for (int r = 0; r < 2; ++r)
          for (int c = 0; c < 2; ++c)
            M[r][c] -= cpt[r][0] * Cm[i - 1][0][c] + cpt[r][1] * Cm[i - 1][1][c];
      }
      float det = M[0][0] * M[1][1] - M[0][1] * M[1][0];
      if (fabsf(det) < kTiny32) det = kTiny32;
      const float idt = 1.0f / det;
      dinv[i][0][0] = M[1][1] * idt;
      dinv[i][0][1] = -M[0][1] * idt;
      dinv[i][1][0] = -M[1][0] * idt;
      dinv[i][1][1] = M[0][0] * idt;
    }
    float nf[NI][2], delta[NI][2];
    for (int i = 0; i < NI; ++i) {
      nf[i][0] = -f[i][0];
      nf[i][1] = -f[i][1];
    }
    thomas(nf, delta);
    float m0 = 0.0f;
    for (int i = 0; i < NI; ++i) m0 += f[i][0] * f[i][0] + f[i][1] * f[i][1];
    float lam_sel = 0.0f, lam = 1.0f;
    for (int j = 0; j < a.n_backtrack; ++j, lam *= 0.5f) {
      float cand[NI][2], sc[NI + 1], dc[NI + 1][3], fc[NI][2];
      for (int i = 0; i < NI; ++i)
        for (int r = 0; r < 2; ++r) cand[i][r] = ab[i][r] + lam * delta[i][r];
      geom(cand, sc, dc, fc);
      float mc = 0.0f;
      for (int i = 0; i < NI; ++i) mc += fc[i][0] * fc[i][0] + fc[i][1] * fc[i][1];
      if (mc < m0) {
        lam_sel = lam;
        break;
      }
    }
    for (int i = 0; i < NI; ++i)
      for (int r = 0; r < 2; ++r) ab[i][r] += lam_sel * delta[i][r];
  }
  geom(ab, s, dh, f);
  // float64 polish: tangent bases from the float64 normals, the Snell
  // residual in float64, one Newton step through the float32 factorisation
  // (the crossing positions enter the arrival direction at first order)
  double B64[NI][3][2], ab64[NI][2];
  for (int i = 0; i < NI; ++i) {
    const double *n = N64[i];
    const bool use_z = fabs(n[2]) < 0.9;
    const double a0 = use_z ? 0.0 : 1.0, a2 = use_z ? 1.0 : 0.0;
    double u[3] = {-a2 * n[1], a2 * n[0] - a0 * n[2], a0 * n[1]};
    const double un = 1.0 / sqrt(dot3v(u, u));
    for (int j = 0; j < 3; ++j) u[j] *= un;
    const double v[3] = {n[1] * u[2] - n[2] * u[1], n[2] * u[0] - n[0] * u[2],
                         n[0] * u[1] - n[1] * u[0]};
    for (int j = 0; j < 3; ++j) {
      B64[i][j][0] = u[j];
      B64[i][j][1] = v[j];
    }
    // re-express the float32 offset in the float64 basis
    const double y[3] = {
        (double)(B[i][0][0] * ab[i][0] + B[i][0][1] * ab[i][1]),
        (double)(B[i][1][0] * ab[i][0] + B[i][1][1] * ab[i][1]),
        (double)(B[i][2][0] * ab[i][0] + B[i][2][1] * ab[i][1])};
    for (int c = 0; c < 2; ++c)
      ab64[i][c] = B64[i][0][c] * y[0] + B64[i][1][c] * y[1] +
                   B64[i][2][c] * y[2];
  }
  const double scale64 = (double)scale;
  double X[NI][3], S64[NI + 1];
  auto geom64 = [&](bool want_f, float (&fo)[NI][2]) {
    for (int i = 0; i < NI; ++i)
      for (int j = 0; j < 3; ++j)
        X[i][j] = O[i][j] + scale64 * (B64[i][j][0] * ab64[i][0] +
                                       B64[i][j][1] * ab64[i][1]);
    double g[NI + 1][3];
    for (int kk = 0; kk <= NI; ++kk) {
      const double *pa = kk == 0 ? p : X[kk - 1];
      const double *pb = kk == NI ? q : X[kk];
      double d[3] = {pb[0] - pa[0], pb[1] - pa[1], pb[2] - pa[2]};
      S64[kk] = sqrt(dot3v(d, d));
      const double gs = a.n_leg[kk] / fmax(S64[kk], kTiny);
      for (int j = 0; j < 3; ++j) g[kk][j] = gs * d[j];
    }
    if (want_f)
      for (int i = 0; i < NI; ++i)
        for (int c = 0; c < 2; ++c)
          fo[i][c] = -(float)(B64[i][0][c] * (g[i][0] - g[i + 1][0]) +
                              B64[i][1][c] * (g[i][1] - g[i + 1][1]) +
                              B64[i][2][c] * (g[i][2] - g[i + 1][2]));
  };
  float nf64[NI][2];
  geom64(a.n_newton > 0, nf64);
  if (a.n_newton > 0) {
    float d64[NI][2];
    thomas(nf64, d64);
    bool fin = true;
    for (int i = 0; i < NI; ++i) fin = fin && isfinite(d64[i][0]) &&
                                       isfinite(d64[i][1]);
    if (fin) {
      for (int i = 0; i < NI; ++i)
        for (int c = 0; c < 2; ++c) ab64[i][c] += (double)d64[i][c];
      geom64(false, nf64);
    }
  }
  // validity (float32): residual, straddling, evanescence
  float residual = 0.0f;
  bool sides = true, evan = false;
  float cinc[NI], cout_[NI];
  for (int i = 0; i < NI; ++i) {
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
    // P_i - x_i = -seg_i, P_{i+2} - x_i = seg_{i+1} (unit directions suffice)
    sides = sides && (-dot3a(n, dh[i]) * dot3a(n, dh[i + 1]) < 0.0f);
    evan = evan || (nm[i] * st1 > nm[i + 1] * (1.0f + 64.0f * kEps32));
  }
  P.valid = (residual <= kTol32) && isfinite(residual) && sides && !evan;
  // radiometry sums (multilayer.py:436-457)
  float c_inc[NI];
  for (int i = 0; i < NI; ++i) c_inc[i] = fmaxf(cinc[i], (float)kCMin);
  const float c_surf = c_inc[a.k_pad];
  float tau2 = 1.0f, loss = 0.0f, sperp = 0.0f, spar = 0.0f;
  double opl = 0.0;
  for (int i = 0; i < NI; ++i) {
    const float g = fresnel_gamma32(k.eps_leg[i], k.eps_leg[i + 1], c_inc[i]);
    tau2 *= (1.0f - g * g);
    if (a.rough_cross) {
      const float kt = k.k0 * (nm[i] * cinc[i] - nm[i + 1] * cout_[i]);
      const float sk = k.sig_c[i] * kt;
      tau2 *= __expf(-2.0f * sk * sk);
    }
    const float cp = i < a.k_pad ? c_surf : c_inc[i];
    const float si = (float)S64[i];
    opl += a.n_leg[i] * S64[i];
    loss += si * (k.att_leg[i] * 1e-3f);
    sperp += si / nm[i];
    spar += si / (nm[i] * cp * cp);
  }
  P.tau2 = tau2;
  P.opl = opl;
  P.loss_db = loss;
  P.sum_perp = sperp;
  P.sum_par = spar;
  P.c0 = c_surf;
  P.c_last = fmaxf(cout_[NI - 1], (float)kCMin);
  for (int j = 0; j < 3; ++j) {
    P.cur[j] = X[NI - 1][j];
    P.xf[j] = X[0][j];
  }
}

template <int NI, int ROUGH>
__global__ void __launch_bounds__(128)
refracted_split_kernel(RefArgs a, RefSplitConsts k) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float2 *hist = reinterpret_cast<float2 *>(smem_raw);
  float *lg = reinterpret_cast<float *>(hist + (size_t)a.tb * a.n_seg);
  __shared__ double s_p[SS_MAX_TB][3];
  __shared__ float s_u[SS_MAX_TB][3], s_pv[SS_MAX_TB][6];
  __shared__ int s_lo[SS_MAX_TB], s_hi[SS_MAX_TB];
  __shared__ float s_drop[SS_MAX_TB];
  __shared__ float s_pat[SS_PAT_MAX];
  __shared__ float s_fad[SS_FAD_N];
  __shared__ int s_rng[2];
  const int chunk = blockIdx.x;
  const int t_base = blockIdx.y * a.tb;
  const int nt = min(a.tb, a.T - t_base);
  const int tid = threadIdx.x;
  int pa_len = 0, pb_len = 0;
  if (a.pat_kind == SS_PAT_ARRAY) { pa_len = 1; pb_len = 4; }
  if (a.pat_kind == SS_PAT_FINITE_DIPOLE) pa_len = 1;
  if (a.pat_kind == SS_PAT_ARRAY_TAPERED) { pa_len = 2 * a.pat_n; pb_len = 4; }
  if (a.pat_kind == SS_PAT_TABULATED) { pa_len = a.pat_n; pb_len = a.pat_n; }
  if (tid < nt) {
    const int t = t_base + tid;
    for (int j = 0; j < 3; ++j) {
      s_p[tid][j] = a.pos[3 * t + j];
      s_u[tid][j] = a.uct ? (float)a.uct[3 * t + j] : 0.0f;
    }
    for (int j = 0; j < 6; ++j)
      s_pv[tid][j] =
          (a.pv && j < a.pv_len) ? (float)a.pv[a.pv_len * t + j] : 0.0f;
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
  if (ROUGH != SS_ROUGH_NONE)
    for (int m = tid; m <= a.n_terms; m += blockDim.x)
      lg[m] = (float)lgamma((double)m + 1.0);
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
  }
  __syncthreads();

  const int nj = a.leg_last;
  const float n0 = k.n_leg[0], njn = k.n_leg[nj];
  const float nsf = (float)a.n_samples;
  for (int i = s_rng[0] + tid; i < s_rng[1]; i += blockDim.x) {
    const double q[3] = {(double)a.F.cx[i], (double)a.F.cy[i],
                         (double)a.F.cz[i]};
    const float fn[3] = {a.F.nx[i], a.F.ny[i], a.F.nz[i]};
    const float fa = a.F.area[i];
    for (int tt = 0; tt < nt; ++tt) {
      if (i < s_lo[tt] || i >= s_hi[tt]) continue;
      PathS P;
      if (NI == 0)
        path_sequential_split(a, k, s_p[tt], q, P);
      else
        path_joint_split<NI == 0 ? 1 : NI>(a, k, s_p[tt], q, P);
      // final leg: crossing -> facet, float64 length for the optical path
      const double d64[3] = {P.cur[0] - q[0], P.cur[1] - q[1],
                             P.cur[2] - q[2]};
      const double s_j64 = sqrt(dot3v(d64, d64));
      const double opl = P.opl + a.n_leg[nj] * s_j64;
      const float s_j = (float)s_j64;
      const float inv = 1.0f / fmaxf(s_j, 1e-30f);
      const float rh[3] = {(float)d64[0] * inv, (float)d64[1] * inv,
                           (float)d64[2] * inv};
      const float loss = P.loss_db + s_j * (k.att_leg[nj] * 1e-3f);
      const float sperp = P.sum_perp + s_j / njn;
      const float spar = P.sum_par + s_j / (njn * P.c_last * P.c_last);
      const float l_perp = n0 * sperp;
      const float l_par = n0 * P.c0 * P.c0 * spar;
      const float flux = (n0 * P.c0) / (njn * P.c_last);
      const float att_f = exp2f(-loss * 0.33219280949f);  // 10^(-loss/10)
      const float cos_t = dot3a(rh, fn);
      float spread = P.tau2 * flux / (l_par * l_perp);
      if (a.pat_kind != SS_PAT_ISOTROPIC) {
        const float d0[3] = {(float)(P.xf[0] - s_p[tt][0]),
                             (float)(P.xf[1] - s_p[tt][1]),
                             (float)(P.xf[2] - s_p[tt][2])};
        const float dm = rsqrtf(fmaxf(dot3a(d0, d0), 1e-30f));
        const float g = gain32(a.pat_kind, a.pat_n, pa_len, s_pat, s_pv[tt],
                               d0[0] * dm, d0[1] * dm, d0[2] * dm);
        spread *= g * g;
      }
      float re, im, pwr;
      if (a.coherent) {
        const float gam = a.F.gamma_f64 ? (float)a.F.gamma_f64[i] : (float)a.gamma;
        const float f1[3] = {a.F.e1x[i], a.F.e1y[i], a.F.e1z[i]};
        const float f2[3] = {a.F.e2x[i], a.F.e2y[i], a.F.e2z[i]};
        // r_hat . e in float64: the sinc arguments k_j (r_hat . e) need the
        // arrival direction to ~1e-8 rad
        const double is64 = 1.0 / fmax(s_j64, 1e-30);
        const float d1 = (float)((d64[0] * (double)f1[0] + d64[1] * (double)f1[1] +
                                  d64[2] * (double)f1[2]) * is64);
        const float d2 = (float)((d64[0] * (double)f2[0] + d64[1] * (double)f2[1] +
                                  d64[2] * (double)f2[2]) * is64);
        const float base = k.amp_pref_j * gam * cos_t * spread * att_f;
        float amp = base * fa * sinc32(k.kj * d1) * sinc32(k.kj * d2);
        if (a.taper) {
          const float ct = fminf(fmaxf(cos_t, (float)kCMin), 1.0f);
          const float ct2 = ct * ct;
          amp *= __expf(-__fdividef(1.0f - ct2, ct2) * k.taper_inv);
        }
        float cr = amp, ci = 0.0f;
        if (ROUGH != SS_ROUGH_NONE) {
          const float sg = a.F.sigma ? a.F.sigma[i] : k.sigma;
          const float lc = a.F.corr ? a.F.corr[i] : k.corr;
          const float l1 = sqrtf(dot3a(f1, f1)), l2 = sqrtf(dot3a(f2, f2));
          const float kk = 2.0f * k.kj * cos_t;
          const float dp = d_phi32<ROUGH>(a.n_terms, lg, s_fad, k.fadL, sg, lc,
                                          kk, 2.0f * k.kj * d1 / l1,
                                          2.0f * k.kj * d2 / l2, l1, l2);
          const float sk = sg * kk;
          cr = amp * __expf(-0.5f * sk * sk);
          if (fa > 0.0f) {
            const float ai = base * sqrtf(dp);
            cr += ai * a.F.phasor[2 * i];
            ci += ai * a.F.phasor[2 * i + 1];
          }
        }
        if (a.F.diffuse_amp && fa > 0.0f) {
          const float ct = fmaxf(cos_t, 0.0f);
          const float ad = sqrtf(fa * 0.15915494309f) *
                           (float)a.F.diffuse_amp[i] * ct *
                           (ct > 0.0f ? __powf(ct, 0.5f * k.n_exp)
                                      : (k.n_exp == 0.0f ? 1.0f : 0.0f)) *
                           spread * att_f;
          cr += ad * a.F.diffuse_phasor[2 * i];
          ci += ad * a.F.diffuse_phasor[2 * i + 1];
        }
        // carrier phase 2 k0 opl reduced modulo 2 pi in float64
        const double ph = 2.0 * a.k0 * opl;
        const double nred = rint(ph * 0.15915494309189535);
        const float red = (float)fma(-nred, 6.283185307179586, ph);
        float sn, cs;
        __sincosf(red, &sn, &cs);
        re = cr * sn - ci * cs;
        im = cr * cs + ci * sn;
        pwr = re * re + im * im;
      } else {
        const float aa = fa * cos_t * spread;
        re = aa * aa * att_f * att_f;
        im = 0.0f;
        pwr = re;
      }
      // fast-time bin from the float64 optical path; exact path near edges
      const double u = (2.0 * opl / a.c - a.t0) / a.dt;
      double fb = floor(u);
      const float frac = (float)(u - fb);
      bool valid = P.valid;
      if ((frac < kBinGuard || frac > 1.0f - kBinGuard) && u > -4.0 &&
          u < (double)a.n_samples + 4.0) {
        bool v64;
        const double o64 = full_opl64<NI>(a, s_p[tt], q, v64);
        const double twtt = __ddiv_rn(__dmul_rn(2.0, o64), a.c);
        fb = floor(__ddiv_rn(__dsub_rn(twtt, a.t0), a.dt));
      }
      const bool ok = valid && fb >= 0.0 && fb < (double)nsf;
      if (ok) {
        int b = (int)fb;
        if (a.split) {
          const float v[3] = {(float)(q[0] - s_p[tt][0]),
                              (float)(q[1] - s_p[tt][1]),
                              (float)(q[2] - s_p[tt][2])};
          if (dot3a(v, s_u[tt]) > 0.0f) b += a.n_samples;
        }
        float2 *h = hist + (size_t)tt * a.n_seg + b;
        atomicAdd(&h->x, re);
        if (a.coherent) atomicAdd(&h->y, im);
      } else {
        atomicAdd(&s_drop[tt], pwr);
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

template <int NI, int ROUGH>
static int launch_split(RefArgs &a, const RefSplitConsts &k, const Plan &p,
                        size_t smem, cudaStream_t st) {
  cudaError_t e = cudaFuncSetAttribute(
      refracted_split_kernel<NI, ROUGH>,
      cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return cuda_status(e, "refracted_split smem");
  dim3 grid(p.n_chunks, p.n_groups);
  refracted_split_kernel<NI, ROUGH><<<grid, p.threads, smem, st>>>(a, k);
  return cuda_status(cudaGetLastError(), "refracted_split launch");
}

template <int NI>
static int launch_split_r(RefArgs &a, const RefSplitConsts &k, const Plan &p,
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

int refracted_split_launch(RefArgs &a, const Plan &p, cudaStream_t st) {
  int pa_len = 0, pb_len = 0;
  if (a.pat_kind == SS_PAT_ARRAY) { pa_len = 1; pb_len = 4; }
  if (a.pat_kind == SS_PAT_FINITE_DIPOLE) pa_len = 1;
  if (a.pat_kind == SS_PAT_ARRAY_TAPERED) { pa_len = 2 * a.pat_n; pb_len = 4; }
  if (a.pat_kind == SS_PAT_TABULATED) { pa_len = a.pat_n; pb_len = a.pat_n; }
  if (pa_len + pb_len > SS_PAT_MAX) {
    set_error("antenna table too large for the split kernel");
    return SS_ERR_UNSUPPORTED;
  }
  if (a.joint && a.ni > 4) {
    set_error("split precision joint solve supports up to 4 interfaces; "
              "use precision='fp64'");
    return SS_ERR_UNSUPPORTED;
  }
  RefSplitConsts k{};
  k.k0 = (float)a.k0;
  const double kj = a.k0 * a.n_leg[a.leg_last];
  k.kj = (float)kj;
  k.amp_pref_j = (float)(kj / kTwoPi);
  k.taper_inv = a.taper ? (float)(1.0 / (2.0 * a.taper_s * a.taper_s)) : 0.f;
  k.sigma = (float)a.sigma;
  k.corr = (float)a.corr;
  k.fadL = (float)a.fad.L;
  k.n_exp = (float)a.n_exp;
  for (int i = 0; i <= a.leg_last; ++i) {
    k.n_leg[i] = (float)a.n_leg[i];
    k.eps_leg[i] = (float)a.eps_leg[i];
    k.att_leg[i] = (float)a.att_leg[i];
  }
  for (int i = 0; i < a.ni; ++i) k.sig_c[i] = (float)a.sig_c[i];
  const size_t smem = (size_t)p.tb * a.n_seg * sizeof(float2) +
                      (a.rough_kind ? (a.n_terms + 1) * sizeof(float) : 0);
  if (!a.joint) return launch_split_r<0>(a, k, p, smem, st);
  switch (a.ni) {
    case 1: return launch_split_r<1>(a, k, p, smem, st);
    case 2: return launch_split_r<2>(a, k, p, smem, st);
    case 3: return launch_split_r<3>(a, k, p, smem, st);
    default: return launch_split_r<4>(a, k, p, smem, st);
  }
}

}  // namespace ss
