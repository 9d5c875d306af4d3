// Refracted multilayer facet sum (FP64 form) on GB300.
//
// Same trace-block x facet-chunk decomposition and shared-memory histograms
// as the surface kernel (ss_coherent.cu). Per (trace, target facet) pair the
// refracted path is solved in float64 exactly as the reference program does:
//   sequential: per crossed interface a 10-iteration two-point Snell solve
//     on the mean plane anchors an affine facet lookup, then a 25-iteration
//     solve on that facet's tangent plane (multilayer.py:352-406);
//   joint: the mean-plane chain anchors every lookup, then a damped Newton on
//     2-D in-plane offsets with block-tridiagonal (Thomas) steps and step
//     halving solves all crossings at once (multilayer.py:408-457,
//     refraction_joint.py:249-322);
// followed by Fresnel transmission, ray-tube spreading, two-way attenuation,
// antenna gain, the facet's sinc response at the local wavenumber,
// roughness, diffuse channel and binning (multilayer.py:500-583).
#include <algorithm>

#include "ss_refracted.cuh"

namespace ss {

constexpr double kTiny = 1e-30;
constexpr double kEps64 = 2.220446049250313e-16;
constexpr double kCMin = 1e-9;

struct Snell64 {
  double x[3];
  double th1, th2, s1, s2, res;
  bool valid;
};

__device__ __forceinline__ double dot3v(const double *a, const double *b) {
  return (a[0] * b[0] + a[1] * b[1]) + a[2] * b[2];
}

// Two-point crossing (refraction.py:78-161; `comp` selects the component
// form of multilayer.py:196-266).
__device__ void snell64(const double *p, const double *q, const double *o,
                        const double *nrm, double n1, double n2, int n_iter,
                        bool comp, Snell64 &R) {
  double po[3] = {p[0] - o[0], p[1] - o[1], p[2] - o[2]};
  double qo[3] = {q[0] - o[0], q[1] - o[1], q[2] - o[2]};
  const double h1 = dot3v(po, nrm), h2 = dot3v(qo, nrm);
  const double a = fabs(h1), b = fabs(h2);
  double fp[3], w[3];
  for (int j = 0; j < 3; ++j) {
    fp[j] = p[j] - h1 * nrm[j];
    w[j] = (q[j] - h2 * nrm[j]) - fp[j];
  }
  const double L = sqrt(dot3v(w, w));
  const double Lm = fmax(L, kTiny);
  const double u[3] = {w[0] / Lm, w[1] / Lm, w[2] / Lm};
  const double s = fmax(a + b + L, kTiny);
  double ah, bh, Lh;
  if (comp) {
    const double inv_s = 1.0 / s;
    ah = a * inv_s; bh = b * inv_s; Lh = L * inv_s;
  } else {
    ah = a / s; bh = b / s; Lh = L / s;
  }
  const bool swap = n1 > n2;
  const double ratio = fmin(n1, n2) / fmax(n1, n2);
  const double ar = swap ? bh : ah, bd = swap ? ah : bh;
  const double hi0 = 1.0 - 8.0 * kEps64;
  double sig = fmin(Lh / fmax(sqrt(Lh * Lh + (ah + bh) * (ah + bh)), kTiny),
                    hi0);
  double lo = 0.0, hi = hi0;
  for (int it = 0; it < n_iter; ++it) {
    const double v = ratio * sig;
    const double c1 = fmax((1.0 - sig) * (1.0 + sig), kTiny);
    const double c2 = fmax((1.0 - v) * (1.0 + v), kTiny);
    const double sc1 = sqrt(c1), sc2 = sqrt(c2);
    const double F = comp ? (ar * sig * (1.0 / sc1) + bd * v * (1.0 / sc2)) - Lh
                          : (ar * sig / sc1 + bd * v / sc2) - Lh;
    if (F <= 0.0) lo = sig; else hi = sig;
    const double Fp = ar / (c1 * sc1) + (bd * ratio) / (c2 * sc2);
    const double sn = sig - F / fmax(Fp, kTiny);
    const bool ok = (sn >= lo) && (sn <= hi) && isfinite(sn);
    sig = ok ? sn : 0.5 * (lo + hi);
  }
  const double c1 = fmax((1.0 - sig) * (1.0 + sig), kTiny);
  const double tr = comp ? ar * sig * (1.0 / sqrt(c1)) : ar * sig / sqrt(c1);
  const double t = fmin(fmax(swap ? Lh - tr : tr, 0.0), Lh);
  const double d2 = Lh - t;
  const double r1 = fmax(sqrt(ah * ah + t * t), kTiny);
  const double r2 = fmax(sqrt(bh * bh + d2 * d2), kTiny);
  R.res = n1 * t / r1 - n2 * d2 / r2;
  R.s1 = s * r1;
  R.s2 = s * r2;
  const double st = s * t;
  for (int j = 0; j < 3; ++j) R.x[j] = fp[j] + st * u[j];
  R.th1 = atan2(t, ah);
  R.th2 = atan2(d2, bh);
  R.valid = (h1 * h2 < 0.0) && (fabs(R.res) <= 1e-9);
}

// Affine (x, y) -> nearest cell; round half to even like np.round.
__device__ __forceinline__ void lookup64(const ss_interface &I, const double *x,
                                         double *pt, double *nr) {
  const double rc0 = __dadd_rn(__dadd_rn(__dmul_rn(x[0], I.coef[0]),
                                         __dmul_rn(x[1], I.coef[2])),
                               I.coef[4]);
  const double rc1 = __dadd_rn(__dadd_rn(__dmul_rn(x[0], I.coef[1]),
                                         __dmul_rn(x[1], I.coef[3])),
                               I.coef[5]);
  const int row = (int)fmin(fmax(rint(rc0), 0.0), (double)(I.ny - 1));
  const int col = (int)fmin(fmax(rint(rc1), 0.0), (double)(I.nx - 1));
  const float *g = I.table + ((size_t)row * I.nx + col) * 6;
  for (int j = 0; j < 3; ++j) {
    pt[j] = (double)g[j];
    nr[j] = (double)g[3 + j];
  }
}

__device__ __forceinline__ double fresnel_gamma64(double e1, double e2,
                                                  double c1) {
  const double n1 = sqrt(e1), n2 = sqrt(e2);
  const double s2 = (e1 / e2) * (1.0 - c1 * c1);
  const double c2 = sqrt(fmax(1.0 - s2, 0.0));
  return (n1 * c1 - n2 * c2) / (n1 * c1 + n2 * c2);
}

// ---------------------------------------------------------------------
// joint N-interface solve (refraction_joint.py:249-322)
// ---------------------------------------------------------------------
template <int NI>
struct JointGeom {
  double x[NI][3], s[NI + 1], dh[NI + 1][3], f[NI][2];
};

template <int NI>
__device__ __forceinline__ void joint_geom(const double (&B)[NI][3][2],
                                           const double (&os)[NI][3],
                                           const double *ps, const double *qs,
                                           const double *nm,
                                           const double (&ab)[NI][2],
                                           JointGeom<NI> &G) {
  for (int i = 0; i < NI; ++i)
    for (int k = 0; k < 3; ++k)
      G.x[i][k] = os[i][k] + (B[i][k][0] * ab[i][0] + B[i][k][1] * ab[i][1]);
  double g[NI + 1][3];
  for (int k = 0; k <= NI; ++k) {
    const double *a = k == 0 ? ps : G.x[k - 1];
    const double *b = k == NI ? qs : G.x[k];
    double d[3] = {b[0] - a[0], b[1] - a[1], b[2] - a[2]};
    G.s[k] = fmax(sqrt(dot3v(d, d)), kTiny);
    for (int j = 0; j < 3; ++j) {
      G.dh[k][j] = d[j] / G.s[k];
      g[k][j] = nm[k] * G.dh[k][j];
    }
  }
  for (int i = 0; i < NI; ++i)
    for (int j = 0; j < 2; ++j) {
      double acc = 0.0;
      for (int k = 0; k < 3; ++k) acc += B[i][k][j] * (g[i][k] - g[i + 1][k]);
      G.f[i][j] = acc;
    }
}

__device__ __forceinline__ void inv2x2(const double (&m)[2][2],
                                       double (&o)[2][2]) {
  double det = m[0][0] * m[1][1] - m[0][1] * m[1][0];
  if (fabs(det) < kTiny) det = kTiny;
  o[0][0] = m[1][1] / det;
  o[0][1] = -m[0][1] / det;
  o[1][0] = -m[1][0] / det;
  o[1][1] = m[0][0] / det;
}

template <int NI>
__device__ void joint64(const double *p, const double *q,
                        const double (&O)[NI][3], const double (&Nn)[NI][3],
                        const double *nm, int n_newton, int n_backtrack,
                        double (&X)[NI][3], double (&th1)[NI],
                        double (&th2)[NI], double (&S)[NI + 1], bool &valid) {
  // chain initialiser: refraction.py two-point form, 25 iterations
  double x0[NI][3];
  {
    double cur[3] = {p[0], p[1], p[2]};
    for (int i = 0; i < NI; ++i) {
      Snell64 R;
      snell64(cur, q, O[i], Nn[i], nm[i], nm[i + 1], 25, false, R);
      for (int j = 0; j < 3; ++j) x0[i][j] = cur[j] = R.x[j];
    }
  }
  double pq[3] = {p[0] - q[0], p[1] - q[1], p[2] - q[2]};
  const double scale = fmax(sqrt(dot3v(pq, pq)), kTiny);
  const double inv = 1.0 / scale;
  double ps[3], qs[3], os[NI][3];
  for (int j = 0; j < 3; ++j) {
    ps[j] = p[j] * inv;
    qs[j] = q[j] * inv;
  }
  for (int i = 0; i < NI; ++i)
    for (int j = 0; j < 3; ++j) os[i][j] = O[i][j] * inv;
  // in-plane bases (refraction_joint.py:196-204)
  double B[NI][3][2];
  for (int i = 0; i < NI; ++i) {
    const double *n = Nn[i];
    const bool use_z = fabs(n[2]) < 0.9;
    const double a0 = use_z ? 0.0 : 1.0, a2 = use_z ? 1.0 : 0.0;
    double u[3] = {0.0 * n[2] - a2 * n[1], a2 * n[0] - a0 * n[2],
                   a0 * n[1] - 0.0 * n[0]};
    const double un = fmax(sqrt(dot3v(u, u)), kTiny);
    for (int j = 0; j < 3; ++j) u[j] /= un;
    const double v[3] = {n[1] * u[2] - n[2] * u[1], n[2] * u[0] - n[0] * u[2],
                         n[0] * u[1] - n[1] * u[0]};
    for (int j = 0; j < 3; ++j) {
      B[i][j][0] = u[j];
      B[i][j][1] = v[j];
    }
  }
  double ab[NI][2];
  for (int i = 0; i < NI; ++i)
    for (int j = 0; j < 2; ++j) {
      double acc = 0.0;
      for (int k = 0; k < 3; ++k)
        acc += B[i][k][j] * (x0[i][k] * inv - os[i][k]);
      ab[i][j] = acc;
    }
  const double mu = pow(kEps64, 0.75);
  JointGeom<NI> G;
  for (int it = 0; it < n_newton; ++it) {
    joint_geom<NI>(B, os, ps, qs, nm, ab, G);
    // W_k = (n_k / s_k) (I - d d^T), k = 0..NI
    double W[NI + 1][3][3];
    for (int k = 0; k <= NI; ++k)
      for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c)
          W[k][r][c] = (nm[k] / G.s[k]) *
                       ((r == c ? 1.0 : 0.0) - G.dh[k][r] * G.dh[k][c]);
    double A[NI][2][2], Cm[NI > 1 ? NI - 1 : 1][2][2];
    for (int i = 0; i < NI; ++i)
      for (int r = 0; r < 2; ++r)
        for (int c = 0; c < 2; ++c) {
          double acc = 0.0;
          for (int k = 0; k < 3; ++k)
            for (int l = 0; l < 3; ++l)
              acc += B[i][k][r] * (W[i][k][l] + W[i + 1][k][l]) * B[i][l][c];
          A[i][r][c] = acc + (r == c ? mu : 0.0);
        }
    for (int i = 0; i + 1 < NI; ++i)
      for (int r = 0; r < 2; ++r)
        for (int c = 0; c < 2; ++c) {
          double acc = 0.0;
          for (int k = 0; k < 3; ++k)
            for (int l = 0; l < 3; ++l)
              acc += B[i][k][r] * W[i + 1][k][l] * B[i + 1][l][c];
          Cm[i][r][c] = -acc;
        }
    // block Thomas (refraction_joint.py:218-246)
    double dinv[NI][2][2], y[NI][2], delta[NI][2];
    for (int i = 0; i < NI; ++i) {
      double M[2][2], rhs[2] = {-G.f[i][0], -G.f[i][1]};
      if (i == 0) {
        for (int r = 0; r < 2; ++r)
          for (int c = 0; c < 2; ++c) M[r][c] = A[i][r][c];
      } else {
        double cpt[2][2];  // C_{i-1}^T dinv_{i-1}
        for (int r = 0; r < 2; ++r)
          for (int c = 0; c < 2; ++c)
            cpt[r][c] = Cm[i - 1][0][r] * dinv[i - 1][0][c] +
                        Cm[i - 1][1][r] * dinv[i - 1][1][c];
        for (int r = 0; r < 2; ++r)
          for (int c = 0; c < 2; ++c)
            M[r][c] = A[i][r][c] - (cpt[r][0] * Cm[i - 1][0][c] +
                                    cpt[r][1] * Cm[i - 1][1][c]);
        for (int r = 0; r < 2; ++r)
          rhs[r] -= cpt[r][0] * y[i - 1][0] + cpt[r][1] * y[i - 1][1];
      }
      inv2x2(M, dinv[i]);
      y[i][0] = rhs[0];
      y[i][1] = rhs[1];
    }
    for (int i = NI - 1; i >= 0; --i) {
      double rr[2] = {y[i][0], y[i][1]};
      if (i < NI - 1)
        for (int r = 0; r < 2; ++r)
          rr[r] -= Cm[i][r][0] * delta[i + 1][0] + Cm[i][r][1] * delta[i + 1][1];
      for (int r = 0; r < 2; ++r)
        delta[i][r] = dinv[i][r][0] * rr[0] + dinv[i][r][1] * rr[1];
    }
    double m0 = 0.0;
    for (int i = 0; i < NI; ++i) m0 += G.f[i][0] * G.f[i][0] + G.f[i][1] * G.f[i][1];
    double lam_sel = 0.0, lam = 1.0;
    for (int j = 0; j < n_backtrack; ++j, lam *= 0.5) {
      double cand[NI][2];
      for (int i = 0; i < NI; ++i)
        for (int r = 0; r < 2; ++r) cand[i][r] = ab[i][r] + lam * delta[i][r];
      JointGeom<NI> Gc;
      joint_geom<NI>(B, os, ps, qs, nm, cand, Gc);
      double mc = 0.0;
      for (int i = 0; i < NI; ++i)
        mc += Gc.f[i][0] * Gc.f[i][0] + Gc.f[i][1] * Gc.f[i][1];
      if (mc < m0) {
        lam_sel = lam;
        break;
      }
    }
    for (int i = 0; i < NI; ++i)
      for (int r = 0; r < 2; ++r) ab[i][r] += lam_sel * delta[i][r];
  }
  joint_geom<NI>(B, os, ps, qs, nm, ab, G);
  for (int i = 0; i < NI; ++i)
    for (int j = 0; j < 3; ++j) X[i][j] = G.x[i][j] * scale;
  // polyline geometry and validity (refraction_joint.py:143-176)
  double dh[NI + 1][3];
  bool fin = true;
  for (int k = 0; k <= NI; ++k) {
    const double *a = k == 0 ? p : X[k - 1];
    const double *b = k == NI ? q : X[k];
    double d[3] = {b[0] - a[0], b[1] - a[1], b[2] - a[2]};
    S[k] = sqrt(dot3v(d, d));
    fin = fin && isfinite(S[k]);
    const double sm = fmax(S[k], kTiny);
    for (int j = 0; j < 3; ++j) dh[k][j] = d[j] / sm;
  }
  double residual = 0.0;
  bool sides = true, evan = false;
  for (int i = 0; i < NI; ++i) {
    const double *n = Nn[i];
    const double ct1 = dot3v(n, dh[i]), ct2 = dot3v(n, dh[i + 1]);
    double t1[3], t2[3], dG[3];
    for (int j = 0; j < 3; ++j) {
      t1[j] = dh[i][j] - ct1 * n[j];
      t2[j] = dh[i + 1][j] - ct2 * n[j];
      dG[j] = nm[i] * dh[i][j] - nm[i + 1] * dh[i + 1][j];
    }
    const double st1 = sqrt(dot3v(t1, t1)), st2 = sqrt(dot3v(t2, t2));
    th1[i] = atan2(st1, fabs(ct1));
    th2[i] = atan2(st2, fabs(ct2));
    const double nd = dot3v(n, dG);
    double rt[3] = {dG[0] - nd * n[0], dG[1] - nd * n[1], dG[2] - nd * n[2]};
    const double res = sqrt(dot3v(rt, rt));
    if (res > residual || isnan(res)) residual = res;
    const double *pa = i == 0 ? p : X[i - 1];
    const double *pb = i == NI - 1 ? q : X[i + 1];
    double hpv[3] = {pa[0] - X[i][0], pa[1] - X[i][1], pa[2] - X[i][2]};
    double hnv[3] = {pb[0] - X[i][0], pb[1] - X[i][1], pb[2] - X[i][2]};
    sides = sides && (dot3v(n, hpv) * dot3v(n, hnv) < 0.0);
    evan = evan || (nm[i] * st1 > nm[i + 1] * (1.0 + 64.0 * kEps64));
    fin = fin && isfinite(X[i][0]) && isfinite(X[i][1]) && isfinite(X[i][2]);
  }
  fin = fin && isfinite(residual);
  valid = (residual <= 1e-9) && fin && sides && !evan;
}

// Path result shared by both solvers (multilayer.py `path` returns).
struct Path64 {
  double cur[3], xf[3];
  bool valid;
  double opl, loss_db, sum_par, sum_perp, tau2, c0, c_last;
};

__device__ void path_sequential64(const RefArgs &a, const double *p,
                                  const double *q, Path64 &P) {
  double cur[3] = {p[0], p[1], p[2]};
  P.valid = true;
  P.opl = P.loss_db = P.sum_par = P.sum_perp = 0.0;
  P.tau2 = 1.0;
  P.c0 = P.c_last = 1.0;
  for (int i = 0; i < a.ni; ++i) {
    const ss_interface &I = a.ifc[i];
    const double n1 = a.n_leg[i], n2 = a.n_leg[i + 1];
    Snell64 R1;
    snell64(cur, q, I.mean_point, I.mean_normal, n1, n2, 10, true, R1);
    double pt[3], nr[3];
    lookup64(I, R1.x, pt, nr);
    const double inn = 1.0 / sqrt(dot3v(nr, nr));
    for (int j = 0; j < 3; ++j) nr[j] *= inn;
    Snell64 R;
    snell64(cur, q, pt, nr, n1, n2, 25, true, R);
    P.valid = P.valid && R.valid;
    const double c_inc = fmax(cos(R.th1), kCMin);
    if (i == 0) {
      P.c0 = c_inc;
      for (int j = 0; j < 3; ++j) P.xf[j] = R.x[j];
    }
    const double g = fresnel_gamma64(a.eps_leg[i], a.eps_leg[i + 1], c_inc);
    P.tau2 = P.tau2 * (1.0 - g * g);
    if (a.rough_cross) {
      const double kt = a.k0 * (n1 * c_inc - n2 * cos(R.th2));
      const double sk = a.sig_c[i] * kt;
      P.tau2 = P.tau2 * exp(-2.0 * (sk * sk));
    }
    P.opl = P.opl + n1 * R.s1;
    P.loss_db = P.loss_db + R.s1 * (a.att_leg[i] / 1000.0);
    P.sum_perp = P.sum_perp + R.s1 / n1;
    P.sum_par = P.sum_par + R.s1 / (n1 * c_inc * c_inc);
    P.c_last = fmax(cos(R.th2), kCMin);
    for (int j = 0; j < 3; ++j) cur[j] = R.x[j];
  }
  for (int j = 0; j < 3; ++j) P.cur[j] = cur[j];
}

template <int NI>
__device__ void path_joint64(const RefArgs &a, const double *p,
                             const double *q, Path64 &P) {
  // pass 1: mean-plane chain (10 iterations) anchors the lookups
  double pt[NI][3], nr[NI][3];
  {
    double cur[3] = {p[0], p[1], p[2]};
    for (int i = 0; i < NI; ++i) {
      Snell64 R;
      snell64(cur, q, a.ifc[i].mean_point, a.ifc[i].mean_normal, a.n_leg[i],
              a.n_leg[i + 1], 10, false, R);
      for (int j = 0; j < 3; ++j) cur[j] = R.x[j];
      lookup64(a.ifc[i], R.x, pt[i], nr[i]);
      const double nn = sqrt(dot3v(nr[i], nr[i]));
      for (int j = 0; j < 3; ++j) nr[i][j] = nr[i][j] / nn;
    }
  }
  double X[NI][3], th1[NI], th2[NI], S[NI + 1];
  bool valid;
  joint64<NI>(p, q, pt, nr, a.n_leg, a.n_newton, a.n_backtrack, X, th1, th2,
              S, valid);
  P.valid = valid;
  double c_inc[NI];
  for (int i = 0; i < NI; ++i) c_inc[i] = fmax(cos(th1[i]), kCMin);
  const double c_surf = c_inc[a.k_pad];
  double tau2 = 1.0, opl = 0.0, loss = 0.0, sperp = 0.0, spar = 0.0;
  for (int i = 0; i < NI; ++i) {
    const double g = fresnel_gamma64(a.eps_leg[i], a.eps_leg[i + 1], c_inc[i]);
    tau2 *= (1.0 - g * g);
  }
  if (a.rough_cross)
    for (int i = 0; i < NI; ++i) {
      const double kt =
          a.k0 * (a.n_leg[i] * cos(th1[i]) - a.n_leg[i + 1] * cos(th2[i]));
      const double sk = a.sig_c[i] * kt;
      tau2 *= exp(-2.0 * (sk * sk));
    }
  for (int i = 0; i < NI; ++i) {
    const double cp = i < a.k_pad ? c_surf : c_inc[i];
    const double nl = a.n_leg[i];
    opl += nl * S[i];
    loss += S[i] * (a.att_leg[i] / 1000.0);
    sperp += S[i] / nl;
    spar += S[i] / (nl * cp * cp);
  }
  P.tau2 = tau2;
  P.opl = opl;
  P.loss_db = loss;
  P.sum_perp = sperp;
  P.sum_par = spar;
  P.c0 = c_surf;
  P.c_last = fmax(cos(th2[NI - 1]), kCMin);
  for (int j = 0; j < 3; ++j) {
    P.cur[j] = X[NI - 1][j];
    P.xf[j] = X[0][j];
  }
}

template <int NI>
__global__ void __launch_bounds__(128)
refracted_fp64_kernel(RefArgs a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  double2 *hist = reinterpret_cast<double2 *>(smem_raw);
  double *lgam = reinterpret_cast<double *>(hist + (size_t)a.tb * a.n_seg);
  __shared__ double s_p[SS_MAX_TB][3], s_u[SS_MAX_TB][3], s_pv[SS_MAX_TB][6];
  __shared__ int s_lo[SS_MAX_TB], s_hi[SS_MAX_TB];
  __shared__ double s_drop[SS_MAX_TB];
  __shared__ int s_rng[2];
  const int chunk = blockIdx.x;
  const int t_base = blockIdx.y * a.tb;
  const int nt = min(a.tb, a.T - t_base);
  const int tid = threadIdx.x;
  if (tid < nt) {
    const int t = t_base + tid;
    for (int j = 0; j < 3; ++j) s_p[tid][j] = a.pos[3 * t + j];
    for (int j = 0; j < 3; ++j) s_u[tid][j] = a.uct ? a.uct[3 * t + j] : 0.0;
    for (int j = 0; j < 6; ++j)
      s_pv[tid][j] = (a.pv && j < a.pv_len) ? a.pv[a.pv_len * t + j] : 0.0;
    long lo = (long)a.off[t] * a.bs;
    long hi = min((long)(a.off[t] + a.n_win) * a.bs, (long)a.N);
    s_lo[tid] = (int)min(lo, (long)a.N);
    s_hi[tid] = (int)hi;
    s_drop[tid] = 0.0;
  }
  for (int j = tid; j < a.tb * a.n_seg; j += blockDim.x)
    hist[j] = make_double2(0.0, 0.0);
  if (a.rough_kind != SS_ROUGH_NONE)
    for (int m = tid; m <= a.n_terms; m += blockDim.x)
      lgam[m] = lgamma((double)m + 1.0);
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

  const int nj = a.ni;  // final medium index
  const double n0 = a.n_leg[0], njn = a.n_leg[nj];
  for (int i = s_rng[0] + tid; i < s_rng[1]; i += blockDim.x) {
    const double q[3] = {(double)a.F.cx[i], (double)a.F.cy[i],
                         (double)a.F.cz[i]};
    const double fn[3] = {(double)a.F.nx[i], (double)a.F.ny[i],
                          (double)a.F.nz[i]};
    const double fa = a.F.area[i];
    for (int tt = 0; tt < nt; ++tt) {
      if (i < s_lo[tt] || i >= s_hi[tt]) continue;
      Path64 P;
      if (NI == 0)
        path_sequential64(a, s_p[tt], q, P);
      else
        path_joint64<NI == 0 ? 1 : NI>(a, s_p[tt], q, P);
      // final leg (medium j): crossing -> facet
      double d[3] = {P.cur[0] - q[0], P.cur[1] - q[1], P.cur[2] - q[2]};
      const double s_j = sqrt(dot3v(d, d));
      const double inv = 1.0 / fmax(s_j, 1e-30);
      const double rh[3] = {d[0] * inv, d[1] * inv, d[2] * inv};
      const double opl = P.opl + njn * s_j;
      const double loss = P.loss_db + s_j * (a.att_leg[nj] / 1000.0);
      const double sperp = P.sum_perp + s_j / njn;
      const double spar = P.sum_par + s_j / (njn * P.c_last * P.c_last);
      const double l_perp = n0 * sperp;
      const double l_par = n0 * P.c0 * P.c0 * spar;
      const double flux = (n0 * P.c0) / (njn * P.c_last);
      const double att_f = pow(10.0, -loss / 10.0);
      const double cos_t = dot3v(rh, fn);
      double spread = P.tau2 * flux / (l_par * l_perp);
      if (a.pat_kind != SS_PAT_ISOTROPIC) {
        double d0[3] = {P.xf[0] - s_p[tt][0], P.xf[1] - s_p[tt][1],
                        P.xf[2] - s_p[tt][2]};
        const double dm = fmax(sqrt(dot3v(d0, d0)), 1e-30);
        const double g = gain64(a.pat_kind, a.pat_n, a.pa, a.pb, s_pv[tt],
                                d0[0] / dm, d0[1] / dm, d0[2] / dm);
        spread = spread * (g * g);
      }
      double re, im, pwr;
      if (a.coherent) {
        const double gam = a.F.gamma_f64 ? a.F.gamma_f64[i] : a.gamma;
        const double kj = a.k0 * njn;
        const double f1[3] = {(double)a.F.e1x[i], (double)a.F.e1y[i],
                              (double)a.F.e1z[i]};
        const double f2[3] = {(double)a.F.e2x[i], (double)a.F.e2y[i],
                              (double)a.F.e2z[i]};
        const double d1 = dot3v(rh, f1), d2 = dot3v(rh, f2);
        const double s1 = sinc_np(d1 * (kj / kPi));
        const double s2 = sinc_np(d2 * (kj / kPi));
        double amp = (kj / kTwoPi) * gam * cos_t * fa * s1 * s2 * spread * att_f;
        if (a.taper) {
          double ct = fmin(fmax(cos_t, kCMin), 1.0);
          const double ct2 = ct * ct;
          amp = amp * exp(-(1.0 - ct2) / (ct2 * (2.0 * a.taper_s * a.taper_s)));
        }
        double cr = amp, ci = 0.0;
        if (a.rough_kind != SS_ROUGH_NONE) {
          const double sg = a.F.sigma ? (double)a.F.sigma[i] : a.sigma;
          const double lc = a.F.corr ? (double)a.F.corr[i] : a.corr;
          const double l1 = sqrt(dot3v(f1, f1)), l2 = sqrt(dot3v(f2, f2));
          const double kk = 2.0 * kj * cos_t;
          const double dp = d_phi64(a.rough_kind, a.n_terms, lgam, a.fad.a,
                                    a.fad.L, sg, lc, kk, 2.0 * kj * d1 / l1,
                                    2.0 * kj * d2 / l2, l1, l2);
          const double sk = sg * kk;
          cr = amp * exp(-0.5 * (sk * sk));
          if (fa > 0.0) {
            const double ai = (kj / kTwoPi) * gam * cos_t * spread * att_f *
                              sqrt(dp);
            cr += ai * (double)a.F.phasor[2 * i];
            ci += ai * (double)a.F.phasor[2 * i + 1];
          }
        }
        if (a.F.diffuse_amp && fa > 0.0) {
          const double ct = fmax(cos_t, 0.0);
          const double ad = sqrt(fmax(fa, 0.0) / kTwoPi) * a.F.diffuse_amp[i] *
                            ct * pow(ct, 0.5 * a.n_exp) * spread * att_f;
          cr += ad * (double)a.F.diffuse_phasor[2 * i];
          ci += ad * (double)a.F.diffuse_phasor[2 * i + 1];
        }
        double sn, cs;
        sincos(2.0 * a.k0 * opl, &sn, &cs);
        re = cr * sn - ci * cs;
        im = cr * cs + ci * sn;
        pwr = re * re + im * im;
      } else {
        const double aa = fa * cos_t * spread;
        re = aa * aa * att_f * att_f;
        im = 0.0;
        pwr = re;
      }
      const double twtt = __ddiv_rn(__dmul_rn(2.0, opl), a.c);
      const double fb = floor(__ddiv_rn(__dsub_rn(twtt, a.t0), a.dt));
      const bool ok = P.valid && fb >= 0.0 && fb < (double)a.n_samples;
      if (ok) {
        int b = (int)fb;
        if (a.split) {
          double v[3] = {q[0] - s_p[tt][0], q[1] - s_p[tt][1],
                         q[2] - s_p[tt][2]};
          if (dot3v(v, s_u[tt]) > 0.0) b += a.n_samples;
        }
        double2 *h = hist + (size_t)tt * a.n_seg + b;
        atomicAdd(&h->x, re);
        if (a.coherent) atomicAdd(&h->y, im);
      } else {
        atomicAdd(&s_drop[tt], pwr);
      }
    }
  }
  __syncthreads();
  double2 *part = reinterpret_cast<double2 *>(a.part);
  for (int tt = 0; tt < nt; ++tt) {
    const size_t base = ((size_t)chunk * a.T + t_base + tt) * a.n_seg;
    for (int j = tid; j < a.n_seg; j += blockDim.x)
      part[base + j] = hist[(size_t)tt * a.n_seg + j];
  }
  if (tid < nt) a.part_drop[(size_t)chunk * a.T + t_base + tid] = s_drop[tid];
}

// ---------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------
static int refracted_plan(const ss_refracted_opts *o, int T, int N, Plan *p) {
  if (o->n_samples <= 0 || T <= 0 || N <= 0 || o->block_size <= 0 ||
      o->n_win <= 0 || o->n_crossed < 1 || o->n_crossed > SS_MAX_IFACE)
    return SS_ERR_ARG;
  const int n_seg = o->n_samples * (o->split_sides ? 2 : 1);
  const size_t elt = o->precision == SS_PREC_FP64 ? 16 : 8;
  const size_t per_trace = (size_t)n_seg * elt;
  if (per_trace > 200 * 1024) return SS_ERR_UNSUPPORTED;
  const size_t budget = 96 * 1024;
  int tb = (int)std::max<size_t>(1, std::min<size_t>(budget / per_trace,
                                                     SS_MAX_TB));
  tb = std::min(tb, T);
  p->tb = tb;
  p->n_groups = (T + tb - 1) / tb;
  p->threads = 128;
  const long window = std::min<long>((long)o->n_win * o->block_size, N);
  const int max_chunks = (int)std::max<long>(1, window / 256);
  const int target = 8 * sm_count();
  p->n_chunks = std::max(1, std::min(max_chunks,
                                     (target + p->n_groups - 1) / p->n_groups));
  p->smem = (size_t)tb * per_trace;
  return SS_OK;
}

static size_t refracted_scratch(const ss_refracted_opts *o, int T, int N) {
  Plan p;
  if (refracted_plan(o, T, N, &p) != SS_OK) return 0;
  const int n_seg = o->n_samples * (o->split_sides ? 2 : 1);
  const size_t elt = o->precision == SS_PREC_FP64 ? 16 : 8;
  size_t hist = (size_t)p.n_chunks * T * n_seg * elt;
  hist = (hist + 255) & ~(size_t)255;
  return hist + (size_t)p.n_chunks * T * sizeof(double);
}

template <int NI>
static int launch_fp64(RefArgs &a, const Plan &p, size_t smem,
                       cudaStream_t st) {
  cudaError_t e = cudaFuncSetAttribute(
      refracted_fp64_kernel<NI>, cudaFuncAttributeMaxDynamicSharedMemorySize,
      (int)smem);
  if (e != cudaSuccess) return cuda_status(e, "refracted_fp64 smem");
  dim3 grid(p.n_chunks, p.n_groups);
  refracted_fp64_kernel<NI><<<grid, p.threads, smem, st>>>(a);
  return cuda_status(cudaGetLastError(), "refracted_fp64 launch");
}

}  // namespace ss

extern "C" size_t ss_refracted_scratch_bytes(const ss_refracted_opts *opts,
                                             int32_t n_traces,
                                             int32_t n_facets) {
  if (!opts) return 0;
  return ss::refracted_scratch(opts, n_traces, n_facets);
}

extern "C" int ss_refracted_fwd(const ss_refracted_opts *opts,
                                const ss_facets *target,
                                const ss_traces *traces,
                                const ss_pattern *pattern,
                                const ss_roughness *rough,
                                const ss_output *out, void *scratch,
                                size_t scratch_bytes, void *stream) {
  using namespace ss;
  if (!opts || !target || !traces || !out || !opts->crossed ||
      !opts->n_leg || !opts->eps_leg || !opts->att_leg) {
    set_error("null argument");
    return SS_ERR_ARG;
  }
  const int T = traces->n_traces, N = target->n_facets;
  if (!traces->pos || !traces->off || !target->cx || !target->area ||
      !out->dropped || (!out->field_c128 && !out->field_c64)) {
    set_error("missing required device pointer");
    return SS_ERR_ARG;
  }
  if (opts->split_sides && !traces->uct) {
    set_error("split_sides needs u_ct");
    return SS_ERR_ARG;
  }
  Plan p;
  int s = refracted_plan(opts, T, N, &p);
  if (s) {
    set_error(s == SS_ERR_UNSUPPORTED ? "n_samples too large" :
              "bad sizes or crossed-interface count (1..8)");
    return s;
  }
  if (opts->joint && (opts->k_pad < 0 || opts->k_pad >= opts->n_crossed)) {
    set_error("k_pad out of range");
    return SS_ERR_ARG;
  }
  const size_t need = refracted_scratch(opts, T, N);
  if (!scratch || scratch_bytes < need) {
    set_error("scratch buffer too small");
    return SS_ERR_SCRATCH;
  }
  RefArgs a{};
  a.F = *target;
  a.pos = traces->pos;
  a.uct = traces->uct;
  a.pv = traces->pv;
  a.off = traces->off;
  a.T = T;
  a.N = N;
  a.pv_len = traces->pv_len;
  a.ni = opts->n_crossed;
  a.k_pad = opts->joint ? opts->k_pad : 0;
  for (int i = 0; i < a.ni; ++i) {
    a.ifc[i] = opts->crossed[i];
    if (!a.ifc[i].table || a.ifc[i].ny < 1 || a.ifc[i].nx < 1) {
      set_error("crossed interface without a lookup table");
      return SS_ERR_ARG;
    }
    a.sig_c[i] = opts->sigma_crossed ? opts->sigma_crossed[i] : 0.0;
  }
  for (int i = 0; i <= a.ni; ++i) {
    a.n_leg[i] = opts->n_leg[i];
    a.eps_leg[i] = opts->eps_leg[i];
    a.att_leg[i] = opts->att_leg[i];
  }
  a.rough_cross = opts->sigma_crossed != nullptr;
  a.k0 = opts->k0;
  a.gamma = opts->gamma;
  a.t0 = opts->t0;
  a.dt = opts->dt;
  a.c = opts->c;
  a.taper_s = opts->taper_s;
  a.n_exp = opts->diffuse_exp;
  a.n_samples = opts->n_samples;
  a.n_seg = opts->n_samples * (opts->split_sides ? 2 : 1);
  a.bs = opts->block_size;
  a.n_win = opts->n_win;
  a.split = opts->split_sides;
  a.coherent = opts->coherent;
  a.joint = opts->joint;
  a.n_newton = opts->joint_newton;
  a.n_backtrack = opts->joint_backtrack;
  a.taper = opts->taper;
  a.precision = opts->precision;
  a.pat_kind = pattern ? pattern->kind : SS_PAT_ISOTROPIC;
  a.pat_n = pattern ? pattern->n : 0;
  a.pa = pattern ? pattern->pa : nullptr;
  a.pb = pattern ? pattern->pb : nullptr;
  if (a.pat_kind != SS_PAT_ISOTROPIC && (!traces->pv || traces->pv_len < 3)) {
    set_error("antenna pattern needs per-trace pattern vectors");
    return SS_ERR_ARG;
  }
  a.rough_kind = rough ? rough->kind : SS_ROUGH_NONE;
  if (a.rough_kind != SS_ROUGH_NONE) {
    if (!target->phasor || rough->n_terms < 0 ||
        rough->n_terms > SS_MAX_TERMS) {
      set_error("roughness needs phasors and 0 <= n_terms <= 4096");
      return SS_ERR_ARG;
    }
    a.n_terms = rough->n_terms;
    a.sigma = rough->sigma;
    a.corr = rough->corr;
    a.fad = faddeeva_coeffs();
  }
  if (!a.coherent && (a.rough_kind || a.rough_cross || target->diffuse_amp ||
                      a.taper || target->gamma_f64)) {
    set_error("roughness, taper, diffuse and per-facet gamma require "
              "coherent mode");
    return SS_ERR_ARG;
  }
  a.part = scratch;
  size_t hist = (size_t)p.n_chunks * T * a.n_seg *
                (opts->precision == SS_PREC_FP64 ? 16 : 8);
  hist = (hist + 255) & ~(size_t)255;
  a.part_drop = reinterpret_cast<double *>(static_cast<char *>(scratch) +
                                           hist);
  a.tb = p.tb;
  a.n_chunks = p.n_chunks;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (opts->precision == SS_PREC_FP64) {
    const size_t smem = (size_t)p.tb * a.n_seg * 16 +
                        (a.rough_kind ? (a.n_terms + 1) * sizeof(double) : 0);
    if (!a.joint) s = launch_fp64<0>(a, p, smem, st);
    else switch (a.ni) {
      case 1: s = launch_fp64<1>(a, p, smem, st); break;
      case 2: s = launch_fp64<2>(a, p, smem, st); break;
      case 3: s = launch_fp64<3>(a, p, smem, st); break;
      case 4: s = launch_fp64<4>(a, p, smem, st); break;
      case 5: s = launch_fp64<5>(a, p, smem, st); break;
      case 6: s = launch_fp64<6>(a, p, smem, st); break;
      case 7: s = launch_fp64<7>(a, p, smem, st); break;
      default: s = launch_fp64<8>(a, p, smem, st); break;
    }
  } else {
    s = refracted_split_launch(a, p, st);
  }
  if (s) return s;
  ReduceArgs r{a.T, a.n_seg, a.n_samples, a.split, a.n_chunks, a.part,
               a.part_drop};
  return launch_reduce(r, opts->precision == SS_PREC_FP64, out, st);
}
