// float64 refracted-path solvers shared by the FP64 kernel and the split
// kernel's exact fallbacks (internal).
#pragma once

#include "ss_refracted.cuh"

namespace ss {

constexpr double kTiny = 1e-30;
constexpr double kEps64 = 2.220446049250313e-16;
constexpr double kCMin = 1e-9;
// Template argument of the deep-stack instantiations: the joint solve's
// arrays hold SS_MAX_IFACE interfaces (in local memory) and the count
// crossed is the call's; every smaller argument is a count of its own.
constexpr int kDeepNI = SS_MAX_IFACE;

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
static __device__ __noinline__ void snell64(const double *p, const double *q, const double *o,
                        const double *nrm, double n1, double n2, int n_iter,
                        bool comp, Snell64 &R, bool early = false,
                        bool x_only = false) {
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
    const double nxt = ok ? sn : 0.5 * (lo + hi);
    // early: stop at the fixed point (the remaining fixed-budget iterations
    // would leave sigma unchanged to within an ulp)
    const bool done = early && fabs(nxt - sig) <= 4.0 * kEps64 * fmax(sig, 1e-12);
    sig = nxt;
    if (done) break;
  }
  const double c1 = fmax((1.0 - sig) * (1.0 + sig), kTiny);
  const double tr = comp ? ar * sig * (1.0 / sqrt(c1)) : ar * sig / sqrt(c1);
  const double t = fmin(fmax(swap ? Lh - tr : tr, 0.0), Lh);
  if (x_only) {  // the crossing point alone (lookup anchors)
    const double st = s * t;
    for (int j = 0; j < 3; ++j) R.x[j] = fp[j] + st * u[j];
    return;
  }
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
                                           JointGeom<NI> &G, int ni = NI) {
  for (int i = 0; i < ni; ++i)
    for (int k = 0; k < 3; ++k)
      G.x[i][k] = os[i][k] + (B[i][k][0] * ab[i][0] + B[i][k][1] * ab[i][1]);
  double g[NI + 1][3];
  for (int k = 0; k <= ni; ++k) {
    const double *a = k == 0 ? ps : G.x[k - 1];
    const double *b = k == ni ? qs : G.x[k];
    double d[3] = {b[0] - a[0], b[1] - a[1], b[2] - a[2]};
    G.s[k] = fmax(sqrt(dot3v(d, d)), kTiny);
    for (int j = 0; j < 3; ++j) {
      G.dh[k][j] = d[j] / G.s[k];
      g[k][j] = nm[k] * G.dh[k][j];
    }
  }
  for (int i = 0; i < ni; ++i)
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
static __device__ __noinline__ void joint64(const double *p, const double *q,
                        const double (&O)[NI][3], const double (&Nn)[NI][3],
                        const double *nm, int n_newton, int n_backtrack,
                        double (&X)[NI][3], double (&th1)[NI],
                        double (&th2)[NI], double (&S)[NI + 1], bool &valid,
                        int ni = NI) {
  // chain initialiser: refraction.py two-point form, 25 iterations
  double x0[NI][3];
  {
    double cur[3] = {p[0], p[1], p[2]};
    for (int i = 0; i < ni; ++i) {
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
  for (int i = 0; i < ni; ++i)
    for (int j = 0; j < 3; ++j) os[i][j] = O[i][j] * inv;
  // in-plane bases (refraction_joint.py:196-204)
  double B[NI][3][2];
  for (int i = 0; i < ni; ++i) {
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
  for (int i = 0; i < ni; ++i)
    for (int j = 0; j < 2; ++j) {
      double acc = 0.0;
      for (int k = 0; k < 3; ++k)
        acc += B[i][k][j] * (x0[i][k] * inv - os[i][k]);
      ab[i][j] = acc;
    }
  const double mu = pow(kEps64, 0.75);
  JointGeom<NI> G;
  for (int it = 0; it < n_newton; ++it) {
    joint_geom<NI>(B, os, ps, qs, nm, ab, G, ni);
    // W_k = (n_k / s_k) (I - d d^T), k = 0..ni
    double W[NI + 1][3][3];
    for (int k = 0; k <= ni; ++k)
      for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c)
          W[k][r][c] = (nm[k] / G.s[k]) *
                       ((r == c ? 1.0 : 0.0) - G.dh[k][r] * G.dh[k][c]);
    double A[NI][2][2], Cm[NI > 1 ? NI - 1 : 1][2][2];
    for (int i = 0; i < ni; ++i)
      for (int r = 0; r < 2; ++r)
        for (int c = 0; c < 2; ++c) {
          double acc = 0.0;
          for (int k = 0; k < 3; ++k)
            for (int l = 0; l < 3; ++l)
              acc += B[i][k][r] * (W[i][k][l] + W[i + 1][k][l]) * B[i][l][c];
          A[i][r][c] = acc + (r == c ? mu : 0.0);
        }
    for (int i = 0; i + 1 < ni; ++i)
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
    for (int i = 0; i < ni; ++i) {
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
    for (int i = ni - 1; i >= 0; --i) {
      double rr[2] = {y[i][0], y[i][1]};
      if (i < ni - 1)
        for (int r = 0; r < 2; ++r)
          rr[r] -= Cm[i][r][0] * delta[i + 1][0] + Cm[i][r][1] * delta[i + 1][1];
      for (int r = 0; r < 2; ++r)
        delta[i][r] = dinv[i][r][0] * rr[0] + dinv[i][r][1] * rr[1];
    }
    double m0 = 0.0;
    for (int i = 0; i < ni; ++i) m0 += G.f[i][0] * G.f[i][0] + G.f[i][1] * G.f[i][1];
    double lam_sel = 0.0, lam = 1.0;
    for (int j = 0; j < n_backtrack; ++j, lam *= 0.5) {
      double cand[NI][2];
      for (int i = 0; i < ni; ++i)
        for (int r = 0; r < 2; ++r) cand[i][r] = ab[i][r] + lam * delta[i][r];
      JointGeom<NI> Gc;
      joint_geom<NI>(B, os, ps, qs, nm, cand, Gc, ni);
      double mc = 0.0;
      for (int i = 0; i < ni; ++i)
        mc += Gc.f[i][0] * Gc.f[i][0] + Gc.f[i][1] * Gc.f[i][1];
      if (mc < m0) {
        lam_sel = lam;
        break;
      }
    }
    for (int i = 0; i < ni; ++i)
      for (int r = 0; r < 2; ++r) ab[i][r] += lam_sel * delta[i][r];
  }
  joint_geom<NI>(B, os, ps, qs, nm, ab, G, ni);
  for (int i = 0; i < ni; ++i)
    for (int j = 0; j < 3; ++j) X[i][j] = G.x[i][j] * scale;
  // polyline geometry and validity (refraction_joint.py:143-176)
  double dh[NI + 1][3];
  bool fin = true;
  for (int k = 0; k <= ni; ++k) {
    const double *a = k == 0 ? p : X[k - 1];
    const double *b = k == ni ? q : X[k];
    double d[3] = {b[0] - a[0], b[1] - a[1], b[2] - a[2]};
    S[k] = sqrt(dot3v(d, d));
    fin = fin && isfinite(S[k]);
    const double sm = fmax(S[k], kTiny);
    for (int j = 0; j < 3; ++j) dh[k][j] = d[j] / sm;
  }
  double residual = 0.0;
  bool sides = true, evan = false;
  for (int i = 0; i < ni; ++i) {
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
    const double *pb = i == ni - 1 ? q : X[i + 1];
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

static __device__ __noinline__ void path_sequential64(const RefArgs &a, const double *p,
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
static __device__ __noinline__ void path_joint64(const RefArgs &a, const double *p,
                             const double *q, Path64 &P) {
  // a deep stack (NI == kDeepNI) holds up to NI interfaces in its arrays
  // and crosses a.ni of them; the other instantiations fold ni to NI
  const int ni = NI == kDeepNI ? a.ni : NI;
  // pass 1: mean-plane chain (10 iterations) anchors the lookups
  double pt[NI][3], nr[NI][3];
  {
    double cur[3] = {p[0], p[1], p[2]};
    for (int i = 0; i < ni; ++i) {
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
              S, valid, ni);
  P.valid = valid;
  double c_inc[NI];
  for (int i = 0; i < ni; ++i) c_inc[i] = fmax(cos(th1[i]), kCMin);
  const double c_surf = c_inc[a.k_pad];
  double tau2 = 1.0, opl = 0.0, loss = 0.0, sperp = 0.0, spar = 0.0;
  for (int i = 0; i < ni; ++i) {
    const double g = fresnel_gamma64(a.eps_leg[i], a.eps_leg[i + 1], c_inc[i]);
    tau2 *= (1.0 - g * g);
  }
  if (a.rough_cross)
    for (int i = 0; i < ni; ++i) {
      const double kt =
          a.k0 * (a.n_leg[i] * cos(th1[i]) - a.n_leg[i + 1] * cos(th2[i]));
      const double sk = a.sig_c[i] * kt;
      tau2 *= exp(-2.0 * (sk * sk));
    }
  for (int i = 0; i < ni; ++i) {
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
  P.c_last = fmax(cos(th2[ni - 1]), kCMin);
  for (int j = 0; j < 3; ++j) {
    P.cur[j] = X[ni - 1][j];
    P.xf[j] = X[0][j];
  }
}

// Full float64 optical path length (crossing legs + final leg) and path
// validity for one pair: the exact reference quantity the split kernel falls
// back to when a pair sits within the bin-edge guard band.
template <int NI>
static __device__ __noinline__ double full_opl64(const RefArgs &a, const double *p,
                                    const double *q, bool &valid) {
  Path64 P;
  if (NI == 0)
    path_sequential64(a, p, q, P);
  else
    path_joint64<NI == 0 ? 1 : NI>(a, p, q, P);
  double d[3] = {P.cur[0] - q[0], P.cur[1] - q[1], P.cur[2] - q[2]};
  valid = P.valid;
  return P.opl + a.n_leg[a.leg_last] * sqrt(dot3v(d, d));
}

}  // namespace ss
