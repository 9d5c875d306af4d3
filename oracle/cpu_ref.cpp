// Float64 host restatement of the reference formulas for the coherent facet
// path: the smooth LPA surface pair, the refracted pair by the sequential
// chain or the joint solve, Fresnel transmission, spreading, attenuation and
// the fast-time bin. It is TEST INFRASTRUCTURE and the timed CPU baseline:
// only the tests and the benchmark's CPU / reference legs load it; nothing
// on the product path does.
//
// It restates, pair by pair, the same steps as the NumPy oracle in this
// directory (lpa.py, refraction.py, refracted.py), which follow soundersim:
//   * kernels/coherent.py:107-128   LPA pair (lpa_contributions)
//   * kernels/geometry.py:18-24     twtt_bin (floor, drop-not-wrap)
//   * kernels/multilayer.py:196-266 two-point Snell solve, component form
//     (refraction.py:78-161 for the division form the joint initialiser uses)
//   * kernels/multilayer.py:352-406 sequential chain with facet lookups
//   * kernels/multilayer.py:408-457 joint path; refraction_joint.py:131-322
//     (chain, polyline, plane basis, 2x2 inverse, block Thomas, damped
//     Gauss-Newton with step halving and a Levenberg shift)
//   * kernels/multilayer.py:459-588 per-pair radiometry, phase and bin
//   * physics.py:33-67              TE Fresnel coefficient
// Host preparation (culling order, windows, lookup tables, affine fits, mean
// planes, joint padding) stays in Python (cpu_ref.py builds it with the
// oracle's own functions). Features the multilayer benchmark does not use
// (roughness, antenna patterns, taper, diffuse channel, side split) are not
// restated; the wrapper refuses them.
//
// Parallel over traces with OpenMP (dynamic schedule); each trace's facet
// window is summed in facet order into that trace's own row, so the result
// does not depend on the thread count. Built with -ffp-contract=off so no
// multiply-add is fused and every operation rounds as the NumPy oracle's
// does.
#include <omp.h>

#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

namespace {

constexpr double kTiny = 1e-30;
constexpr double kEps64 = 2.220446049250313e-16;
constexpr double kCMin = 1e-9;
constexpr double kPi = 3.141592653589793238462643383279502884;
constexpr double kTwoPi = 2.0 * kPi;

inline double dot3(const double *a, const double *b) {
  return (a[0] * b[0] + a[1] * b[1]) + a[2] * b[2];
}

inline double sinc_np(double x) {  // numpy's sin(pi x) / (pi x)
  if (x == 0.0) return 1.0;
  const double y = kPi * x;
  return std::sin(y) / y;
}

struct Crossing {
  double x[3];
  double th1, th2, s1, s2, residual;
  bool valid;
};

// Two-point flat-interface solve (multilayer.py:196-266 when component is
// true; refraction.py:78-161 otherwise).
void snell(const double *p, const double *q, const double *o,
           const double *nrm, double n1, double n2, int n_iter,
           bool component, double tol, Crossing &R) {
  double po[3], qo[3];
  for (int j = 0; j < 3; ++j) {
    po[j] = p[j] - o[j];
    qo[j] = q[j] - o[j];
  }
  const double h1 = dot3(po, nrm), h2 = dot3(qo, nrm);
  const double a = std::fabs(h1), b = std::fabs(h2);
  double fp[3], fq[3], w[3];
  for (int j = 0; j < 3; ++j) {
    fp[j] = p[j] - h1 * nrm[j];
    fq[j] = q[j] - h2 * nrm[j];
    w[j] = fq[j] - fp[j];
  }
  const double L = std::sqrt(dot3(w, w));
  double u[3];
  const double Lc = std::fmax(L, kTiny);
  for (int j = 0; j < 3; ++j) u[j] = w[j] / Lc;
  const double s = std::fmax(a + b + L, kTiny);
  double ah, bh, Lh;
  if (component) {
    const double inv_s = 1.0 / s;
    ah = a * inv_s;
    bh = b * inv_s;
    Lh = L * inv_s;
  } else {
    ah = a / s;
    bh = b / s;
    Lh = L / s;
  }
  const bool swap = n1 > n2;
  const double ratio = std::fmin(n1, n2) / std::fmax(n1, n2);
  const double ar = swap ? bh : ah, bd = swap ? ah : bh;
  const double hi0 = 1.0 - 8.0 * kEps64;
  const double apb = ah + bh;
  double sig = std::fmin(Lh / std::fmax(std::sqrt(Lh * Lh + apb * apb), kTiny),
                         hi0);
  double lo = 0.0, hi = hi0;
  for (int it = 0; it < n_iter; ++it) {
    const double v = ratio * sig;
    const double c1 = std::fmax((1.0 - sig) * (1.0 + sig), kTiny);
    const double c2 = std::fmax((1.0 - v) * (1.0 + v), kTiny);
    double F;
    if (component)
      F = ar * sig * (1.0 / std::sqrt(c1)) + bd * v * (1.0 / std::sqrt(c2)) -
          Lh;
    else
      F = ar * sig / std::sqrt(c1) + bd * v / std::sqrt(c2) - Lh;
    if (F <= 0.0) lo = sig; else hi = sig;
    const double Fp = ar / (c1 * std::sqrt(c1)) +
                      (bd * ratio) / (c2 * std::sqrt(c2));
    const double sn = sig - F / std::fmax(Fp, kTiny);
    const bool ok = (sn >= lo) && (sn <= hi) && std::isfinite(sn);
    sig = ok ? sn : 0.5 * (lo + hi);
  }
  const double c1 = std::fmax((1.0 - sig) * (1.0 + sig), kTiny);
  const double tr = component ? ar * sig * (1.0 / std::sqrt(c1))
                              : ar * sig / std::sqrt(c1);
  const double t = std::fmin(std::fmax(swap ? Lh - tr : tr, 0.0), Lh);
  const double d2 = Lh - t;
  const double r1 = std::fmax(std::sqrt(ah * ah + t * t), kTiny);
  const double r2 = std::fmax(std::sqrt(bh * bh + d2 * d2), kTiny);
  R.residual = n1 * t / r1 - n2 * d2 / r2;
  for (int j = 0; j < 3; ++j) R.x[j] = fp[j] + (s * t) * u[j];
  R.th1 = std::atan2(t, ah);
  R.th2 = std::atan2(d2, bh);
  R.s1 = s * r1;
  R.s2 = s * r2;
  R.valid = (h1 * h2 < 0.0) && (std::fabs(R.residual) <= tol);
}

double fresnel_te(double e1, double e2, double c1) {
  const double n1 = std::sqrt(e1), n2 = std::sqrt(e2);
  const double s2 = (e1 / e2) * (1.0 - c1 * c1);
  const double c2 = std::sqrt(std::fmax(1.0 - s2, 0.0));
  return (n1 * c1 - n2 * c2) / (n1 * c1 + n2 * c2);
}

// One crossed interface of the stack: float32 lookup grids, affine
// (x, y, 1) -> (row, col) fit, mean plane.
struct Iface {
  const float *gc, *gn;  // (ny, nx, 3)
  int ny, nx;
  double coef[6];        // rows x, y, 1; columns row, col
  double mp[3], mn[3];
};

// Nearest-facet plane (multilayer.py:377-386 / :422-431): affine index,
// round half to even, clip, gather.
void lookup(const Iface &I, const double *x, double *pt, double *nr) {
  const double rc0 = x[0] * I.coef[0] + x[1] * I.coef[2] + I.coef[4];
  const double rc1 = x[0] * I.coef[1] + x[1] * I.coef[3] + I.coef[5];
  const double r = std::fmin(std::fmax(std::nearbyint(rc0), 0.0),
                             (double)(I.ny - 1));
  const double c = std::fmin(std::fmax(std::nearbyint(rc1), 0.0),
                             (double)(I.nx - 1));
  const size_t k = ((size_t)r * I.nx + (size_t)c) * 3;
  for (int j = 0; j < 3; ++j) {
    pt[j] = (double)I.gc[k + j];
    nr[j] = (double)I.gn[k + j];
  }
}

struct Params {
  int ni, k_pad, joint, n_newton, n_backtrack;
  const double *n_leg, *eps_leg, *att_leg;  // ni + 1 legs
  double k0, t0, dt, c;
  int n_samples;
};

struct PathOut {
  double cur[3], x_first[3];
  bool valid;
  double opl, loss_db, sum_par, sum_perp, tau2, c0, c_last;
};

void path_sequential(const Params &P, const Iface *ifc, const double *p,
                     const double *q, PathOut &o) {
  double cur[3] = {p[0], p[1], p[2]};
  o.valid = true;
  o.opl = o.loss_db = o.sum_par = o.sum_perp = 0.0;
  o.tau2 = 1.0;
  for (int i = 0; i < P.ni; ++i) {
    const Iface &I = ifc[i];
    Crossing Rm, R;
    snell(cur, q, I.mp, I.mn, P.n_leg[i], P.n_leg[i + 1], 10, true, 1e-9, Rm);
    double pt[3], nr[3];
    lookup(I, Rm.x, pt, nr);
    const double inv = 1.0 / std::sqrt(dot3(nr, nr));
    for (int j = 0; j < 3; ++j) nr[j] = nr[j] * inv;
    snell(cur, q, pt, nr, P.n_leg[i], P.n_leg[i + 1], 25, true, 1e-9, R);
    o.valid = o.valid && R.valid;
    const double c_inc = std::fmax(std::cos(R.th1), kCMin);
    if (i == 0) {
      o.c0 = c_inc;
      for (int j = 0; j < 3; ++j) o.x_first[j] = R.x[j];
    }
    const double g = fresnel_te(P.eps_leg[i], P.eps_leg[i + 1], c_inc);
    o.tau2 = o.tau2 * (1.0 - g * g);
    o.opl = o.opl + P.n_leg[i] * R.s1;
    o.loss_db = o.loss_db + R.s1 * (P.att_leg[i] / 1000.0);
    o.sum_perp = o.sum_perp + R.s1 / P.n_leg[i];
    o.sum_par = o.sum_par + R.s1 / (P.n_leg[i] * c_inc * c_inc);
    o.c_last = std::fmax(std::cos(R.th2), kCMin);
    for (int j = 0; j < 3; ++j) cur[j] = R.x[j];
  }
  for (int j = 0; j < 3; ++j) o.cur[j] = cur[j];
}

// Orthonormal in-plane basis (refraction_joint.py:196-204): columns u, v.
void plane_basis(const double *n, double B[3][2]) {
  const bool use_z = std::fabs(n[2]) < 0.9;
  const double r0 = use_z ? 0.0 : 1.0, r2 = use_z ? 1.0 : 0.0;
  // u = ref x n with ref = (r0, 0, r2)
  double u[3] = {0.0 * n[2] - r2 * n[1], r2 * n[0] - r0 * n[2],
                 r0 * n[1] - 0.0 * n[0]};
  const double un = std::fmax(std::sqrt(dot3(u, u)), kTiny);
  for (int j = 0; j < 3; ++j) u[j] = u[j] / un;
  const double v[3] = {n[1] * u[2] - n[2] * u[1], n[2] * u[0] - n[0] * u[2],
                       n[0] * u[1] - n[1] * u[0]};
  for (int j = 0; j < 3; ++j) {
    B[j][0] = u[j];
    B[j][1] = v[j];
  }
}

void inv2(const double m[2][2], double out[2][2]) {
  double det = m[0][0] * m[1][1] - m[0][1] * m[1][0];
  if (std::fabs(det) < kTiny) det = kTiny;
  out[0][0] = m[1][1] / det;
  out[0][1] = -m[0][1] / det;
  out[1][0] = -m[1][0] / det;
  out[1][1] = m[0][0] / det;
}

// Joint stationary path through the looked-up planes
// (refraction_joint.py:249-322), then the polyline's geometry and validity
// (:143-176). x (ni, 3) out; th1, th2 (ni,); s (ni + 1,).
// Per-thread scratch of the joint path (sized once per thread, reused for
// every pair).
struct JointWork {
  std::vector<double> o, nrm, B, ab, x, s, dh, f, A, Cm, dinv, y, delta, cand,
      fc, sc, dhc, xv, xc, dhp, O, Nn, X, th1, th2, S, cinc;
};

void joint_solve(const Params &P, const double *p, const double *q,
                 const double *O, const double *Nn, JointWork &W, double *x,
                 double *th1, double *th2, double *s_out, bool &valid) {
  const int N = P.ni;
  const double *nm = P.n_leg;
  // chain initialiser, division form, 25 iterations
  std::vector<double> &x0 = W.x;
  x0.assign(3 * N, 0.0);
  {
    double cur[3] = {p[0], p[1], p[2]};
    for (int i = 0; i < N; ++i) {
      Crossing R;
      snell(cur, q, O + 3 * i, Nn + 3 * i, nm[i], nm[i + 1], 25, false, 1e-9,
            R);
      for (int j = 0; j < 3; ++j) x0[3 * i + j] = cur[j] = R.x[j];
    }
  }
  double pq[3] = {p[0] - q[0], p[1] - q[1], p[2] - q[2]};
  const double scale = std::fmax(std::sqrt(dot3(pq, pq)), kTiny);
  const double inv = 1.0 / scale;
  double ps[3], qs[3];
  for (int j = 0; j < 3; ++j) {
    ps[j] = p[j] * inv;
    qs[j] = q[j] * inv;
  }
  std::vector<double> &os = W.o, &B = W.B, &ab = W.ab;
  os.resize(3 * N);
  B.resize(6 * N);
  ab.resize(2 * N);
  for (int i = 0; i < N; ++i) {
    for (int j = 0; j < 3; ++j) os[3 * i + j] = O[3 * i + j] * inv;
    plane_basis(Nn + 3 * i, reinterpret_cast<double(*)[2]>(&B[6 * i]));
    double rel[3];
    for (int j = 0; j < 3; ++j) rel[j] = x0[3 * i + j] * inv - os[3 * i + j];
    for (int c = 0; c < 2; ++c)
      ab[2 * i + c] = (B[6 * i + 0 + c] * rel[0] + B[6 * i + 2 + c] * rel[1]) +
                      B[6 * i + 4 + c] * rel[2];
  }
  const double mu = std::pow(kEps64, 0.75);
  auto geom = [&](const double *abv, double *xv, double *sv, double *dv,
                  double *fv) {
    for (int i = 0; i < N; ++i)
      for (int k = 0; k < 3; ++k)
        xv[3 * i + k] = os[3 * i + k] + (B[6 * i + 2 * k] * abv[2 * i] +
                                         B[6 * i + 2 * k + 1] * abv[2 * i + 1]);
    for (int seg = 0; seg <= N; ++seg) {
      const double *a = seg == 0 ? ps : xv + 3 * (seg - 1);
      const double *b = seg == N ? qs : xv + 3 * seg;
      double d[3] = {b[0] - a[0], b[1] - a[1], b[2] - a[2]};
      const double ss = std::fmax(std::sqrt(dot3(d, d)), kTiny);
      sv[seg] = ss;
      for (int j = 0; j < 3; ++j) dv[3 * seg + j] = d[j] / ss;
    }
    for (int i = 0; i < N; ++i) {
      double g[3];
      for (int k = 0; k < 3; ++k)
        g[k] = nm[i] * dv[3 * i + k] - nm[i + 1] * dv[3 * (i + 1) + k];
      for (int c = 0; c < 2; ++c)
        fv[2 * i + c] = (B[6 * i + c] * g[0] + B[6 * i + 2 + c] * g[1]) +
                        B[6 * i + 4 + c] * g[2];
    }
  };
  W.s.resize(N + 1);
  W.dh.resize(3 * (N + 1));
  W.f.resize(2 * N);
  W.A.resize(4 * N);
  W.Cm.resize(4 * (N > 1 ? N - 1 : 1));
  W.dinv.resize(4 * N);
  W.y.resize(2 * N);
  W.delta.resize(2 * N);
  W.cand.resize(2 * N);
  W.fc.resize(2 * N);
  W.sc.resize(N + 1);
  W.dhc.resize(3 * (N + 1));
  std::vector<double> &xv = W.xv, &xc = W.xc;
  xv.resize(3 * N);
  xc.resize(3 * N);
  // B_i^T w B_j for w = (n/s)(I - d d^T)
  auto btwb = [&](int i, int j, double n_over_s, const double *d,
                  double out[2][2]) {
    double w[3][3], wb[3][2];
    for (int k = 0; k < 3; ++k)
      for (int l = 0; l < 3; ++l)
        w[k][l] = n_over_s * ((k == l ? 1.0 : 0.0) - d[k] * d[l]);
    for (int k = 0; k < 3; ++k)
      for (int c = 0; c < 2; ++c)
        wb[k][c] = (w[k][0] * B[6 * j + c] + w[k][1] * B[6 * j + 2 + c]) +
                   w[k][2] * B[6 * j + 4 + c];
    for (int r = 0; r < 2; ++r)
      for (int c = 0; c < 2; ++c)
        out[r][c] = (B[6 * i + r] * wb[0][c] + B[6 * i + 2 + r] * wb[1][c]) +
                    B[6 * i + 4 + r] * wb[2][c];
  };
  for (int it = 0; it < P.n_newton; ++it) {
    geom(ab.data(), xv.data(), W.s.data(), W.dh.data(), W.f.data());
    for (int i = 0; i < N; ++i) {
      // B_i^T (w_i + w_{i+1}) B_i + mu I
      double a1[2][2], a2[2][2];
      btwb(i, i, nm[i] / W.s[i], &W.dh[3 * i], a1);
      btwb(i, i, nm[i + 1] / W.s[i + 1], &W.dh[3 * (i + 1)], a2);
      for (int r = 0; r < 2; ++r)
        for (int c = 0; c < 2; ++c)
          W.A[4 * i + 2 * r + c] =
              a1[r][c] + a2[r][c] + (r == c ? mu : 0.0);
    }
    for (int i = 0; i + 1 < N; ++i) {
      double cm[2][2];
      btwb(i, i + 1, nm[i + 1] / W.s[i + 1], &W.dh[3 * (i + 1)], cm);
      for (int r = 0; r < 2; ++r)
        for (int c = 0; c < 2; ++c) W.Cm[4 * i + 2 * r + c] = -cm[r][c];
    }
    // block Thomas (refraction_joint.py:218-246) on A delta = -f
    double dprev[2][2] = {{0, 0}, {0, 0}}, yprev[2] = {0, 0};
    for (int i = 0; i < N; ++i) {
      double cp[2][2] = {{0, 0}, {0, 0}};
      if (i > 0)
        for (int r = 0; r < 2; ++r)
          for (int c = 0; c < 2; ++c) cp[r][c] = W.Cm[4 * (i - 1) + 2 * r + c];
      double cpt[2][2];  // cp^T dinv_prev
      for (int r = 0; r < 2; ++r)
        for (int c = 0; c < 2; ++c)
          cpt[r][c] = cp[0][r] * dprev[0][c] + cp[1][r] * dprev[1][c];
      double m[2][2];
      for (int r = 0; r < 2; ++r)
        for (int c = 0; c < 2; ++c)
          m[r][c] = W.A[4 * i + 2 * r + c] -
                    (cpt[r][0] * cp[0][c] + cpt[r][1] * cp[1][c]);
      double di[2][2];
      inv2(m, di);
      double yi[2];
      for (int r = 0; r < 2; ++r)
        yi[r] = -W.f[2 * i + r] - (cpt[r][0] * yprev[0] + cpt[r][1] * yprev[1]);
      for (int r = 0; r < 2; ++r) {
        W.y[2 * i + r] = yi[r];
        for (int c = 0; c < 2; ++c) W.dinv[4 * i + 2 * r + c] = di[r][c];
      }
      std::memcpy(dprev, di, sizeof(di));
      yprev[0] = yi[0];
      yprev[1] = yi[1];
    }
    double dnext[2] = {0, 0};
    for (int i = N - 1; i >= 0; --i) {
      double cn[2][2] = {{0, 0}, {0, 0}};
      if (i < N - 1)
        for (int r = 0; r < 2; ++r)
          for (int c = 0; c < 2; ++c) cn[r][c] = W.Cm[4 * i + 2 * r + c];
      double rr[2];
      for (int r = 0; r < 2; ++r)
        rr[r] = W.y[2 * i + r] - (cn[r][0] * dnext[0] + cn[r][1] * dnext[1]);
      for (int r = 0; r < 2; ++r)
        W.delta[2 * i + r] = W.dinv[4 * i + 2 * r] * rr[0] +
                             W.dinv[4 * i + 2 * r + 1] * rr[1];
      dnext[0] = W.delta[2 * i];
      dnext[1] = W.delta[2 * i + 1];
    }
    double m0 = 0.0;
    for (int i = 0; i < 2 * N; ++i) m0 += W.f[i] * W.f[i];
    double lam_sel = 0.0, lam = 1.0;
    for (int j = 0; j < P.n_backtrack; ++j, lam *= 0.5) {
      for (int i = 0; i < 2 * N; ++i) W.cand[i] = ab[i] + lam * W.delta[i];
      geom(W.cand.data(), xc.data(), W.sc.data(), W.dhc.data(), W.fc.data());
      double mc = 0.0;
      for (int i = 0; i < 2 * N; ++i) mc += W.fc[i] * W.fc[i];
      if (mc < m0) {
        lam_sel = lam;
        break;
      }
    }
    for (int i = 0; i < 2 * N; ++i) ab[i] = ab[i] + lam_sel * W.delta[i];
  }
  geom(ab.data(), xv.data(), W.s.data(), W.dh.data(), W.f.data());
  for (int i = 0; i < 3 * N; ++i) x[i] = xv[i] * scale;
  // polyline p -> x_0 .. x_{N-1} -> q in metres
  double residual = 0.0;
  bool sides = true, evan = false, fin = true, res_nan = false;
  std::vector<double> &dh = W.dhp;
  dh.resize(3 * (N + 1));
  for (int seg = 0; seg <= N; ++seg) {
    const double *a = seg == 0 ? p : x + 3 * (seg - 1);
    const double *b = seg == N ? q : x + 3 * seg;
    double d[3] = {b[0] - a[0], b[1] - a[1], b[2] - a[2]};
    const double s = std::sqrt(dot3(d, d));
    s_out[seg] = s;
    fin = fin && std::isfinite(s);
    const double sc = std::fmax(s, kTiny);
    for (int j = 0; j < 3; ++j) dh[3 * seg + j] = d[j] / sc;
  }
  for (int i = 0; i < N; ++i) {
    const double *n = Nn + 3 * i;
    const double *din = &dh[3 * i], *dout = &dh[3 * (i + 1)];
    const double ct1 = dot3(n, din), ct2 = dot3(n, dout);
    double t1[3], t2[3], dG[3];
    for (int j = 0; j < 3; ++j) {
      t1[j] = din[j] - ct1 * n[j];
      t2[j] = dout[j] - ct2 * n[j];
      dG[j] = nm[i] * din[j] - nm[i + 1] * dout[j];
    }
    const double st1 = std::sqrt(dot3(t1, t1)), st2 = std::sqrt(dot3(t2, t2));
    th1[i] = std::atan2(st1, std::fabs(ct1));
    th2[i] = std::atan2(st2, std::fabs(ct2));
    const double nd = dot3(n, dG);
    const double rt[3] = {dG[0] - nd * n[0], dG[1] - nd * n[1],
                          dG[2] - nd * n[2]};
    const double res = std::sqrt(dot3(rt, rt));
    if (std::isnan(res)) res_nan = true;
    else if (res > residual) residual = res;
    const double *prev = i == 0 ? p : x + 3 * (i - 1);
    const double *next = i == N - 1 ? q : x + 3 * (i + 1);
    double a[3], b[3];
    for (int j = 0; j < 3; ++j) {
      a[j] = prev[j] - x[3 * i + j];
      b[j] = next[j] - x[3 * i + j];
    }
    sides = sides && (dot3(n, a) * dot3(n, b) < 0.0);
    evan = evan || (nm[i] * st1 > nm[i + 1] * (1.0 + 64.0 * kEps64));
    for (int j = 0; j < 3; ++j) fin = fin && std::isfinite(x[3 * i + j]);
  }
  const bool res_fin = !res_nan && std::isfinite(residual);
  const bool converged = (residual <= 1e-9) && res_fin && fin;
  valid = converged && sides && !evan && fin && res_fin;
}

void path_joint(const Params &P, const Iface *ifc, const double *p,
                const double *q, JointWork &W, PathOut &o) {
  const int N = P.ni;
  const double *nm = P.n_leg;
  // mean-plane chain (division form, 10 iterations) anchors the lookups
  std::vector<double> &O = W.O, &Nn = W.Nn, &x = W.X, &th1 = W.th1,
                      &th2 = W.th2, &s = W.S, &c_inc = W.cinc;
  O.resize(3 * N);
  Nn.resize(3 * N);
  x.resize(3 * N);
  th1.resize(N);
  th2.resize(N);
  s.resize(N + 1);
  c_inc.resize(N);
  {
    double cur[3] = {p[0], p[1], p[2]};
    for (int i = 0; i < N; ++i) {
      Crossing R;
      snell(cur, q, ifc[i].mp, ifc[i].mn, nm[i], nm[i + 1], 10, false, 1e-9,
            R);
      double pt[3], nr[3];
      lookup(ifc[i], R.x, pt, nr);
      const double nn = std::sqrt(dot3(nr, nr));
      for (int j = 0; j < 3; ++j) {
        O[3 * i + j] = pt[j];
        Nn[3 * i + j] = nr[j] / nn;
        cur[j] = R.x[j];
      }
    }
  }
  bool valid;
  joint_solve(P, p, q, O.data(), Nn.data(), W, x.data(), th1.data(),
              th2.data(), s.data(), valid);
  o.valid = valid;
  double c_inc_surf = 0.0;
  for (int i = 0; i < N; ++i) c_inc[i] = std::fmax(std::cos(th1[i]), kCMin);
  c_inc_surf = c_inc[P.k_pad];
  double tau2 = 1.0, opl = 0.0, loss = 0.0, sperp = 0.0, spar = 0.0;
  for (int i = 0; i < N; ++i) {
    const double g = fresnel_te(P.eps_leg[i], P.eps_leg[i + 1], c_inc[i]);
    tau2 = tau2 * (1.0 - g * g);
    const double cp = i < P.k_pad ? c_inc_surf : c_inc[i];
    opl = opl + nm[i] * s[i];
    loss = loss + s[i] * (P.att_leg[i] / 1000.0);
    sperp = sperp + s[i] / nm[i];
    spar = spar + s[i] / (nm[i] * cp * cp);
  }
  o.tau2 = tau2;
  o.opl = opl;
  o.loss_db = loss;
  o.sum_perp = sperp;
  o.sum_par = spar;
  o.c0 = c_inc_surf;
  o.c_last = std::fmax(std::cos(th2[N - 1]), kCMin);
  for (int j = 0; j < 3; ++j) {
    o.cur[j] = x[3 * (N - 1) + j];
    o.x_first[j] = x[j];
  }
}

}  // namespace

extern "C" {

// Smooth isotropic surface sum (coherent.py:107-128 per pair, binned with
// drop-not-wrap). Facet columns are float64 (already float32-quantised and
// in culling order); window [lo[t], hi[t]) per trace; gamma per facet when
// gamma_f is not null. field (T, n_samples) complex128 interleaved, zeroed
// here; dropped (T,).
int cpu_ref_coherent(int T, const double *pos, const int64_t *lo,
                     const int64_t *hi, const double *cen, const double *nrm,
                     const double *area, const double *e1, const double *e2,
                     const double *gamma_f, double gamma, double k, double t0,
                     double dt, double c, int n_samples, double *field,
                     double *dropped) {
#pragma omp parallel for schedule(dynamic, 1)
  for (int t = 0; t < T; ++t) {
    double *row = field + (size_t)t * n_samples * 2;
    std::memset(row, 0, sizeof(double) * 2 * n_samples);
    double drop = 0.0;
    const double *p = pos + 3 * t;
    for (int64_t i = lo[t]; i < hi[t]; ++i) {
      double d[3] = {p[0] - cen[3 * i], p[1] - cen[3 * i + 1],
                     p[2] - cen[3 * i + 2]};
      const double r = std::sqrt(dot3(d, d));
      const double cs = dot3(d, nrm + 3 * i) / r;
      double rh[3] = {d[0] / r, d[1] / r, d[2] / r};
      const double s1 = sinc_np(dot3(rh, e1 + 3 * i) * (k / kPi));
      const double s2 = sinc_np(dot3(rh, e2 + 3 * i) * (k / kPi));
      const double g = gamma_f ? gamma_f[i] : gamma;
      const double amp = (k / kTwoPi) * g * cs * area[i] * s1 * s2 / (r * r);
      const double ph = (-2.0 * k) * r;
      // j amp e^{j ph}
      const double re = -amp * std::sin(ph), im = amp * std::cos(ph);
      const double b = std::floor((2.0 * r / c - t0) / dt);
      if (b >= 0.0 && b < (double)n_samples) {
        row[2 * (size_t)b] += re;
        row[2 * (size_t)b + 1] += im;
      } else {
        drop += re * re + im * im;
      }
    }
    dropped[t] = drop;
  }
  return 0;
}

// Refracted target sum (multilayer.py:459-588 per pair) by the sequential
// chain (joint = 0) or the joint solve (joint = 1) through n_crossed
// interfaces (joint pads first). Per interface i: float32 grids gc[i], gn[i]
// (ny[i], nx[i], 3), coef[6 i..6 i+5] (rows x, y, 1), mean point mp[3 i..],
// unit mean normal mn[3 i..]. Legs n_leg, eps_leg, att_leg (n_legs >=
// n_crossed + 1 entries; the final segment takes the last leg, as
// multilayer.py:506 does).
int cpu_ref_refracted(int T, const double *pos, const int64_t *lo,
                      const int64_t *hi, const double *cen,
                      const double *nrm, const double *area, const double *e1,
                      const double *e2, const double *gamma_f, double gamma,
                      int n_crossed, int k_pad, const float *const *gc,
                      const float *const *gn, const int *ny, const int *nx,
                      const double *coef, const double *mp, const double *mn,
                      const double *n_leg, const double *eps_leg,
                      const double *att_leg, int n_legs, int joint,
                      int n_newton,
                      int n_backtrack, double k0, double t0, double dt,
                      double c, int n_samples, double *field,
                      double *dropped) {
  if (n_crossed < 1 || k_pad < 0 || k_pad >= n_crossed ||
      n_legs < n_crossed + 1 || (joint && n_legs != n_crossed + 1))
    return 1;
  std::vector<Iface> ifc(n_crossed);
  for (int i = 0; i < n_crossed; ++i) {
    ifc[i].gc = gc[i];
    ifc[i].gn = gn[i];
    ifc[i].ny = ny[i];
    ifc[i].nx = nx[i];
    for (int j = 0; j < 6; ++j) ifc[i].coef[j] = coef[6 * i + j];
    for (int j = 0; j < 3; ++j) {
      ifc[i].mp[j] = mp[3 * i + j];
      ifc[i].mn[j] = mn[3 * i + j];
    }
  }
  Params P{n_crossed, k_pad, joint, n_newton, n_backtrack, n_leg, eps_leg,
           att_leg, k0, t0, dt, c, n_samples};
  const int last = n_legs - 1;
  const double nj = n_leg[last];
  const double kj = k0 * nj;
#pragma omp parallel
  {
    JointWork W;
#pragma omp for schedule(dynamic, 1)
    for (int t = 0; t < T; ++t) {
      double *row = field + (size_t)t * n_samples * 2;
      std::memset(row, 0, sizeof(double) * 2 * n_samples);
      double drop = 0.0;
      const double *p = pos + 3 * t;
      for (int64_t i = lo[t]; i < hi[t]; ++i) {
        const double *q = cen + 3 * i;
        PathOut o;
        if (joint) path_joint(P, ifc.data(), p, q, W, o);
        else path_sequential(P, ifc.data(), p, q, o);
        double d[3] = {o.cur[0] - q[0], o.cur[1] - q[1], o.cur[2] - q[2]};
        const double s_j = std::sqrt(dot3(d, d));
        const double is = 1.0 / std::fmax(s_j, 1e-30);
        double rh[3] = {d[0] * is, d[1] * is, d[2] * is};
        const double opl = o.opl + nj * s_j;
        const double loss = o.loss_db + s_j * (att_leg[last] / 1000.0);
        const double sperp = o.sum_perp + s_j / nj;
        const double spar = o.sum_par + s_j / (nj * o.c_last * o.c_last);
        const double l_perp = n_leg[0] * sperp;
        const double l_par = n_leg[0] * o.c0 * o.c0 * spar;
        const double flux = (n_leg[0] * o.c0) / (nj * o.c_last);
        const double att_f = std::pow(10.0, -loss / 10.0);
        const double cos_t = dot3(rh, nrm + 3 * i);
        const double spread = o.tau2 * flux / (l_par * l_perp);
        const double g = gamma_f ? gamma_f[i] : gamma;
        const double s1 = sinc_np(dot3(rh, e1 + 3 * i) * (kj / kPi));
        const double s2 = sinc_np(dot3(rh, e2 + 3 * i) * (kj / kPi));
        const double amp = (kj / kTwoPi) * g * cos_t * area[i] * s1 * s2 *
                           spread * att_f;
        const double ph = -2.0 * k0 * opl;
        const double re = -amp * std::sin(ph), im = amp * std::cos(ph);
        const double b = std::floor((2.0 * opl / c - t0) / dt);
        if (o.valid && b >= 0.0 && b < (double)n_samples) {
          row[2 * (size_t)b] += re;
          row[2 * (size_t)b + 1] += im;
        } else {
          drop += re * re + im * im;
        }
      }
      dropped[t] = drop;
    }
  }
  return 0;
}

int cpu_ref_threads(void) { return omp_get_max_threads(); }

void cpu_ref_set_threads(int n) {
  if (n > 0) omp_set_num_threads(n);
}

}  // extern "C"
