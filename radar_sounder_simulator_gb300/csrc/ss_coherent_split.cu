// Split-precision surface coherent kernel.
//
// Same decomposition as the FP64 form (ss_coherent.cu). Per pair, only three
// quantities need more than float32: the slant range r (20 km at 1 mm f32
// ulp; 1e-3 rad at 450 MHz needs ~50 um), the carrier phase 2 k r and the
// fast-time bin floor((2r/c - t0)/dt). They are formed in two stages.
//
//   * Once per facet and trace block (a CTA's `tb` neighbouring traces): the
//     range r_c to the block's middle trace as a double-float (exact
//     difference of the double-float platform and the float32 centroid,
//     exact squares, rsqrt + Newton), its phase 2 k r_c reduced modulo 2 pi
//     (double-float product, two-constant Cody-Waite whose first step is
//     exact), its bin position split into an integer and a fraction, and the
//     products of q = p_c - c with the facet's normal and edge vectors.
//   * Per trace t of the block, with w = p_t - p_c (a few trace spacings):
//     r_t^2 - r_c^2 = 2 q.w + |w|^2 = N, so r_t - r_c = N / (r_c + r_t).
//     Within a block the track is straight to well under a metre, so
//     w = lam u + eps with u the block's track direction: q.u is formed
//     once per facet as a double-float, and N = 2 (lam q.u + q.eps) +
//     |w|^2 takes one exact product per pair (q.eps, |eps| < 1 m, in
//     float32). N is thus a double-float; the division
//     takes a float32 quotient and one correction against the double-float
//     denominator 2 r_c + dr, so dr = r_t - r_c is good to ~2e-11 of its
//     size (3e-9 m at |w| = 160 m; a float32 dr would carry ulp(|w|)/2 of
//     rounding: 4e-6 m at 100 m, 8e-5 rad of phase at 450 MHz). The middle
//     trace has w = 0 and its pairs are exact to the reference's
//     double-float.
//
// The bin position ubc + fc + A dr is then good to ~2e-7 bins; a pair
// within 2e-6 bins of an edge recomputes its own double-float range and
// bin (~1e-10 bins, FP32 pipe), and only within 1e-8 bins of an edge does
// the float64 round-to-nearest chain of the oracle decide, so bins are
// bit-identical to the float64 form while the slow FP64 pipe almost never
// runs. A block whose traces lie more than 160 m from its middle trace or
// more than 1 m off its straight track line (sparse or crooked tracks)
// takes a reference per trace instead (w = 0 for every pair).
//
// Everything else (incidence, sincs, taper, antenna gain, roughness series)
// runs in float32 from q + w and the facet's per-block products;
// histograms accumulate float32 per CTA chunk and the reduce kernel sums
// the chunks by float32 two-sums (~2^-48 relative).
#include <algorithm>

#include "ss_coherent.cuh"
#include "ss_df.cuh"
#include "ss_f32.cuh"

namespace ss {

// Widest trace block (largest |p_t - p_c|, metres) served by one reference:
// eight traces at 40 m.
constexpr float kWideBlock = 160.0f;
// Largest offset of a block's traces from its straight track line
// (metres): q.eps is formed in float32, ~1e-3 |eps| m^2 of rounding.
constexpr double kBlockBend = 1.0;
// Bin-edge band of the per-trace bin position (~10x its error).
constexpr float kBinBand = 2e-6f;

// Integer value of an integral float with |x| < 2^22: adding 1.5 * 2^23
// places it in the low mantissa bits (exact), read back as an integer --
// two FP32/integer-pipe instructions instead of a conversion.
__device__ __forceinline__ int small_int(float x) {
  return __float_as_int(x + 12582912.0f) - 0x4B400000;
}

// One CTA's work item: facet chunk `chunk` of trace block `group`. Shared
// by the one-call kernel (item = block index) and the batched persistent
// kernel (item pulled from a work queue).
template <int ROUGH>
__device__ __forceinline__ void coherent_split_cta(const CoArgs &a,
                                                   const SplitConsts &k,
                                                   int chunk, int group,
                                                   unsigned char *smem_raw) {
  const int hs = split_hist_stride(a.n_seg);
  float *hre = reinterpret_cast<float *>(smem_raw);
  float *him = hre + (size_t)a.tb * hs;
  float *inv = him + (size_t)a.tb * hs;  // 1/m of the series (rough only)
  __shared__ float s_ph[SS_MAX_TB][3], s_pl[SS_MAX_TB][3];
  __shared__ double s_p64[SS_MAX_TB][3];
  // trace offsets w = p_t - p_c = lam u + eps, u the block's track
  // direction: w (float) and |w|^2 (hi), lam (hi, lo) and |w|^2 (lo), eps
  __shared__ float4 s_w[SS_MAX_TB];
  __shared__ float4 s_lw[SS_MAX_TB];
  __shared__ float4 s_we[SS_MAX_TB];
  __shared__ float s_tu[6];  // u as hi (3) and lo (3)
  __shared__ float s_u[SS_MAX_TB][3];
  __shared__ float s_pv[SS_MAX_TB][6];
  __shared__ int2 s_win[SS_MAX_TB];
  __shared__ float s_drop[SS_MAX_TB];
  __shared__ float s_pat[SS_PAT_MAX];
  __shared__ float s_slope[SS_PAT_MAX / 2];  // tabulated pattern's slopes
  __shared__ float s_tinv;
  __shared__ float s_fad[SS_FAD_N];
  __shared__ int s_rng[2];
  __shared__ int s_next;
  __shared__ int s_ref;      // the block's reference trace; -1: per trace

  const int t_base = group * a.tb;
  const int nt = min(a.tb, a.T - t_base);
  const int tid = threadIdx.x;
  int pa_len, pb_len;
  pattern_lengths(a.pat_kind, a.pat_n, pa_len, pb_len);

  if (tid < nt) {
    const int t = t_base + tid;
    const int tc = t_base + nt / 2;
    double w[3], w2 = 0.0;
    for (int j = 0; j < 3; ++j) {
      const double pj = a.pos[3 * t + j];
      const df v = df_from_double(pj);
      s_ph[tid][j] = v.hi;
      s_pl[tid][j] = v.lo;
      s_p64[tid][j] = pj;
      s_u[tid][j] = a.uct ? (float)a.uct[3 * t + j] : 0.0f;
      w[j] = pj - a.pos[3 * tc + j];
      w2 += w[j] * w[j];
    }
    const float w2h = (float)w2;
    s_w[tid] = make_float4((float)w[0], (float)w[1], (float)w[2], w2h);
    s_lw[tid].z = (float)(w2 - (double)w2h);
    for (int j = 0; j < 6; ++j)
      s_pv[tid][j] =
          (a.pv && j < a.pv_len) ? (float)a.pv[a.pv_len * t + j] : 0.0f;
    long lo = (long)a.off[t] * a.bs;
    long hi = min((long)(a.off[t] + a.n_win) * a.bs, (long)a.N);
    s_win[tid] = make_int2((int)min(lo, (long)a.N), (int)hi);
    s_drop[tid] = 0.0f;
  }
  for (int j = tid; j < pa_len; j += blockDim.x) s_pat[j] = (float)a.pa[j];
  for (int j = tid; j < pb_len; j += blockDim.x)
    s_pat[pa_len + j] = (float)a.pb[j];
  if (ROUGH == SS_ROUGH_GAUSS_FULL && tid < SS_FAD_N)
    s_fad[tid] = (float)a.fad.a[tid];
  for (int j = tid; j < 2 * a.tb * hs; j += blockDim.x) hre[j] = 0.0f;
  if (ROUGH != SS_ROUGH_NONE) fill_inv_table(inv, a.n_terms, tid, blockDim.x);
  __syncthreads();
  if (a.pat_kind == SS_PAT_TABULATED)
    tab_slopes(a.pat_n, s_pat, s_pat + pa_len, s_slope, &s_tinv, tid,
               blockDim.x);
  if (tid == 0) {
    int lo = s_win[0].x, hi = s_win[0].y;
    for (int j = 1; j < nt; ++j) {
      lo = min(lo, s_win[j].x);
      hi = max(hi, s_win[j].y);
    }
    long len = max(hi - lo, 0);
    s_rng[0] = lo + (int)(len * chunk / a.n_chunks);
    s_rng[1] = lo + (int)(len * (chunk + 1) / a.n_chunks);
    s_next = s_rng[0];
    // track direction u of the block (first to last trace) and each
    // trace's offset w = lam u + eps from the middle trace, in float64
    const int c = nt / 2;
    double u[3], un = 0.0;
    for (int j = 0; j < 3; ++j) {
      u[j] = s_p64[nt - 1][j] - s_p64[0][j];
      un += u[j] * u[j];
    }
    un = sqrt(un);
    for (int j = 0; j < 3; ++j) u[j] = un > 0.0 ? u[j] / un : (j == 0);
    double wmax = 0.0, emax = 0.0;
    for (int t = 0; t < nt; ++t) {
      double w[3], lam = 0.0, e2 = 0.0;
      for (int j = 0; j < 3; ++j) {
        w[j] = s_p64[t][j] - s_p64[c][j];
        lam += w[j] * u[j];
      }
      float e[3];
      for (int j = 0; j < 3; ++j) {
        const double ej = w[j] - lam * u[j];
        e[j] = (float)ej;
        e2 += ej * ej;
      }
      const float lh = (float)lam;
      s_lw[t].x = lh;
      s_lw[t].y = (float)(lam - (double)lh);
      s_we[t] = make_float4(e[0], e[1], e[2], 0.0f);
      wmax = fmax(wmax, sqrt(w[0] * w[0] + w[1] * w[1] + w[2] * w[2]));
      emax = fmax(emax, sqrt(e2));
    }
    for (int j = 0; j < 3; ++j) {
      s_tu[j] = (float)u[j];
      s_tu[3 + j] = (float)(u[j] - (double)s_tu[j]);
    }
    s_ref = wmax <= kWideBlock && emax <= kBlockBend ? c : -1;
  }
  __syncthreads();

  const float nsf = (float)a.n_samples;
  const int ref = s_ref;
  // lane l meets the block's traces starting at trace l mod nt, so the 32
  // neighbouring facets of a warp -- often in one bin -- spread their
  // histogram atomics over the block's traces; dropped power collects per
  // thread and step (L1-resident local memory) and reaches shared memory
  // once per trace at the end
  const int rot = (tid & 31) % max(nt, 1);
  float dropl[SS_MAX_TB];
#pragma unroll
  for (int j = 0; j < SS_MAX_TB; ++j) dropl[j] = 0.0f;
  // warps take 32 consecutive facets at a time from a shared counter (the
  // roughness series makes pair costs uneven)
  const int lane = tid & 31;
  const int i_end = s_rng[1];
  for (;;) {
    int base = 0;
    if (lane == 0) base = atomicAdd(&s_next, 32);
    base = __shfl_sync(0xffffffffu, base, 0);
    if (base >= i_end) break;
    const int i = base + lane;
    if (i >= i_end) continue;
    const float cx = a.F.cx[i], cy = a.F.cy[i], cz = a.F.cz[i];
    const float nx = a.F.nx[i], ny = a.F.ny[i], nz = a.F.nz[i];
    const float e1x = a.F.e1x[i], e1y = a.F.e1y[i], e1z = a.F.e1z[i];
    const float e2x = a.F.e2x[i], e2y = a.F.e2y[i], e2z = a.F.e2z[i];
    const float area = a.F.area[i];
    const float gam = a.F.gamma_f32 ? a.F.gamma_f32[i] : k.gamma;
    const float amp_f = k.amp_pref * gam * area;
    float sg = 0.f, lc = 0.f, phr = 0.f, phi = 0.f, l1 = 0.f, l2 = 0.f;
    if (ROUGH != SS_ROUGH_NONE) {
      sg = a.F.sigma ? a.F.sigma[i] : k.sigma;
      lc = a.F.corr ? a.F.corr[i] : k.corr;
      phr = a.F.phasor[2 * i];
      phi = a.F.phasor[2 * i + 1];
      l1 = sqrtf(dot3f(e1x, e1y, e1z, e1x, e1y, e1z));
      l2 = sqrtf(dot3f(e2x, e2y, e2z, e2x, e2y, e2z));
    }

    // --- per-facet reference at the platform of trace `j` ---
    float qhx, qhy, qhz, qlx, qly, qlz, rch, phc, ubc, fc, cosc, qe1, qe2;
    float rcl, xnx = 0.f, xny = 0.f, xnz = 0.f;  // q x n (taper's sin^2)
    float quh, qul;                               // q.u as a double-float
    auto reference = [&](int j) {
      float e;
      two_sum(s_ph[j][0], -cx, qhx, e);
      fast_two_sum(qhx, e + s_pl[j][0], qhx, qlx);
      two_sum(s_ph[j][1], -cy, qhy, e);
      fast_two_sum(qhy, e + s_pl[j][1], qhy, qly);
      two_sum(s_ph[j][2], -cz, qhz, e);
      fast_two_sum(qhz, e + s_pl[j][2], qhz, qlz);
      // S = |q|^2 (double-float), r_c = sqrt(S): rsqrt + one Newton step
      float sx, ex, sy, ey, sz, ez, s1, e1_, Sh, e2_;
      two_prod(qhx, qhx, sx, ex);
      two_prod(qhy, qhy, sy, ey);
      two_prod(qhz, qhz, sz, ez);
      two_sum(sx, sy, s1, e1_);
      two_sum(s1, sz, Sh, e2_);
      float Sl = (e1_ + e2_) + (ex + ey + ez) +
                 2.0f * (qhx * qlx + qhy * qly + qhz * qlz);
      fast_two_sum(Sh, Sl, Sh, Sl);
      const float y = rsqrtf(Sh);
      const float r0 = Sh * y;
      const float res = __fmaf_rn(-r0, r0, Sh) + Sl;
      fast_two_sum(r0, res * (0.5f * y), rch, rcl);
      // phase 2 k r_c mod 2 pi (double-float product, exact first step)
      float ph, pe;
      two_prod(k.K2h, rch, ph, pe);
      const float pl = pe + __fmaf_rn(k.K2h, rcl, k.K2l * rch);
      const float n2 = rintf(ph * 0.159154943091895336f);
      const float red = __fmaf_rn(-n2, 6.28318548202514648f, ph);
      phc = __fmaf_rn(-n2, -1.74845553146951e-07f, red) + pl;
      // bin position u = r_c A - B = ubc + fc
      float up, ue, us, ue2;
      two_prod(rch, k.Ah, up, ue);
      two_sum(up, -k.Bh, us, ue2);
      const float ul = (ue2 + ue) + __fmaf_rn(rch, k.Al, rcl * k.Ah) - k.Bl;
      ubc = floorf(us);
      fc = (us - ubc) + ul;
      // cos of incidence at the reference, q.n / r_c with q.n from exact
      // products and a corrected division (~1 ulp): the 0.05 taper turns a
      // cosine error into a ~400x larger relative amplitude error
      float pnx, enx, pny, eny, pnz, enz, sn1, es1, qnh, es2;
      two_prod(qhx, nx, pnx, enx);
      two_prod(qhy, ny, pny, eny);
      two_prod(qhz, nz, pnz, enz);
      two_sum(pnx, pny, sn1, es1);
      two_sum(sn1, pnz, qnh, es2);
      const float qnl = (es1 + es2) + (enx + eny + enz) +
                        dot3f(qlx, qly, qlz, nx, ny, nz);
      const float yc = __frcp_rn(rch);
      const float c0 = qnh * yc;
      const float ce = __fmaf_rn(-c0, rch, qnh) + qnl - c0 * rcl;
      cosc = __fmaf_rn(ce, yc, c0);
      if (a.taper) {
        xnx = __fmaf_rn(qhy, nz, -qhz * ny) + __fmaf_rn(qly, nz, -qlz * ny);
        xny = __fmaf_rn(qhz, nx, -qhx * nz) + __fmaf_rn(qlz, nx, -qlx * nz);
        xnz = __fmaf_rn(qhx, ny, -qhy * nx) + __fmaf_rn(qlx, ny, -qly * nx);
      }
      // q.u (u the block's track direction) as a double-float
      {
        float p1, e1, p2, e2, p3, e3, s1, f1, s2, f2;
        two_prod(qhx, s_tu[0], p1, e1);
        two_prod(qhy, s_tu[1], p2, e2);
        two_prod(qhz, s_tu[2], p3, e3);
        two_sum(p1, p2, s1, f1);
        two_sum(s1, p3, s2, f2);
        const float l = (f1 + f2) + (e1 + e2 + e3) +
                        dot3f(qlx, qly, qlz, s_tu[0], s_tu[1], s_tu[2]) +
                        dot3f(qhx, qhy, qhz, s_tu[3], s_tu[4], s_tu[5]);
        fast_two_sum(s2, l, quh, qul);
      }
      // products with the edge vectors (q_lo matters for the sinc
      // arguments: k (r_hat . e) reaches tens of radians)
      qe1 = dot3f(qhx, qhy, qhz, e1x, e1y, e1z) +
            dot3f(qlx, qly, qlz, e1x, e1y, e1z);
      qe2 = dot3f(qhx, qhy, qhz, e2x, e2y, e2z) +
            dot3f(qlx, qly, qlz, e2x, e2y, e2z);
    };

    // --- bin of a pair near an edge, decided as the float64 form does ---
    // First the pair's own double-float range (exact difference of the
    // double-float platform and the float32 centroid, exact squares, rsqrt +
    // Newton) and bin position u = r A - B, accurate to ~1e-10 bins on the
    // FP32 pipe; the float64 round-to-nearest chain of the oracle (~1e-12
    // bins from the exact u) runs only within 1e-8 bins of an edge, where
    // the two could round differently.
    auto exact_bin = [&](int tt, float &fb, float &frac) {
      float dxh, dxl, dyh, dyl, dzh, dzl, e;
      two_sum(s_ph[tt][0], -cx, dxh, e);
      fast_two_sum(dxh, e + s_pl[tt][0], dxh, dxl);
      two_sum(s_ph[tt][1], -cy, dyh, e);
      fast_two_sum(dyh, e + s_pl[tt][1], dyh, dyl);
      two_sum(s_ph[tt][2], -cz, dzh, e);
      fast_two_sum(dzh, e + s_pl[tt][2], dzh, dzl);
      float sx, ex, sy, ey, sz, ez, s1, e1_, Sh, e2_;
      two_prod(dxh, dxh, sx, ex);
      two_prod(dyh, dyh, sy, ey);
      two_prod(dzh, dzh, sz, ez);
      two_sum(sx, sy, s1, e1_);
      two_sum(s1, sz, Sh, e2_);
      float Sl = (e1_ + e2_) + (ex + ey + ez) +
                 2.0f * (dxh * dxl + dyh * dyl + dzh * dzl);
      fast_two_sum(Sh, Sl, Sh, Sl);
      const float y = rsqrtf(Sh);
      const float r0 = Sh * y;
      const float res = __fmaf_rn(-r0, r0, Sh) + Sl;
      float rh, rl;
      fast_two_sum(r0, res * (0.5f * y), rh, rl);
      float up, ue, us, ue2;
      two_prod(rh, k.Ah, up, ue);
      two_sum(up, -k.Bh, us, ue2);
      const float ul = (ue2 + ue) + __fmaf_rn(rh, k.Al, rl * k.Ah) - k.Bl;
      float f2 = floorf(us);
      float fr2 = (us - f2) + ul;
      if (fr2 < 0.0f) { f2 -= 1.0f; fr2 += 1.0f; }
      else if (fr2 >= 1.0f) { f2 += 1.0f; fr2 -= 1.0f; }
      if (fr2 < 1e-8f || fr2 > 1.0f - 1e-8f) {
        const double ddx = __dsub_rn(s_p64[tt][0], (double)cx);
        const double ddy = __dsub_rn(s_p64[tt][1], (double)cy);
        const double ddz = __dsub_rn(s_p64[tt][2], (double)cz);
        const double rd = __dsqrt_rn(__dadd_rn(
            __dadd_rn(__dmul_rn(ddx, ddx), __dmul_rn(ddy, ddy)),
            __dmul_rn(ddz, ddz)));
        const double u64 = __ddiv_rn(
            __dsub_rn(__ddiv_rn(__dmul_rn(2.0, rd), a.c), a.t0), a.dt);
        const double f64b = floor(u64);
        f2 = (float)f64b;
        fr2 = (float)(u64 - f64b);
      }
      fb = f2;
      frac = fr2;
    };

    // --- one pair: facet i, trace tt at offset w = lam u + eps ---
    auto pair = [&](int tt, float4 w, float4 lw, float4 we) -> float {
      // N = r_t^2 - r_c^2 = 2 q.w + |w|^2 as a double-float, with
      // q.w = lam (q.u) + q.eps: one exact product of the hi parts, the lo
      // parts' products and q.eps (|eps| < 1 m) in float
      float pq, eq;
      two_prod(lw.x, quh, pq, eq);
      const float lo = eq + __fmaf_rn(lw.x, qul, lw.y * quh) +
                       dot3f(qhx, qhy, qhz, we.x, we.y, we.z);
      // (2 lo + |w|^2 can reach 4e4 m^2 on a bent block: it joins the
      // compensated sum, so N comes out renormalised)
      float Nh, g;
      two_sum(2.0f * pq, __fmaf_rn(2.0f, lo, w.w), Nh, g);
      const float Nl = g + lw.z;
      // float32 r_t for the amplitude and a first dr, then dr = N / D with
      // D = r_c + r_t = 2 r_c + dr as a double-float and one correction:
      // dr is then good to ~2e-11 of its size
      const float rr = __fmaf_rn(rch, rch, Nh);
      const float inv_r = rsqrtf(rr);
      const float dr0 = __fdividef(Nh, rch + rr * inv_r);
      float Dh, De;
      fast_two_sum(2.0f * rch, dr0, Dh, De);
      const float Dl = __fmaf_rn(2.0f, rcl, De);
      const float iD = __fdividef(1.0f, Dh);
      const float dr = Nh * iD;
      const float drl =
          (__fmaf_rn(-dr, Dh, Nh) + __fmaf_rn(-dr, Dl, Nl)) * iD;
      // --- amplitude (float32) ---
      // cos_t = (q.n + w.n) / r_t = cos_c + (w.n - cos_c dr) / r_t
      const float cosv = __fmaf_rn(
          __fmaf_rn(-cosc, dr, dot3f(nx, ny, nz, w.x, w.y, w.z)), inv_r,
          cosc);
      const float d1 = (qe1 + dot3f(e1x, e1y, e1z, w.x, w.y, w.z)) * inv_r;
      const float d2 = (qe2 + dot3f(e2x, e2y, e2z, w.x, w.y, w.z)) * inv_r;
      const float inv_r2 = inv_r * inv_r;
      float amp = amp_f * cosv * sinc32(k.k * d1) * sinc32(k.k * d2) *
                  inv_r2;
      if (a.taper) {
        // tan^2 = sin^2 / cos^2 with sin^2 = |(q + w) x n|^2 / r_t^2 (no
        // 1 - cos^2 cancellation near nadir)
        const float sx = xnx + __fmaf_rn(w.y, nz, -w.z * ny);
        const float sy = xny + __fmaf_rn(w.z, nx, -w.x * nz);
        const float sz = xnz + __fmaf_rn(w.x, ny, -w.y * nx);
        const float s2 = dot3f(sx, sy, sz, sx, sy, sz) * inv_r2;
        const float cc = fminf(fmaxf(cosv, 1e-9f), 1.0f);
        amp *= __expf(-__fdividef(s2, cc * cc) * k.taper_inv);
      }
      float cr = amp, ci = 0.0f;
      if (ROUGH != SS_ROUGH_NONE) {
        const float kk = 2.0f * k.k * cosv;
        const float dp = d_phi32<ROUGH>(a.n_terms, inv, s_fad, k.fadL,
                                        sg, lc, kk, 2.0f * k.k * d1 / l1,
                                        2.0f * k.k * d2 / l2, l1, l2);
        const float amp_i = area > 0.0f ? k.amp_pref * gam * cosv * inv_r2 *
                                              sqrtf(dp)
                                        : 0.0f;
        const float sk = sg * kk;
        const float att = __expf(-0.5f * sk * sk);
        cr = amp * att + amp_i * phr;
        ci = amp_i * phi;
      }
      // --- carrier phase: phc + 2 k dr (exact product, exact first step) ---
      float pp, pe;
      two_prod(k.K2h, dr, pp, pe);
      pe += __fmaf_rn(k.K2h, drl, k.K2l * dr);
      const float n2 = rintf(pp * 0.159154943091895336f);
      float red = __fmaf_rn(-n2, 6.28318548202514648f, pp);
      red = __fmaf_rn(-n2, -1.74845553146951e-07f, red) + (pe + phc);
      float sn, cs;
      __sincosf(red, &sn, &cs);
      float re = cr * sn - ci * cs;
      float im = cr * cs + ci * sn;
      const float qtx = qhx + w.x, qty = qhy + w.y, qtz = qhz + w.z;
      if (a.pat_kind != SS_PAT_ISOTROPIC) {
        const float g =
            a.pat_kind == SS_PAT_TABULATED
                ? gain_tab32(a.pat_n, s_pat, s_pat + pa_len, s_slope, s_tinv,
                             s_pv[tt], -qtx * inv_r, -qty * inv_r,
                             -qtz * inv_r)
                : gain32(a.pat_kind, a.pat_n, pa_len, s_pat, s_pv[tt],
                               -qtx * inv_r, -qty * inv_r, -qtz * inv_r);
        re *= g * g;
        im *= g * g;
      }
      // --- bin: u = ubc + fc + A dr, exact re-bin near edges ---
      float dh, de, sb, se;
      two_prod(k.Ah, dr, dh, de);
      two_sum(fc, dh, sb, se);
      const float fl = floorf(sb);
      float frac = (sb - fl) + (se + de + __fmaf_rn(k.Ah, drl, k.Al * dr));
      float fb = ubc + fl;
      if (frac < 0.0f) { fb -= 1.0f; frac += 1.0f; }
      else if (frac >= 1.0f) { fb += 1.0f; frac -= 1.0f; }
      if ((frac < kBinBand || frac > 1.0f - kBinBand) && fb > -4.0f &&
          fb < nsf + 4.0f)
        exact_bin(tt, fb, frac);
      int side_off = 0;
      if (a.split &&
          dot3f(-qtx, -qty, -qtz, s_u[tt][0], s_u[tt][1], s_u[tt][2]) > 0.0f)
        side_off = a.n_samples;
      const int row = tt * hs + side_off;
      float drop = 0.0f;
      if (a.interp) {
        const float wq[2] = {1.0f - frac, frac};
#pragma unroll
        for (int q = 0; q < 2; ++q) {
          const float bq = fb + (float)q;
          const float pr = re * wq[q], pim = im * wq[q];
          if (bq >= 0.0f && bq < nsf) {
            const int j = row + small_int(bq);
            atomicAdd(hre + j, pr);
            atomicAdd(him + j, pim);
          } else {
            drop += pr * pr + pim * pim;
          }
        }
      } else if (fb >= 0.0f && fb < nsf) {
        const int j = row + small_int(fb);
        atomicAdd(hre + j, re);
        atomicAdd(him + j, im);
      } else {
        drop = re * re + im * im;
      }
      return drop;
    };

    if (ref >= 0) {
      reference(ref);
#pragma unroll 1
      for (int st = 0; st < nt; ++st) {
        const int tt = rot + st < nt ? rot + st : rot + st - nt;
        const int2 win = s_win[tt];
        if (i >= win.x && i < win.y) {
          const float d = pair(tt, s_w[tt], s_lw[tt], s_we[tt]);
          if (d != 0.0f) dropl[st] += d;
        }
      }
    } else {
      for (int tt = 0; tt < nt; ++tt) {
        const int2 win = s_win[tt];
        if (i < win.x || i >= win.y) continue;
        reference(tt);
        const float4 z = make_float4(0.f, 0.f, 0.f, 0.f);
        const float d = pair(tt, z, z, z);
        if (d != 0.0f) atomicAdd(&s_drop[tt], d);
      }
    }
  }
#pragma unroll
  for (int st = 0; st < SS_MAX_TB; ++st) {
    if (st < nt && dropl[st] != 0.0f) {
      const int tt = rot + st < nt ? rot + st : rot + st - nt;
      atomicAdd(&s_drop[tt], dropl[st]);
    }
  }
  __syncthreads();
  float2 *part = reinterpret_cast<float2 *>(a.part);
  for (int tt = 0; tt < nt; ++tt) {
    const size_t base = ((size_t)chunk * a.T + t_base + tt) * a.n_seg;
    for (int j = tid; j < a.n_seg; j += blockDim.x)
      part[base + j] = make_float2(hre[tt * hs + j], him[tt * hs + j]);
  }
  if (tid < nt)
    a.part_drop[(size_t)chunk * a.T + t_base + tid] = (double)s_drop[tid];
}

// Smooth facets: up to 512 threads, 64 registers (two 512-thread or four
// 256-thread CTAs per SM). With the roughness series inlined: up to 256
// threads, 80 registers (three CTAs per SM, no spills).
#define SS_SPLIT_MAXT(R) ((R) == SS_ROUGH_NONE ? 512 : 256)
#define SS_SPLIT_MINB(R) ((R) == SS_ROUGH_NONE ? 2 : 3)

template <int ROUGH>
__global__ void __launch_bounds__(SS_SPLIT_MAXT(ROUGH), SS_SPLIT_MINB(ROUGH))
coherent_split_kernel(CoArgs a, SplitConsts k) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  coherent_split_cta<ROUGH>(a, k, blockIdx.x, blockIdx.y, smem_raw);
}

// Batched persistent kernel: CTAs pull (job, trace block, facet chunk)
// items from a global counter until the queue is empty, so jobs of very
// different sizes share one launch without tail effects. Two builds:
// MAXT = 512 (smooth facets only, 64 registers, two CTAs per SM) and
// MAXT = 256 (80 registers, three CTAs per SM, no spills); the batch's CTA
// size picks one, and the autotuner times both.
template <int ROUGH, int MAXT>
__global__ void __launch_bounds__(MAXT, MAXT == 512 ? 2 : 3)
coherent_batch_split_kernel(const BatchJob *jobs, int n_jobs,
                            long long n_items, unsigned long long *counter) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ long long s_item;
  __shared__ int s_job;
  for (;;) {
    __syncthreads();  // the previous item's shared memory is free
    if (threadIdx.x == 0) {
      const long long it = (long long)atomicAdd(counter, 1ull);
      s_item = it;
      s_job = it < n_items ? batch_find_job(jobs, n_jobs, it, true) : 0;
    }
    __syncthreads();
    const long long it = s_item;
    if (it >= n_items) break;
    const BatchJob &J = jobs[s_job];
    const long long local = it - J.item0;
    coherent_split_cta<ROUGH>(J.a, J.k, (int)(local % J.n_chunks),
                              (int)(local / J.n_chunks), smem_raw);
  }
}

// The build of the batch kernel for a CTA size (512 only for smooth
// facets, which the batch layout enforces).
template <int ROUGH>
static void *batch_split_fn(int threads) {
  if constexpr (ROUGH == SS_ROUGH_NONE) {
    if (threads > 256)
      return reinterpret_cast<void *>(
          coherent_batch_split_kernel<ROUGH, 512>);
  }
  return reinterpret_cast<void *>(coherent_batch_split_kernel<ROUGH, 256>);
}

static void *batch_split_fn_kind(int rough_kind, int threads) {
  switch (rough_kind) {
    case SS_ROUGH_NONE: return batch_split_fn<SS_ROUGH_NONE>(threads);
    case SS_ROUGH_GAUSS_FULL:
      return batch_split_fn<SS_ROUGH_GAUSS_FULL>(threads);
    case SS_ROUGH_GAUSS_AREA:
      return batch_split_fn<SS_ROUGH_GAUSS_AREA>(threads);
    default: return batch_split_fn<SS_ROUGH_EXP_AREA>(threads);
  }
}

int coherent_batch_split_launch(const BatchJob *jobs, int n_jobs,
                                long long n_items,
                                unsigned long long *counter, int rough_kind,
                                int threads, int ctas, size_t smem,
                                cudaStream_t st) {
  // the dynamic shared-memory limit was raised at prepare time, so this
  // path holds only stream operations (it may run under graph capture)
  void *fn = batch_split_fn_kind(rough_kind, threads);
  void *args[] = {(void *)&jobs, (void *)&n_jobs, (void *)&n_items,
                  (void *)&counter};
  return cuda_status(cudaLaunchKernel(fn, dim3(ctas), dim3(threads), args,
                                      smem, st),
                     "batch split launch");
}

int batch_split_blocks_per_sm(int rough_kind, int threads, size_t smem) {
  // raise the kernel's dynamic shared-memory limit to the largest size any
  // prepared batch uses (never lowered: earlier batches stay launchable)
  static size_t limit[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  const int r = (rough_kind & 3) * 2 + (threads > 256 ? 1 : 0);
  limit[r] = std::max(limit[r], smem);
  void *fn = batch_split_fn_kind(rough_kind, threads);
  int n = 0;
  cudaError_t e = cudaFuncSetAttribute(
      fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)limit[r]);
  if (e == cudaSuccess)
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, fn, threads, smem);
  return e == cudaSuccess ? n : 0;
}

SplitConsts coherent_split_consts(const CoArgs &a) {
  SplitConsts k{};
  k.k = (float)a.k;
  k.amp_pref = (float)(a.k / kTwoPi);
  k.gamma = (float)a.gamma;
  k.taper_inv = a.taper ? (float)(1.0 / (2.0 * a.taper_s * a.taper_s)) : 0.f;
  const df k2 = df_from_double(2.0 * a.k);
  k.K2h = k2.hi;
  k.K2l = k2.lo;
  const df A = df_from_double(2.0 / (a.c * a.dt));
  const df B = df_from_double(a.t0 / a.dt);
  k.Ah = A.hi;
  k.Al = A.lo;
  k.Bh = B.hi;
  k.Bl = B.lo;
  k.fadL = (float)a.fad.L;
  k.sigma = (float)a.sigma;
  k.corr = (float)a.corr;
  return k;
}

int coherent_split_launch(CoArgs &a, const Plan &p, cudaStream_t st) {
  int pa_len, pb_len;
  pattern_lengths(a.pat_kind, a.pat_n, pa_len, pb_len);
  if (pa_len + pb_len > SS_PAT_MAX) {
    set_error("antenna table too large for the split kernel");
    return SS_ERR_UNSUPPORTED;
  }
  const SplitConsts k = coherent_split_consts(a);
  dim3 grid(p.n_chunks, p.n_groups);
  size_t smem = split_hist_bytes(a.n_seg, p.tb) +
                (a.rough_kind ? (size_t)(a.n_terms + 1) * sizeof(float) : 0);
  cudaError_t e = cudaSuccess;
  switch (a.rough_kind) {
#define SS_LAUNCH(R)                                                         \
  case R:                                                                    \
    e = cudaFuncSetAttribute(coherent_split_kernel<R>,                       \
                             cudaFuncAttributeMaxDynamicSharedMemorySize,    \
                             (int)smem);                                     \
    if (e != cudaSuccess) return cuda_status(e, "coherent_split smem");      \
    coherent_split_kernel<R><<<grid, p.threads, smem, st>>>(a, k);           \
    break;
    SS_LAUNCH(SS_ROUGH_NONE)
    SS_LAUNCH(SS_ROUGH_GAUSS_FULL)
    SS_LAUNCH(SS_ROUGH_GAUSS_AREA)
    SS_LAUNCH(SS_ROUGH_EXP_AREA)
#undef SS_LAUNCH
    default:
      return SS_ERR_ARG;
  }
  return cuda_status(cudaGetLastError(), "coherent_split launch");
}

}  // namespace ss
