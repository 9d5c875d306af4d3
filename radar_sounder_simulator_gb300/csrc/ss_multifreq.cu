// Frequency-sampled facet synthesis ("Mode F"), generalised from the
// per-position referee of compare/multifreq.py:58-98 to every trace:
//
//   H[t, k] = sum_n contrib_n(t, f_k),   f_k = f0 - B/2 + (k + 1/2) B/K
//   y[t, b] = sum_k Wbar_k H[t, k] exp(+2j pi (f_k - f0) twtt_b)
//
// with contrib the LPA facet field of kernels/coherent.py:107-128 evaluated
// at wavenumber 2 pi f_k / c -- either with every factor at f_k (full) or
// with the amplitude frozen at f0 and the exact per-frequency phase
// exp(-2j k_k r) (the post-convolution model, multifreq.py:82-86).
//
// Band response (the hot part, T x N x K phasors):
//   CTA = (facet chunk, trace block, frequency block); thread <-> a run of
//   consecutive frequencies. Per tile of facets the CTA first evaluates
//   each (trace, facet) pair once -- range, amplitude, and the phase step
//   between neighbouring frequencies -- into shared memory; every thread
//   then turns each pair into its frequencies' phasors: one carrier phase
//   per pair and run (double-float R f_s reduced mod 2 pi, ulp-accurate
//   sincos), then a complex rotation by the per-pair step for each further
//   frequency. Per-chunk
//   partial spectra go through the ordered chunk reduction.
//   Split form: float32 with double-float range and phase (as the delta-
//   binned split kernel); FP64 form: float64 throughout.
// Synthesis (T x K x B): thread <-> output sample; the factor
//   exp(2j pi (f_k - f0) twtt_b) is re-anchored every 8 frequencies from a
//   float64 cycle count and rotated in between; split-form sums are
//   compensated (two-sum).
#include <algorithm>

#include "ss_df.cuh"
#include "ss_f32.cuh"

namespace ss {

struct MfArgs {
  ss_facets F;
  const double *pos;
  const int32_t *off;
  int T, N, K;
  int bs, n_win;
  double f0, bw, c, gamma, taper_s;
  int taper, freeze;
  int rough_kind, n_terms;
  double sigma, corr;
  FadCoeffs fad;
  int tb, n_chunks;
  void *part;
};

// split form: 128 threads x 8 frequencies = 1024 frequencies per CTA,
// 4 traces per CTA, tiles of 32 facets (4 x 32 = one pair per thread)
constexpr int kMfThreads = 128, kMfF = 8, kMfTB = 4, kMfP = 32;
constexpr int kMfFBlock = kMfThreads * kMfF;
// FP64 form: 2 traces per CTA, tiles of 64 facets
constexpr int kMf64TB = 2, kMf64P = 64;

struct MfSplitConsts {
  float Rch, Rcl;   // 4 pi / c (rad per metre per hertz) as double-float
  float dfh, dfl;   // frequency step B / K
  float f1h, f1l;   // first frequency f0 - B/2 + B/(2K)
  float k0, amp0;   // 2 pi f0 / c and k0 / (2 pi)
  float kf1, dk;    // wavenumber of the first frequency and the step
  float gamma, taper_inv, fadL, sigma, corr;
};

// Compensated float sum: value = s + c (two-sum error terms gathered in c).
struct Acc2 {
  float s, c;
};

__device__ __forceinline__ void acc2_add(Acc2 &a, float x) {
  float s, e;
  two_sum(a.s, x, s, e);
  a.s = s;
  a.c += e;
}

// x * y of a double-float and a double-float, rounded to a double-float.
__device__ __forceinline__ void df_prod(float xh, float xl, float yh, float yl,
                                        float &ph, float &pl) {
  float p, e;
  two_prod(xh, yh, p, e);
  e = __fmaf_rn(xh, yl, __fmaf_rn(xl, yh, e));
  fast_two_sum(p, e, ph, pl);
}

// hi + lo reduced modulo 2 pi (hi carries the integer turns).
__device__ __forceinline__ float reduce_df_2pi(float hi, float lo) {
  const float n = rintf(hi * 0.159154943091895336f);
  float r = __fmaf_rn(-n, 6.28318548202514648f, hi);  // exact
  return __fmaf_rn(-n, -1.74845553146951e-07f, r) + lo;
}

// sin(x)/x to float32 accuracy for any x: the full-amplitude form evaluates
// it per frequency, and the sinc product's errors add across frequencies
// into the synthesised profile, so the library sinf (ulp-accurate) is used
// rather than the MUFU approximation; series below |x| = 0.5.
__device__ __forceinline__ float sinc_acc(float x) {
  const float x2 = x * x;
  if (x2 < 0.25f)
    return __fmaf_rn(x2, __fmaf_rn(x2, __fmaf_rn(x2, __fmaf_rn(
               x2, 2.7557319e-06f, -1.9841270e-04f), 8.3333333e-03f),
               -1.6666667e-01f), 1.0f);
  return sinf(x) / x;
}

// Per-trace facet window [lo, hi) (the coherent kernel's culling).
__device__ __forceinline__ void trace_window(const MfArgs &a, int t, int &lo,
                                             int &hi) {
  long l = (long)a.off[t] * a.bs;
  long h = min((long)(a.off[t] + a.n_win) * a.bs, (long)a.N);
  lo = (int)min(l, (long)a.N);
  hi = (int)h;
}

template <bool FULL, int ROUGH>
__global__ void __launch_bounds__(kMfThreads)
multifreq_split_kernel(MfArgs a, MfSplitConsts k) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float *lg = reinterpret_cast<float *>(smem_raw);
  __shared__ float s_ph[kMfTB][3], s_pl[kMfTB][3];
  __shared__ int s_lo[kMfTB], s_hi[kMfTB];
  __shared__ int s_rng[2];
  __shared__ float s_fad[SS_FAD_N];
  // pair data: R (hi, lo), amplitude (re, im) or (g, -), d1, d2, step (re, im)
  __shared__ float4 s_pa[kMfTB * kMfP];
  __shared__ float4 s_pb[kMfTB * kMfP];
  const int chunk = blockIdx.x;
  const int t_base = blockIdx.y * kMfTB;
  const int nt = min(kMfTB, a.T - t_base);
  const int tid = threadIdx.x;
  if (tid < kMfTB) {
    const int t = min(t_base + tid, a.T - 1);
    for (int j = 0; j < 3; ++j) {
      const df v = df_from_double(a.pos[3 * t + j]);
      s_ph[tid][j] = v.hi;
      s_pl[tid][j] = v.lo;
    }
    int lo, hi;
    trace_window(a, t, lo, hi);
    s_lo[tid] = tid < nt ? lo : a.N;
    s_hi[tid] = tid < nt ? hi : 0;
  }
  if (ROUGH == SS_ROUGH_GAUSS_FULL && tid < SS_FAD_N)
    s_fad[tid] = (float)a.fad.a[tid];
  if (ROUGH != SS_ROUGH_NONE) fill_inv_table(lg, a.n_terms, tid, blockDim.x);
  __syncthreads();
  if (tid == 0) {
    int lo = s_lo[0], hi = s_hi[0];
    for (int j = 1; j < nt; ++j) {
      lo = min(lo, s_lo[j]);
      hi = max(hi, s_hi[j]);
    }
    const long len = max(hi - lo, 0);
    s_rng[0] = lo + (int)(len * chunk / a.n_chunks);
    s_rng[1] = lo + (int)(len * (chunk + 1) / a.n_chunks);
  }
  __syncthreads();

  // this thread's first frequency index and its frequency / wavenumber
  const int kn = blockIdx.z * kMfFBlock + tid * kMfF;
  float fsh, fsl;
  {
    float p, e;
    two_prod((float)kn, k.dfh, p, e);
    e = __fmaf_rn((float)kn, k.dfl, e);
    float s, e2;
    two_sum(k.f1h, p, s, e2);
    fast_two_sum(s, e2 + e + k.f1l, fsh, fsl);
  }
  const float ks = __fmaf_rn((float)kn, k.dk, k.kf1);
  float2 acc[kMfTB][kMfF];
#pragma unroll
  for (int tt = 0; tt < kMfTB; ++tt)
#pragma unroll
    for (int q = 0; q < kMfF; ++q) acc[tt][q] = make_float2(0.0f, 0.0f);

  for (int base = s_rng[0]; base < s_rng[1]; base += kMfP) {
    // --- phase A: one (trace, facet) pair per thread ---
    {
      const int tt = tid / kMfP, i = base + tid % kMfP;
      float4 pa = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
      float4 pb = make_float4(1.0f, 0.0f, 0.0f, 0.0f);
      if (i < s_rng[1] && i >= s_lo[tt] && i < s_hi[tt]) {
        const float cx = a.F.cx[i], cy = a.F.cy[i], cz = a.F.cz[i];
        float dxh, dxl, dyh, dyl, dzh, dzl, e;
        two_sum(s_ph[tt][0], -cx, dxh, e);
        fast_two_sum(dxh, e + s_pl[tt][0], dxh, dxl);
        two_sum(s_ph[tt][1], -cy, dyh, e);
        fast_two_sum(dyh, e + s_pl[tt][1], dyh, dyl);
        two_sum(s_ph[tt][2], -cz, dzh, e);
        fast_two_sum(dzh, e + s_pl[tt][2], dzh, dzl);
        const df r = df_norm3(df{dxh, dxl}, df{dyh, dyl}, df{dzh, dzl});
        const float inv_r = 1.0f / r.hi;
        const float cosv = dot3f(dxh, dyh, dzh, a.F.nx[i], a.F.ny[i],
                                 a.F.nz[i]) * inv_r;
        const float e1x = a.F.e1x[i], e1y = a.F.e1y[i], e1z = a.F.e1z[i];
        const float e2x = a.F.e2x[i], e2y = a.F.e2y[i], e2z = a.F.e2z[i];
        // r_hat . e from the exact (double-float) d: k (r_hat . e) reaches
        // tens of radians and cancels near nadir
        float p1, q1, p2, q2, p3, q3, s1, s2, s3, s4;
        two_prod(dxh, e1x, p1, q1);
        two_prod(dyh, e1y, p2, q2);
        two_prod(dzh, e1z, p3, q3);
        two_sum(p1, p2, s1, s2);
        two_sum(s1, p3, s3, s4);
        const float d1 = (s3 + ((s2 + s4) + (q1 + q2 + q3) +
                                __fmaf_rn(dxl, e1x, __fmaf_rn(dyl, e1y,
                                                              dzl * e1z)))) *
                         inv_r;
        two_prod(dxh, e2x, p1, q1);
        two_prod(dyh, e2y, p2, q2);
        two_prod(dzh, e2z, p3, q3);
        two_sum(p1, p2, s1, s2);
        two_sum(s1, p3, s3, s4);
        const float d2 = (s3 + ((s2 + s4) + (q1 + q2 + q3) +
                                __fmaf_rn(dxl, e2x, __fmaf_rn(dyl, e2y,
                                                              dzl * e2z)))) *
                         inv_r;
        const float area = a.F.area[i];
        const float gam = a.F.gamma_f32 ? a.F.gamma_f32[i] : k.gamma;
        float g = gam * cosv * area * inv_r * inv_r;
        if (a.taper) {
          const float cc = fminf(fmaxf(cosv, 1e-9f), 1.0f);
          const float c2 = cc * cc;
          g *= __expf(-__fdividef(1.0f - c2, c2) * k.taper_inv);
        }
        // R = 4 pi r / c; phase of frequency f is R f
        float Rh, Rl;
        df_prod(k.Rch, k.Rcl, r.hi, r.lo, Rh, Rl);
        // step between neighbouring frequencies: exp(-j R df)
        float dh, dl;
        df_prod(Rh, Rl, k.dfh, k.dfl, dh, dl);
        float sn, cs;
        sincosf(reduce_df_2pi(dh, dl), &sn, &cs);
        pb = make_float4(cs, -sn, d1, d2);
        if (FULL) {
          // amplitude (k / 2 pi) g sinc(k d1) sinc(k d2), evaluated per
          // frequency; contribution j amp exp(-j phase)
          pa = make_float4(Rh, Rl, g * 0.159154943091895336f, 0.0f);
        } else {
          const float amp = k.amp0 * g * sinc32(k.k0 * d1) *
                            sinc32(k.k0 * d2);
          float cr = amp, ci = 0.0f;
          if (ROUGH != SS_ROUGH_NONE) {
            const float sg = a.F.sigma ? a.F.sigma[i] : k.sigma;
            const float lc = a.F.corr ? a.F.corr[i] : k.corr;
            const float l1 = sqrtf(dot3f(e1x, e1y, e1z, e1x, e1y, e1z));
            const float l2 = sqrtf(dot3f(e2x, e2y, e2z, e2x, e2y, e2z));
            const float kk = 2.0f * k.k0 * cosv;
            const float dp = d_phi32<ROUGH>(a.n_terms, lg, s_fad, k.fadL, sg,
                                            lc, kk, 2.0f * k.k0 * d1 / l1,
                                            2.0f * k.k0 * d2 / l2, l1, l2);
            const float amp_i = area > 0.0f
                                    ? k.amp0 * gam * cosv * inv_r * inv_r *
                                          sqrtf(dp)
                                    : 0.0f;
            const float sk = sg * kk;
            cr = amp * __expf(-0.5f * sk * sk) + amp_i * a.F.phasor[2 * i];
            ci = amp_i * a.F.phasor[2 * i + 1];
          }
          // j (cr + j ci)
          pa = make_float4(Rh, Rl, -ci, cr);
        }
      }
      __syncthreads();
      s_pa[tid] = pa;
      s_pb[tid] = pb;
      __syncthreads();
    }
    // --- phase B: every thread, every pair of the tile, its frequencies ---
#pragma unroll
    for (int tt = 0; tt < kMfTB; ++tt) {
      for (int f = 0; f < kMfP; ++f) {
        const float4 pa = s_pa[tt * kMfP + f];
        const float4 pb = s_pb[tt * kMfP + f];
        if (pa.z == 0.0f && pa.w == 0.0f) continue;  // outside the window
        float ph, pl;
        df_prod(pa.x, pa.y, fsh, fsl, ph, pl);
        // ulp-accurate sincos: the band response sums many partly
        // cancelling phasors, and MUFU's ~4e-7 absolute error would show
        // at -60 dB of the synthesised profile
        float sn, cs;
        sincosf(reduce_df_2pi(ph, pl), &sn, &cs);
        float er = cs, ei = -sn;  // exp(-j phase)
        if (FULL) {
#pragma unroll
          for (int q = 0; q < kMfF; ++q) {
            const float kq = __fmaf_rn((float)q, k.dk, ks);
            const float amp = pa.z * kq * sinc_acc(kq * pb.z) *
                              sinc_acc(kq * pb.w);
            acc[tt][q].x -= amp * ei;  // j amp e
            acc[tt][q].y += amp * er;
            const float nr = er * pb.x - ei * pb.y;
            ei = er * pb.y + ei * pb.x;
            er = nr;
          }
        } else {
          float zr = pa.z * er - pa.w * ei;
          float zi = pa.z * ei + pa.w * er;
#pragma unroll
          for (int q = 0; q < kMfF; ++q) {
            acc[tt][q].x += zr;
            acc[tt][q].y += zi;
            const float nr = zr * pb.x - zi * pb.y;
            zi = zr * pb.y + zi * pb.x;
            zr = nr;
          }
        }
      }
    }
  }
  float2 *part = reinterpret_cast<float2 *>(a.part);
#pragma unroll
  for (int tt = 0; tt < kMfTB; ++tt) {
    if (tt >= nt) break;
    const size_t row = ((size_t)chunk * a.T + t_base + tt) * a.K;
#pragma unroll
    for (int q = 0; q < kMfF; ++q)
      if (kn + q < a.K) part[row + kn + q] = acc[tt][q];
  }
}

// FP64 form: same decomposition, float64 throughout.
template <bool FULL>
__global__ void __launch_bounds__(kMfThreads)
multifreq_fp64_kernel(MfArgs a) {
  __shared__ double s_p[kMf64TB][3];
  __shared__ int s_lo[kMf64TB], s_hi[kMf64TB];
  __shared__ int s_rng[2];
  // pair data: R, amplitude (re, im) or g, d1, d2, step (re, im)
  __shared__ double s_d[kMf64TB * kMf64P][6];
  const int chunk = blockIdx.x;
  const int t_base = blockIdx.y * kMf64TB;
  const int nt = min(kMf64TB, a.T - t_base);
  const int tid = threadIdx.x;
  if (tid < kMf64TB) {
    const int t = min(t_base + tid, a.T - 1);
    for (int j = 0; j < 3; ++j) s_p[tid][j] = a.pos[3 * t + j];
    int lo, hi;
    trace_window(a, t, lo, hi);
    s_lo[tid] = tid < nt ? lo : a.N;
    s_hi[tid] = tid < nt ? hi : 0;
  }
  __syncthreads();
  if (tid == 0) {
    int lo = s_lo[0], hi = s_hi[0];
    for (int j = 1; j < nt; ++j) {
      lo = min(lo, s_lo[j]);
      hi = max(hi, s_hi[j]);
    }
    const long len = max(hi - lo, 0);
    s_rng[0] = lo + (int)(len * chunk / a.n_chunks);
    s_rng[1] = lo + (int)(len * (chunk + 1) / a.n_chunks);
  }
  __syncthreads();
  const double dfq = a.bw / a.K;
  const double f1 = a.f0 - 0.5 * a.bw + 0.5 * dfq;
  const int kn = blockIdx.z * kMfFBlock + tid * kMfF;
  const double fs = f1 + kn * dfq;
  const double k0 = kTwoPi * a.f0 / a.c;
  double2 acc[kMf64TB][kMfF];
#pragma unroll
  for (int tt = 0; tt < kMf64TB; ++tt)
#pragma unroll
    for (int q = 0; q < kMfF; ++q) acc[tt][q] = make_double2(0.0, 0.0);
  for (int base = s_rng[0]; base < s_rng[1]; base += kMf64P) {
    for (int pr = tid; pr < kMf64TB * kMf64P; pr += blockDim.x) {
      const int tt = pr / kMf64P, i = base + pr % kMf64P;
      double d[6] = {0.0, 0.0, 0.0, 0.0, 1.0, 0.0};
      if (i < s_rng[1] && i >= s_lo[tt] && i < s_hi[tt]) {
        const double dx = s_p[tt][0] - (double)a.F.cx[i];
        const double dy = s_p[tt][1] - (double)a.F.cy[i];
        const double dz = s_p[tt][2] - (double)a.F.cz[i];
        const double r = sqrt(dx * dx + dy * dy + dz * dz);
        const double cosv = dot3(dx, dy, dz, a.F.nx[i], a.F.ny[i],
                                 a.F.nz[i]) / r;
        const double d1 = dot3(dx, dy, dz, a.F.e1x[i], a.F.e1y[i],
                               a.F.e1z[i]) / r;
        const double d2 = dot3(dx, dy, dz, a.F.e2x[i], a.F.e2y[i],
                               a.F.e2z[i]) / r;
        const double gam = a.F.gamma_f32 ? (double)a.F.gamma_f32[i] : a.gamma;
        double g = gam * cosv * (double)a.F.area[i] / (r * r);
        if (a.taper) {
          const double cc = fmin(fmax(cosv, 1e-9), 1.0);
          const double c2 = cc * cc;
          g *= exp(-(1.0 - c2) / (c2 * (2.0 * a.taper_s * a.taper_s)));
        }
        const double R = 4.0 * kPi * r / a.c;
        double sn, cs;
        sincos(R * dfq, &sn, &cs);
        if (FULL) {
          d[0] = R; d[1] = g / kTwoPi; d[2] = d1; d[3] = d2;
        } else {
          const double amp = (k0 / kTwoPi) * g * sinc_np(k0 * d1 / kPi) *
                             sinc_np(k0 * d2 / kPi);
          d[0] = R; d[1] = 0.0; d[2] = amp; d[3] = 0.0;  // j amp
        }
        d[4] = cs;
        d[5] = -sn;
      }
      for (int j = 0; j < 6; ++j) s_d[pr][j] = d[j];
    }
    __syncthreads();
#pragma unroll
    for (int tt = 0; tt < kMf64TB; ++tt) {
      for (int f = 0; f < kMf64P; ++f) {
        const double *d = s_d[tt * kMf64P + f];
        if (d[1] == 0.0 && d[2] == 0.0 && d[3] == 0.0) continue;
        double sn, cs;
        sincos(fmod(d[0] * fs, kTwoPi), &sn, &cs);
        double er = cs, ei = -sn;
        if (FULL) {
          for (int q = 0; q < kMfF; ++q) {
            const double kq = kTwoPi * (fs + q * dfq) / a.c;
            const double amp = d[1] * kq * sinc_np(kq * d[2] / kPi) *
                               sinc_np(kq * d[3] / kPi);
            acc[tt][q].x -= amp * ei;
            acc[tt][q].y += amp * er;
            const double nr = er * d[4] - ei * d[5];
            ei = er * d[5] + ei * d[4];
            er = nr;
          }
        } else {
          // j amp exp(-j phase): (0 + j amp)(er + j ei)
          double zr = -d[2] * ei, zi = d[2] * er;
          for (int q = 0; q < kMfF; ++q) {
            acc[tt][q].x += zr;
            acc[tt][q].y += zi;
            const double nr = zr * d[4] - zi * d[5];
            zi = zr * d[5] + zi * d[4];
            zr = nr;
          }
        }
      }
    }
    __syncthreads();
  }
  double2 *part = reinterpret_cast<double2 *>(a.part);
#pragma unroll
  for (int tt = 0; tt < kMf64TB; ++tt) {
    if (tt >= nt) break;
    const size_t row = ((size_t)chunk * a.T + t_base + tt) * a.K;
    for (int q = 0; q < kMfF; ++q)
      if (kn + q < a.K) part[row + kn + q] = acc[tt][q];
  }
}

// Synthesis y[t, b] = sum_k wbar_k H[t, k] exp(2j pi (f_k - f0) twtt_b).
constexpr int kSynTile = 256;
// Re-anchoring interval of the synthesis rotation: a float32 step carries
// ~6e-8 relative rounding that compounds linearly between anchors, and an
// error of 1e-6 of the peak is 0.01 dB at -60 dB, so anchors come every 8
// frequencies (drift <= 5e-7).
constexpr int kSynAnchor = 8;

template <bool F64>
__global__ void __launch_bounds__(kSynTile)
multifreq_synth_kernel(int T, int K, int B, double f0, double bw,
                       const double *H, const double *wbar,
                       const double *twtt, double *y) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int t = blockIdx.y;
  const int b = blockIdx.x * kSynTile + threadIdx.x;
  const double dfq = bw / K;
  const double f1 = f0 - 0.5 * bw + 0.5 * dfq;  // f_k - f0 = off + k dfq
  const double off = f1 - f0;
  if (F64) {
    double2 *g = reinterpret_cast<double2 *>(smem_raw);
    for (int k = threadIdx.x; k < K; k += kSynTile)
      g[k] = make_double2(wbar[k] * H[2 * ((size_t)t * K + k)],
                          wbar[k] * H[2 * ((size_t)t * K + k) + 1]);
    __syncthreads();
    if (b >= B) return;
    const double tau = twtt[b];
    double sr, si;
    const double cstep = dfq * tau;
    sincospi(2.0 * (cstep - rint(cstep)), &si, &sr);
    double yr = 0.0, yi = 0.0, er = 1.0, ei = 0.0;
    for (int k = 0; k < K; ++k) {
      if (k % kSynAnchor == 0) {
        const double cyc = (off + k * dfq) * tau;
        sincospi(2.0 * (cyc - rint(cyc)), &ei, &er);
      }
      yr += g[k].x * er - g[k].y * ei;
      yi += g[k].x * ei + g[k].y * er;
      const double nr = er * sr - ei * si;
      ei = er * si + ei * sr;
      er = nr;
    }
    y[2 * ((size_t)t * B + b)] = yr;
    y[2 * ((size_t)t * B + b) + 1] = yi;
  } else {
    float2 *g = reinterpret_cast<float2 *>(smem_raw);
    for (int k = threadIdx.x; k < K; k += kSynTile)
      g[k] = make_float2((float)(wbar[k] * H[2 * ((size_t)t * K + k)]),
                         (float)(wbar[k] * H[2 * ((size_t)t * K + k) + 1]));
    __syncthreads();
    if (b >= B) return;
    const double tau = twtt[b];
    float sr, si;
    const double cstep = dfq * tau;
    sincospif((float)(2.0 * (cstep - rint(cstep))), &si, &sr);
    Acc2 yr{0.0f, 0.0f}, yi{0.0f, 0.0f};
    float er = 1.0f, ei = 0.0f;
    for (int k = 0; k < K; ++k) {
      if (k % kSynAnchor == 0) {
        const double cyc = (off + k * dfq) * tau;
        sincospif((float)(2.0 * (cyc - rint(cyc))), &ei, &er);
      }
      const float2 gk = g[k];
      acc2_add(yr, __fmaf_rn(gk.x, er, -gk.y * ei));
      acc2_add(yi, __fmaf_rn(gk.x, ei, gk.y * er));
      const float nr = er * sr - ei * si;
      ei = er * si + ei * sr;
      er = nr;
    }
    y[2 * ((size_t)t * B + b)] = (double)yr.s + (double)yr.c;
    y[2 * ((size_t)t * B + b) + 1] = (double)yi.s + (double)yi.c;
  }
}

static int mf_plan(const ss_multifreq_opts *o, int T, int N, Plan *p) {
  if (!o || T <= 0 || N <= 0 || o->n_freq <= 0 || o->block_size <= 0 ||
      o->n_win <= 0 || !(o->bandwidth > 0.0) || !(o->c > 0.0))
    return SS_ERR_ARG;
  const bool f64 = o->precision == SS_PREC_FP64;
  p->tb = f64 ? kMf64TB : kMfTB;
  p->n_groups = (T + p->tb - 1) / p->tb;
  p->threads = kMfThreads;
  const int fblk = (o->n_freq + kMfFBlock - 1) / kMfFBlock;
  const long window = std::min<long>((long)o->n_win * o->block_size, N);
  const int tile = f64 ? kMf64P : kMfP;
  const int max_chunks = (int)std::max<long>(1, window / (4 * tile));
  const int target = 8 * sm_count();
  const int per = p->n_groups * fblk;
  p->n_chunks = std::max(1, std::min(max_chunks, (target + per - 1) / per));
  p->smem = 0;
  return SS_OK;
}

static size_t mf_scratch(const ss_multifreq_opts *o, int T, int N) {
  Plan p;
  if (mf_plan(o, T, N, &p) != SS_OK) return 0;
  const size_t elt = o->precision == SS_PREC_FP64 ? 16 : 8;
  size_t part = ((size_t)p.n_chunks * T * o->n_freq * elt + 255) &
                ~(size_t)255;
  size_t drop = ((size_t)p.n_chunks * T * sizeof(double) + 255) &
                ~(size_t)255;
  return part + drop + (size_t)T * sizeof(double);
}

}  // namespace ss

extern "C" size_t ss_multifreq_scratch_bytes(const ss_multifreq_opts *opts,
                                             int32_t n_traces,
                                             int32_t n_facets) {
  return ss::mf_scratch(opts, n_traces, n_facets);
}

extern "C" int ss_multifreq_response(const ss_multifreq_opts *o,
                                     const ss_facets *facets,
                                     const ss_traces *traces,
                                     const ss_roughness *rough, double *H,
                                     void *scratch, size_t scratch_bytes,
                                     void *stream) {
  using namespace ss;
  if (!o || !facets || !traces || !H) {
    set_error("null argument");
    return SS_ERR_ARG;
  }
  const int T = traces->n_traces, N = facets->n_facets;
  if (!traces->pos || !traces->off || !facets->cx || !facets->area) {
    set_error("missing required device pointer");
    return SS_ERR_ARG;
  }
  if (o->precision != SS_PREC_FP64 && o->precision != SS_PREC_SPLIT) {
    set_error("unknown precision");
    return SS_ERR_ARG;
  }
  Plan p;
  if (mf_plan(o, T, N, &p) != SS_OK) {
    set_error("bad sizes (n_freq, block_size, n_win > 0; bandwidth, c > 0)");
    return SS_ERR_ARG;
  }
  const int rk = rough ? rough->kind : SS_ROUGH_NONE;
  if (rk != SS_ROUGH_NONE) {
    if (!o->freeze_amplitudes || o->precision == SS_PREC_FP64) {
      set_error("roughness is supported with frozen amplitudes in the split "
                "form only");
      return SS_ERR_UNSUPPORTED;
    }
    if (!facets->phasor || rough->n_terms < 0 ||
        rough->n_terms > SS_MAX_TERMS) {
      set_error("roughness needs phasors and 0 <= n_terms <= 4096");
      return SS_ERR_ARG;
    }
  }
  const size_t need = mf_scratch(o, T, N);
  if (!scratch || scratch_bytes < need) {
    set_error("scratch buffer too small");
    return SS_ERR_SCRATCH;
  }
  MfArgs a{};
  a.F = *facets;
  a.pos = traces->pos;
  a.off = traces->off;
  a.T = T;
  a.N = N;
  a.K = o->n_freq;
  a.bs = o->block_size;
  a.n_win = o->n_win;
  a.f0 = o->f0;
  a.bw = o->bandwidth;
  a.c = o->c;
  a.gamma = o->gamma;
  a.taper_s = o->taper_s;
  a.taper = o->taper;
  a.freeze = o->freeze_amplitudes;
  a.rough_kind = rk;
  if (rk != SS_ROUGH_NONE) {
    a.n_terms = rough->n_terms;
    a.sigma = rough->sigma;
    a.corr = rough->corr;
    a.fad = faddeeva_coeffs();
  }
  a.tb = p.tb;
  a.n_chunks = p.n_chunks;
  const bool f64 = o->precision == SS_PREC_FP64;
  const size_t elt = f64 ? 16 : 8;
  const size_t part = ((size_t)p.n_chunks * T * a.K * elt + 255) &
                      ~(size_t)255;
  const size_t drop = ((size_t)p.n_chunks * T * sizeof(double) + 255) &
                      ~(size_t)255;
  a.part = scratch;
  double *part_drop = reinterpret_cast<double *>(
      static_cast<char *>(scratch) + part);
  double *dropped = reinterpret_cast<double *>(static_cast<char *>(scratch) +
                                               part + drop);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  cudaError_t e = cudaMemsetAsync(part_drop, 0, drop, st);
  if (e != cudaSuccess) return cuda_status(e, "multifreq scratch clear");
  const int fblk = (a.K + kMfFBlock - 1) / kMfFBlock;
  dim3 grid(p.n_chunks, p.n_groups, fblk);
  if (f64) {
    if (o->freeze_amplitudes)
      multifreq_fp64_kernel<false><<<grid, kMfThreads, 0, st>>>(a);
    else
      multifreq_fp64_kernel<true><<<grid, kMfThreads, 0, st>>>(a);
  } else {
    MfSplitConsts k{};
    const double dfq = o->bandwidth / o->n_freq;
    const double f1 = o->f0 - 0.5 * o->bandwidth + 0.5 * dfq;
    const df rc = df_from_double(4.0 * kPi / o->c);
    const df dd = df_from_double(dfq);
    const df ff = df_from_double(f1);
    k.Rch = rc.hi;
    k.Rcl = rc.lo;
    k.dfh = dd.hi;
    k.dfl = dd.lo;
    k.f1h = ff.hi;
    k.f1l = ff.lo;
    k.k0 = (float)(kTwoPi * o->f0 / o->c);
    k.amp0 = (float)(o->f0 / o->c);  // k0 / (2 pi)
    k.kf1 = (float)(kTwoPi * f1 / o->c);
    k.dk = (float)(kTwoPi * dfq / o->c);
    k.gamma = (float)o->gamma;
    k.taper_inv =
        o->taper ? (float)(1.0 / (2.0 * o->taper_s * o->taper_s)) : 0.0f;
    k.fadL = (float)a.fad.L;
    k.sigma = (float)a.sigma;
    k.corr = (float)a.corr;
    const size_t smem = rk ? (size_t)(a.n_terms + 1) * sizeof(float) : 0;
    if (!o->freeze_amplitudes) {
      multifreq_split_kernel<true, SS_ROUGH_NONE>
          <<<grid, kMfThreads, smem, st>>>(a, k);
    } else {
      switch (rk) {
        case SS_ROUGH_NONE:
          multifreq_split_kernel<false, SS_ROUGH_NONE>
              <<<grid, kMfThreads, smem, st>>>(a, k);
          break;
        case SS_ROUGH_GAUSS_FULL:
          multifreq_split_kernel<false, SS_ROUGH_GAUSS_FULL>
              <<<grid, kMfThreads, smem, st>>>(a, k);
          break;
        case SS_ROUGH_GAUSS_AREA:
          multifreq_split_kernel<false, SS_ROUGH_GAUSS_AREA>
              <<<grid, kMfThreads, smem, st>>>(a, k);
          break;
        default:
          multifreq_split_kernel<false, SS_ROUGH_EXP_AREA>
              <<<grid, kMfThreads, smem, st>>>(a, k);
          break;
      }
    }
  }
  e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_status(e, "multifreq launch");
  ReduceArgs r{T, a.K, a.K, 0, p.n_chunks, a.part, part_drop};
  ss_output out{H, nullptr, dropped};
  return launch_reduce(r, f64, &out, st);
}

extern "C" int ss_multifreq_synth(const ss_multifreq_opts *o,
                                  int32_t n_traces, const double *H,
                                  const double *wbar, const double *twtt,
                                  int32_t n_twtt, double *y, void *stream) {
  using namespace ss;
  if (!o || !H || !wbar || !twtt || !y) {
    set_error("null argument");
    return SS_ERR_ARG;
  }
  if (n_traces <= 0 || n_traces > 65535 || n_twtt <= 0 || o->n_freq <= 0 ||
      !(o->bandwidth > 0.0)) {
    set_error("bad synthesis sizes (1 <= n_traces <= 65535, n_twtt > 0)");
    return SS_ERR_ARG;
  }
  const bool f64 = o->precision == SS_PREC_FP64;
  const size_t smem = (size_t)o->n_freq * (f64 ? 16 : 8);
  if (smem > 200 * 1024) {
    set_error("n_freq too large for the synthesis kernel");
    return SS_ERR_UNSUPPORTED;
  }
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  dim3 grid((n_twtt + kSynTile - 1) / kSynTile, n_traces);
  cudaError_t e;
  if (f64) {
    e = cudaFuncSetAttribute(multifreq_synth_kernel<true>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)smem);
    if (e != cudaSuccess) return cuda_status(e, "synth smem");
    multifreq_synth_kernel<true><<<grid, kSynTile, smem, st>>>(
        n_traces, o->n_freq, n_twtt, o->f0, o->bandwidth, H, wbar, twtt, y);
  } else {
    e = cudaFuncSetAttribute(multifreq_synth_kernel<false>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)smem);
    if (e != cudaSuccess) return cuda_status(e, "synth smem");
    multifreq_synth_kernel<false><<<grid, kSynTile, smem, st>>>(
        n_traces, o->n_freq, n_twtt, o->f0, o->bandwidth, H, wbar, twtt, y);
  }
  return cuda_status(cudaGetLastError(), "multifreq synth launch");
}
