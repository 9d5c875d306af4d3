// Focused SAR: straight-track time-domain backprojection on GB300.
//
// Replaces the per-trace NumPy loop of soundersim processing.py:301-329
// (`focused_sar`). Output sample (i, b) sums, over the aperture traces j with
// |s_j - s_i| <= L/2, the field of trace j linearly interpolated at the
// range-migrated delay twtt[b] + 2 dr / c (dr = sqrt(r0^2 + d^2) - r0,
// r0 = c twtt[b] / 2, d = s_j - s_i), times the carrier correction
// exp(+2j k dr) and the aperture weight (hann or rectangular). Samples whose
// lower index falls outside [0, nb - 2] contribute nothing.
//
// Each thread accumulates one bin of one or more output traces over their
// apertures; a whole (T, nb) complex64 field of a 1024 x 2048 track is
// 16.8 MB and stays in L2. The aperture bounds of every output trace come
// from a small binary-search kernel (s is non-decreasing, so the aperture is
// a contiguous range).
//
// Two precisions:
//   FP64  -- the reference's float64 chain with round-to-nearest intrinsics
//            (no contraction): same delay, interpolation, phase and sum
//            order (j ascending), so it agrees with the float64 oracle to a
//            few ulps of the sine/cosine.
//   FP32  -- dr = d^2 / (sqrt(r0^2 + d^2) + r0) (no cancellation), the delay
//            as a float offset from the per-bin float64 base position, the
//            phase reduced modulo 2 pi before the MUFU sine/cosine, float32
//            accumulation.
#include "ss_f32.cuh"
#include "ss_internal.cuh"

namespace ss {

struct FocusArgs {
  const void *field;   // (T, nb) complex64 or complex128
  const double *twtt;  // (nb,)
  const double *s;     // (T,) along-track arc length
  const int *jr;       // (T, 2) aperture [lo, hi) per output trace
  float4 *bins;        // (nb,) split form: i00 (as int bits), frac0, r0, -
  int T, nb, window, in_f64;
  double k, c, half;
  ss_focus_output out;
};

// One output sample: complex128 and/or complex64 field, and float32 power
// |out|^2 with |out| rounded to float32 first (processing.py:345).
__device__ __forceinline__ void write_out(const FocusArgs &a, long o,
                                          double re, double im) {
  if (a.out.field_c128) {
    a.out.field_c128[2 * o] = re;
    a.out.field_c128[2 * o + 1] = im;
  }
  if (a.out.field_c64) {
    a.out.field_c64[2 * o] = (float)re;
    a.out.field_c64[2 * o + 1] = (float)im;
  }
  if (a.out.power) {
    const float m = (float)hypot(re, im);
    a.out.power[o] = m * m;
  }
}

// Aperture bounds: the contiguous j range with |s_j - s_i| <= half, found
// with the reference's predicate (float64 difference, then |.| <= half).
__device__ __forceinline__ void aperture_bounds(const double *s, int T,
                                                double half, int i, int *jr) {
  const double si = s[i];
  // lo: first j with s_j - s_i >= -half (monotone in j)
  int lo = 0, hi = i + 1;
  while (lo < hi) {
    const int m = (lo + hi) >> 1;
    if (fabs(__dsub_rn(s[m], si)) <= half) hi = m; else lo = m + 1;
  }
  const int jlo = lo;
  // hi: first j > i with s_j - s_i > half
  lo = i + 1;
  hi = T;
  while (lo < hi) {
    const int m = (lo + hi) >> 1;
    if (fabs(__dsub_rn(s[m], si)) <= half) lo = m + 1; else hi = m;
  }
  // an empty aperture (half < 0) gives lo > i: keep the range empty
  jr[2 * i] = jlo;
  jr[2 * i + 1] = jlo <= i ? lo : jlo;
}

// Per-bin constants shared by both forms: r0 = c twtt / 2 and the delay of
// the d = 0 term, (twtt[b] - t0) / dt, as an integer base and a fraction.
struct BinConsts {
  double t0, dt, tb, r0, frac0;
  int i00;
};

__device__ __forceinline__ BinConsts bin_consts(const FocusArgs &a, int b) {
  BinConsts q;
  q.t0 = a.twtt[0];
  q.dt = __dsub_rn(a.twtt[1], q.t0);
  q.tb = b < a.nb ? a.twtt[b] : q.t0;
  q.r0 = __dmul_rn(a.c, q.tb) * 0.5;
  const double x0 = __ddiv_rn(__dsub_rn(q.tb, q.t0), q.dt);
  const double fl0 = floor(x0);
  q.i00 = (int)fl0;
  q.frac0 = __dsub_rn(x0, fl0);
  return q;
}

// Setup: aperture bounds of every output trace (threads [0, T)) and, for
// the split form, the per-bin table of float32 constants (threads
// [T, T + nb)), so the split kernel does no float64 arithmetic per bin.
__global__ void focus_setup_kernel(FocusArgs a) {
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g < a.T) {
    aperture_bounds(a.s, a.T, a.half, g, const_cast<int *>(a.jr));
    return;
  }
  const int b = g - a.T;
  if (a.bins && b < a.nb) {
    const BinConsts q = bin_consts(a, b);
    // a fraction just below 1 must not round up to 1.0f: the base index
    // (and with it the validity of the last bin) is the float64 one
    a.bins[b] = make_float4(__int_as_float(q.i00),
                            fminf((float)q.frac0, 0.99999994f), (float)q.r0,
                            (float)(2.0 / (a.c * q.dt)));
  }
}

// hann 0.5 (1 + cos(pi d / half)) (processing.py:315-316), or 1.
__device__ __forceinline__ double aperture_weight(const FocusArgs &a,
                                                  double d) {
  return a.window == SS_WIN_HANN
             ? 0.5 * __dadd_rn(1.0, cos(__ddiv_rn(__dmul_rn(kPi, d), a.half)))
             : 1.0;
}

// FP64 form: one output trace x 256 bins per CTA, the reference's float64
// chain term by term.
__global__ void __launch_bounds__(256) focus_fp64_kernel(FocusArgs a) {
  __shared__ double s_d[256];
  __shared__ double s_w[256];
  const int tid = threadIdx.x;
  const int i = blockIdx.x;  // output traces fastest: neighbours share rows
  const int b = blockIdx.y * 256 + tid;
  const bool live = b < a.nb;
  const BinConsts q = bin_consts(a, b);
  const int jlo = a.jr[2 * i], jhi = a.jr[2 * i + 1];
  const double si = a.s[i];
  const int nb1 = a.nb - 1;
  double accr = 0.0, acci = 0.0;

  for (int j0 = jlo; j0 < jhi; j0 += 256) {
    __syncthreads();
    if (j0 + tid < jhi) {
      const double d = __dsub_rn(a.s[j0 + tid], si);
      s_d[tid] = d;
      s_w[tid] = aperture_weight(a, d);
    }
    __syncthreads();
    const int nj = min(256, jhi - j0);
    if (!live) continue;
    for (int jj = 0; jj < nj; ++jj) {
      const long row = (long)(j0 + jj) * a.nb;
      const double d = s_d[jj];
      const double dr = __dsub_rn(
          __dsqrt_rn(__dadd_rn(__dmul_rn(q.r0, q.r0), __dmul_rn(d, d))),
          q.r0);
      const double x = __ddiv_rn(
          __dsub_rn(__dadd_rn(q.tb, __ddiv_rn(__dmul_rn(2.0, dr), a.c)),
                    q.t0),
          q.dt);
      const double fl = floor(x);
      if (fl < 0.0 || fl >= (double)nb1) continue;
      const int ix = (int)fl;
      const double fr = __dsub_rn(x, fl);
      double ar, ai, br, bi;
      if (a.in_f64) {
        const double2 *f = reinterpret_cast<const double2 *>(a.field);
        const double2 u = f[row + ix], v = f[row + ix + 1];
        ar = u.x; ai = u.y; br = v.x; bi = v.y;
      } else {
        const float2 *f = reinterpret_cast<const float2 *>(a.field);
        const float2 u = f[row + ix], v = f[row + ix + 1];
        ar = u.x; ai = u.y; br = v.x; bi = v.y;
      }
      const double om = __dsub_rn(1.0, fr);
      const double sr = __dadd_rn(__dmul_rn(ar, om), __dmul_rn(br, fr));
      const double sim = __dadd_rn(__dmul_rn(ai, om), __dmul_rn(bi, fr));
      double sn, cs;
      sincos(__dmul_rn(2.0 * a.k, dr), &sn, &cs);
      const double w = s_w[jj];
      const double pr = __dmul_rn(w, sr), pi = __dmul_rn(w, sim);
      accr = __dadd_rn(accr, __dsub_rn(__dmul_rn(pr, cs), __dmul_rn(pi, sn)));
      acci = __dadd_rn(acci, __dadd_rn(__dmul_rn(pr, sn), __dmul_rn(pi, cs)));
    }
  }
  if (live) write_out(a, (long)i * a.nb + b, accr, acci);
}

// Split (float32) form: TI output traces x 256 bins per CTA. The rows of
// the traces' union aperture are staged RJ at a time in shared memory, bins
// [b0 - 1, b0 - 1 + W) with W covering the largest range migration of the
// tile, so each row is read from L2 once for all TI output traces. A sample
// outside the staged span (a migration wider than the cap) is read from
// global memory instead.
constexpr int kFocTI = 8;    // output traces per CTA
constexpr int kFocRJ = 8;    // aperture rows staged per step
constexpr int kFocWMax = 736;  // staged bins per row (cap; 46 KB of rows)

__global__ void __launch_bounds__(256) focus_split_kernel(FocusArgs a) {
  __shared__ float2 s_row[kFocRJ][kFocWMax];
  __shared__ float s_d[kFocTI][kFocRJ], s_w[kFocTI][kFocRJ];
  __shared__ int s_W;
  const int tid = threadIdx.x;
  const int i0 = blockIdx.x * kFocTI;
  const int ni = min(kFocTI, a.T - i0);
  const int b0 = blockIdx.y * 256;
  const int b = b0 + tid;
  const int base = b0 - 1;  // the d = 0 sample may sit one bin below b
  const bool live = b < a.nb;
  // per-bin base index, fraction, r0 and bins per metre of dr
  const float4 bt = a.bins[live ? b : 0];
  const int i00 = __float_as_int(bt.x);
  const float frac0f = bt.y, r0f = bt.z, kx = bt.w;
  const int J0 = a.jr[2 * i0], J1 = a.jr[2 * (i0 + ni - 1) + 1];
  const int nb1 = a.nb - 1;
  const float half_f = (float)a.half;
  if (tid == 0) {
    // widest migration of the tile: largest |d| at the nearest bin
    double dmax = 0.0;
    for (int t = 0; t < ni; ++t) {
      const int lo = a.jr[2 * (i0 + t)], hi = a.jr[2 * (i0 + t) + 1];
      if (hi > lo) {
        const double si = a.s[i0 + t];
        dmax = fmax(dmax, fmax(fabs(a.s[lo] - si), fabs(a.s[hi - 1] - si)));
      }
    }
    const double r0n = 0.5 * a.c * a.twtt[b0];
    const double drm = dmax * dmax / (sqrt(r0n * r0n + dmax * dmax) + r0n);
    const double h = 258.0 + 4.0 + drm * (double)kx;
    s_W = (int)fmin(h, (double)kFocWMax);
  }
  const float r0sq = r0f * r0f;
  const float k2f = (float)(2.0 * a.k);
  float accr[kFocTI], acci[kFocTI];
#pragma unroll
  for (int t = 0; t < kFocTI; ++t) accr[t] = acci[t] = 0.f;
  const float2 *F = reinterpret_cast<const float2 *>(a.field);

  for (int j0 = J0; j0 < J1; j0 += kFocRJ) {
    __syncthreads();  // previous rows consumed; s_W visible
    const int W = s_W;
    const int nr = min(kFocRJ, J1 - j0);
    for (int r = 0; r < nr; ++r) {
      const long row = (long)(j0 + r) * a.nb;
      for (int k = tid; k < W; k += 256) {
        const int g = base + k;
        float2 v = make_float2(0.f, 0.f);
        if (g >= 0 && g < a.nb) {
          if (a.in_f64) {
            const double2 u =
                reinterpret_cast<const double2 *>(a.field)[row + g];
            v = make_float2((float)u.x, (float)u.y);
          } else {
            v = __ldg(F + row + g);
          }
        }
        s_row[r][k] = v;
      }
    }
    if (tid < kFocTI * kFocRJ) {
      const int t = tid / kFocRJ, r = tid % kFocRJ;
      float d = 0.f, w = 0.f;  // w = 0: row outside this trace's aperture
      if (t < ni && r < nr) {
        const int i = i0 + t, j = j0 + r;
        if (j >= a.jr[2 * i] && j < a.jr[2 * i + 1]) {
          d = (float)__dsub_rn(a.s[j], a.s[i]);
          w = a.window == SS_WIN_HANN
                  ? 0.5f * (1.0f + cospif(__fdiv_rn(d, half_f)))
                  : 1.0f;
        }
      }
      s_d[t][r] = d;
      s_w[t][r] = w;
    }
    __syncthreads();
    if (!live) continue;
    for (int r = 0; r < nr; ++r) {
#pragma unroll
      for (int t = 0; t < kFocTI; ++t) {
        const float w = s_w[t][r];
        if (w == 0.f) continue;
        const float d = s_d[t][r];
        const float q2 = __fmaf_rn(d, d, r0sq);
        const float R = q2 * rsqrtf(q2);
        const float dr = __fdividef(d * d, R + r0f);
        const float xf = __fmaf_rn(dr, kx, frac0f);
        const float fl = floorf(xf);
        const int ix = i00 + (int)fl;
        if ((unsigned)ix >= (unsigned)nb1) continue;
        const float fr = xf - fl;
        const int loc = ix - base;
        float2 u, v;
        if (loc + 1 < W) {
          u = s_row[r][loc];
          v = s_row[r][loc + 1];
        } else {
          const long row = (long)(j0 + r) * a.nb;
          if (a.in_f64) {
            const double2 *f = reinterpret_cast<const double2 *>(a.field);
            u = make_float2((float)f[row + ix].x, (float)f[row + ix].y);
            v = make_float2((float)f[row + ix + 1].x,
                            (float)f[row + ix + 1].y);
          } else {
            u = __ldg(F + row + ix);
            v = __ldg(F + row + ix + 1);
          }
        }
        const float sr = __fmaf_rn(fr, v.x - u.x, u.x);
        const float sim = __fmaf_rn(fr, v.y - u.y, u.y);
        float sn, cs;
        __sincosf(reduce_2pi(k2f * dr), &sn, &cs);
        const float pr = w * sr, pi = w * sim;
        accr[t] += pr * cs - pi * sn;
        acci[t] += pr * sn + pi * cs;
      }
    }
  }
  if (!live) return;
#pragma unroll
  for (int t = 0; t < kFocTI; ++t)
    if (t < ni) write_out(a, (long)(i0 + t) * a.nb + b, accr[t], acci[t]);
}

}  // namespace ss

using namespace ss;

// Scratch: aperture bounds (T, 2) int32, then the (nb,) float4 bin table.
static size_t focus_bounds_bytes(int T) {
  return ((size_t)T * 2 * sizeof(int) + 15) & ~(size_t)15;
}

extern "C" size_t ss_focused_sar_scratch_bytes(const ss_focus_opts *opts) {
  if (!opts || opts->n_traces <= 0 || opts->n_bins <= 0) return 0;
  return focus_bounds_bytes(opts->n_traces) +
         (size_t)opts->n_bins * sizeof(float4);
}

extern "C" int ss_focused_sar(const ss_focus_opts *opts, const void *field,
                              const double *twtt, const double *s,
                              const ss_focus_output *out, void *scratch,
                              size_t scratch_bytes, void *stream) {
  if (!opts || !field || !twtt || !s || !out ||
      !(out->field_c128 || out->field_c64 || out->power)) {
    set_error("ss_focused_sar: null argument");
    return SS_ERR_ARG;
  }
  if (opts->n_traces <= 0 || opts->n_bins < 2 ||
      !(opts->wavelength > 0.0) || !(opts->c > 0.0) ||
      (opts->window != SS_WIN_HANN && opts->window != SS_WIN_RECT) ||
      (opts->precision != SS_PREC_FP64 && opts->precision != SS_PREC_SPLIT)) {
    set_error("ss_focused_sar: bad sizes or options");
    return SS_ERR_ARG;
  }
  const size_t need = ss_focused_sar_scratch_bytes(opts);
  if (!scratch || scratch_bytes < need) {
    set_error("ss_focused_sar: scratch too small");
    return SS_ERR_SCRATCH;
  }
  FocusArgs a{};
  a.field = field;
  a.twtt = twtt;
  a.s = s;
  a.jr = reinterpret_cast<int *>(scratch);
  a.bins = reinterpret_cast<float4 *>(reinterpret_cast<char *>(scratch) +
                                      focus_bounds_bytes(opts->n_traces));
  a.T = opts->n_traces;
  a.nb = opts->n_bins;
  a.window = opts->window;
  a.in_f64 = opts->in_f64 ? 1 : 0;
  a.k = 2.0 * kPi / opts->wavelength;  // processing.py:304
  a.c = opts->c;
  a.half = opts->aperture_m / 2.0;
  a.out = *out;
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  const long n_setup = (long)a.T + a.nb;
  focus_setup_kernel<<<(int)((n_setup + 255) / 256), 256, 0, st>>>(a);
  int e = cuda_status(cudaGetLastError(), "focus setup launch");
  if (e != SS_OK) return e;
  if ((a.nb + 255) / 256 > 65535) {
    set_error("ss_focused_sar: too many bins");
    return SS_ERR_UNSUPPORTED;
  }
  if (opts->precision == SS_PREC_FP64) {
    dim3 grid(a.T, (a.nb + 255) / 256);
    focus_fp64_kernel<<<grid, 256, 0, st>>>(a);
  } else {
    dim3 grid((a.T + kFocTI - 1) / kFocTI, (a.nb + 255) / 256);
    focus_split_kernel<<<grid, 256, 0, st>>>(a);
  }
  return cuda_status(cudaGetLastError(), "focus launch");
}
