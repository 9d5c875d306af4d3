// Post-kernel pulse compression: 'same'-mode convolution of each trace's
// fast-time samples with the compressed pulse (waveform.py:126-160).
//
// The reference convolves by FFT in complex128 and casts the result to
// complex64 (coherent) or clips and casts to float32 (incoherent power
// envelope). Here each output sample is a direct sum over the pulse taps,
// y[i] = sum_j p[j] x[i + center - j], with the taps carried as
// double-floats and every product formed exactly (FMA two-product) and
// accumulated with a two-sum compensation term on the FP32 pipe -- the
// result carries ~2^-44 relative error in the sum of |terms|, well inside
// the float32 rounding of the output, at a fraction of the FP64 pipe's
// cost.
//
// CTA = 256 consecutive output samples of one (trace, lane) row. Taps are
// streamed through shared memory in chunks of kTapChunk together with the
// matching input window, so any pulse length works.
#include "ss_df.cuh"
#include "ss_internal.cuh"

namespace ss {

constexpr int kWfTile = 256;
constexpr int kTapChunk = 512;

// Compensated accumulator: value = s + c.
struct Acc {
  float s, c;
};

__device__ __forceinline__ void acc_add_prod(Acc &a, float th, float tl,
                                             float x) {
  float p, e;
  two_prod(th, x, p, e);
  float s, e2;
  two_sum(a.s, p, s, e2);
  a.s = s;
  a.c += e2 + __fmaf_rn(tl, x, e);
}

template <bool POWER, bool IN_F64>
__global__ void __launch_bounds__(kWfTile)
range_compress_kernel(int T, int B, int L, int n_taps, int center,
                      const double *taps, const void *in, void *out) {
  // taps as double-floats: (re_hi, re_lo, im_hi, im_lo)
  __shared__ float4 s_tap[kTapChunk];
  __shared__ float2 s_x[kWfTile + kTapChunk];
  const int row = blockIdx.y;  // t * L + l
  const int t = row / L, l = row % L;
  const int i0 = blockIdx.x * kWfTile;
  const int tid = threadIdx.x;
  const int i = i0 + tid;
  Acc ar{0.0f, 0.0f}, ai{0.0f, 0.0f};
  for (int j0 = 0; j0 < n_taps; j0 += kTapChunk) {
    const int J = min(kTapChunk, n_taps - j0);
    __syncthreads();
    for (int j = tid; j < J; j += kWfTile) {
      if (POWER) {
        const df v = df_from_double(taps[j0 + j]);
        s_tap[j] = make_float4(v.hi, v.lo, 0.0f, 0.0f);
      } else {
        const df re = df_from_double(taps[2 * (j0 + j)]);
        const df im = df_from_double(taps[2 * (j0 + j) + 1]);
        s_tap[j] = make_float4(re.hi, re.lo, im.hi, im.lo);
      }
    }
    // input window: x[i0 + center - j0 - J + 1 + k], k in [0, kWfTile + J - 1)
    const long xb = (long)i0 + center - j0 - J + 1;
    const int W = kWfTile + J - 1;
    for (int k = tid; k < W; k += kWfTile) {
      const long xi = xb + k;
      float2 v = make_float2(0.0f, 0.0f);
      if (xi >= 0 && xi < B) {
        const size_t e = ((size_t)t * B + xi) * L + l;
        if (POWER) {
          v.x = IN_F64 ? (float)static_cast<const double *>(in)[e]
                       : static_cast<const float *>(in)[e];
        } else if (IN_F64) {
          const double *d = static_cast<const double *>(in) + 2 * e;
          v = make_float2((float)d[0], (float)d[1]);
        } else {
          v = static_cast<const float2 *>(in)[e];
        }
      }
      s_x[k] = v;
    }
    __syncthreads();
    // output i uses x[i + center - j] = s_x[tid + (J - 1) - (j - j0)]
    const float2 *xp = s_x + tid + J - 1;
    for (int j = 0; j < J; ++j) {
      const float4 tp = s_tap[j];
      const float2 x = xp[-j];
      if (POWER) {
        acc_add_prod(ar, tp.x, tp.y, x.x);
      } else {
        acc_add_prod(ar, tp.x, tp.y, x.x);
        acc_add_prod(ar, -tp.z, -tp.w, x.y);
        acc_add_prod(ai, tp.x, tp.y, x.y);
        acc_add_prod(ai, tp.z, tp.w, x.x);
      }
    }
  }
  if (i < B) {
    const size_t e = ((size_t)t * B + i) * L + l;
    if (POWER) {
      static_cast<float *>(out)[e] = fmaxf(ar.s + ar.c, 0.0f);
    } else {
      static_cast<float2 *>(out)[e] = make_float2(ar.s + ar.c, ai.s + ai.c);
    }
  }
}

}  // namespace ss

extern "C" int ss_range_compress(const ss_waveform_opts *o,
                                 const double *taps, const void *in,
                                 void *out, void *stream) {
  using namespace ss;
  if (!o || !taps || !in || !out) {
    set_error("null argument");
    return SS_ERR_ARG;
  }
  if (o->n_traces <= 0 || o->n_samples <= 0 || o->n_lanes <= 0 ||
      o->n_taps <= 0 || o->center < 0 || o->center >= o->n_taps) {
    set_error("bad waveform sizes (n_traces, n_samples, n_lanes, n_taps > 0;"
              " 0 <= center < n_taps)");
    return SS_ERR_ARG;
  }
  const long rows = (long)o->n_traces * o->n_lanes;
  if (rows > 65535) {
    set_error("n_traces x n_lanes above 65535 rows per call");
    return SS_ERR_UNSUPPORTED;
  }
  dim3 grid((o->n_samples + kWfTile - 1) / kWfTile, (unsigned)rows);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const int T = o->n_traces, B = o->n_samples, L = o->n_lanes;
  if (o->power) {
    if (o->in_f64)
      range_compress_kernel<true, true><<<grid, kWfTile, 0, st>>>(
          T, B, L, o->n_taps, o->center, taps, in, out);
    else
      range_compress_kernel<true, false><<<grid, kWfTile, 0, st>>>(
          T, B, L, o->n_taps, o->center, taps, in, out);
  } else {
    if (o->in_f64)
      range_compress_kernel<false, true><<<grid, kWfTile, 0, st>>>(
          T, B, L, o->n_taps, o->center, taps, in, out);
    else
      range_compress_kernel<false, false><<<grid, kWfTile, 0, st>>>(
          T, B, L, o->n_taps, o->center, taps, in, out);
  }
  return cuda_status(cudaGetLastError(), "range_compress launch");
}

// ---------------------------------------------------------------------
// FFT form: the reference's own method (waveform.py:126-138 convolves by
// FFT in complex128), in float64 in shared memory. One CTA per (trace,
// lane) row: the row is zero-padded to a power of two N >= B + M - 1, put
// in bit-reversed order, transformed by an iterative radix-2 decimation-in-
// time FFT, multiplied by the pulse spectrum, transformed back, and the
// 'same'-mode window [center, center + B) written out. The pulse spectrum
// and the twiddles are computed once per call into the caller's scratch.
// For N up to 8192 (128 KB of complex128 in shared memory).
// ---------------------------------------------------------------------
namespace ss {

constexpr int kFftThreads = 512;
constexpr int kFftMaxLog = 13;

__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
  return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

__device__ __forceinline__ unsigned bitrev(unsigned i, int log_n) {
  return __brev(i) >> (32 - log_n);
}

// e^{-2 pi i k / N}, k < N/2
__global__ void fft_twiddle_kernel(int N, double2 *tw) {
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < N / 2;
       k += gridDim.x * blockDim.x) {
    double s, c;
    sincospi(-2.0 * (double)k / (double)N, &s, &c);
    tw[k] = make_double2(c, s);
  }
}

// In-place radix-2 DIT on bit-reversed input (natural-order output).
// inverse: conjugate twiddles (no scaling).
__device__ void fft_dit(double2 *x, int N, int log_n, const double2 *tw,
                        bool inverse) {
  for (int s = 1; s <= log_n; ++s) {
    const int half = 1 << (s - 1);
    const int stride = N >> s;
    for (int b = threadIdx.x; b < N / 2; b += blockDim.x) {
      const int grp = b >> (s - 1), pos = b & (half - 1);
      const int i0 = (grp << s) + pos, i1 = i0 + half;
      double2 w = tw[pos * stride];
      if (inverse) w.y = -w.y;
      const double2 u = x[i0], v = cmul(x[i1], w);
      x[i0] = make_double2(u.x + v.x, u.y + v.y);
      x[i1] = make_double2(u.x - v.x, u.y - v.y);
    }
    __syncthreads();
  }
}

// Spectrum of the pulse taps (zero-padded to N).
__global__ void __launch_bounds__(kFftThreads)
fft_pulse_kernel(int N, int log_n, int n_taps, int power, const double *taps,
                 const double2 *tw, double2 *spec) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  double2 *x = reinterpret_cast<double2 *>(smem_raw);
  for (int i = threadIdx.x; i < N; i += blockDim.x) {
    double2 v = make_double2(0.0, 0.0);
    if (i < n_taps)
      v = power ? make_double2(taps[i], 0.0)
                : make_double2(taps[2 * i], taps[2 * i + 1]);
    x[bitrev(i, log_n)] = v;
  }
  __syncthreads();
  fft_dit(x, N, log_n, tw, false);
  for (int i = threadIdx.x; i < N; i += blockDim.x) spec[i] = x[i];
}

template <bool POWER, bool IN_F64>
__global__ void __launch_bounds__(kFftThreads)
range_compress_fft_kernel(int B, int L, int N, int log_n, int center,
                          const double2 *tw, const double2 *spec,
                          const void *in, void *out) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  double2 *x = reinterpret_cast<double2 *>(smem_raw);
  const int row = blockIdx.x;  // t * L + l
  const int t = row / L, l = row % L;
  for (int i = threadIdx.x; i < N; i += blockDim.x) {
    double2 v = make_double2(0.0, 0.0);
    if (i < B) {
      const size_t e = ((size_t)t * B + i) * L + l;
      // the reference convolves the kernels' complex64 output: the input
      // is rounded to float32 first, as there
      if (POWER) {
        v.x = IN_F64 ? (double)(float)static_cast<const double *>(in)[e]
                     : (double)static_cast<const float *>(in)[e];
      } else if (IN_F64) {
        const double *d = static_cast<const double *>(in) + 2 * e;
        v = make_double2((double)(float)d[0], (double)(float)d[1]);
      } else {
        const float2 f = static_cast<const float2 *>(in)[e];
        v = make_double2(f.x, f.y);
      }
    }
    x[bitrev(i, log_n)] = v;
  }
  __syncthreads();
  fft_dit(x, N, log_n, tw, false);
  // multiply by the pulse spectrum and return to bit-reversed order
  for (int i = threadIdx.x; i < N; i += blockDim.x) x[i] = cmul(x[i], spec[i]);
  __syncthreads();
  for (int i = threadIdx.x; i < N; i += blockDim.x) {
    const int r = bitrev(i, log_n);
    if (i < r) {
      const double2 a = x[i];
      x[i] = x[r];
      x[r] = a;
    }
  }
  __syncthreads();
  fft_dit(x, N, log_n, tw, true);
  const double inv = 1.0 / N;
  for (int i = threadIdx.x; i < B; i += blockDim.x) {
    const double2 y = x[center + i];
    const size_t e = ((size_t)t * B + i) * L + l;
    if (POWER)
      static_cast<float *>(out)[e] = (float)fmax(y.x * inv, 0.0);
    else
      static_cast<float2 *>(out)[e] =
          make_float2((float)(y.x * inv), (float)(y.y * inv));
  }
}

// ---------------------------------------------------------------------
// Double-float FFT form: the same FFT convolution with every value carried
// as a double-float complex (hi + lo floats, ~48 significant bits) on the
// FP32 pipe, which GB300 runs at ~75x its FP64 rate.
//
// Radix-4 decimation in frequency takes the natural-order row to a base-4
// digit-reversed spectrum; the pulse spectrum, made by the same transform,
// is in the same order, so the pointwise product needs no reordering, and
// the mirrored radix-4 decimation-in-time inverse (conjugate twiddles)
// returns natural order. When log2 N is odd a radix-2 stage of block
// length 2 (twiddle 1) ends the forward transform and starts the inverse.
// Butterfly sums are double-float additions (two-sum of the high parts);
// twiddle products form both leading products exactly by FMA, so each
// value carries ~2^-46 relative error per stage: after both transforms the
// result agrees with the float64 FFT to ~1e-14 of the row's magnitude,
// below the float32 rounding of the output.
//
// Twiddles: for the radix-4 stage of quarter length q (block L = 4q) the
// table holds w^{jk}, w = e^{-2 pi i / L}, k = 1..3, j < q, consecutive in
// j (entries [N - 4q, N - q) of an N-entry table), read through the
// read-only cache: threads of a warp read consecutive entries, or the same
// one, in every stage.
//
// Plan (once per pulse): twiddle table and pulse spectrum, 32 N bytes.
// Apply: one CTA per (trace, lane) row, the row in shared memory as
// float4 (re.hi, re.lo, im.hi, im.lo): 16 N bytes, two CTAs per SM at
// N = 4096.
// ---------------------------------------------------------------------
constexpr int kDfThreads = 512;

struct cdf {
  df re, im;
};

__device__ __forceinline__ cdf c_ld(const float4 *x, int i) {
  const float4 v = x[i];
  return cdf{df{v.x, v.y}, df{v.z, v.w}};
}

__device__ __forceinline__ cdf c_ldg(const float4 *x, int i) {
  const float4 v = __ldg(x + i);
  return cdf{df{v.x, v.y}, df{v.z, v.w}};
}

__device__ __forceinline__ void c_st(float4 *x, int i, const cdf &a) {
  x[i] = make_float4(a.re.hi, a.re.lo, a.im.hi, a.im.lo);
}

__device__ __forceinline__ cdf c_add(const cdf &a, const cdf &b) {
  return cdf{df_add(a.re, b.re), df_add(a.im, b.im)};
}

__device__ __forceinline__ cdf c_sub(const cdf &a, const cdf &b) {
  return cdf{df_sub(a.re, b.re), df_sub(a.im, b.im)};
}

// a b + c d: both leading products exact (FMA two-product) and summed by
// a two-sum, the cross terms added to the low part
__device__ __forceinline__ df df_dot2(df a, df b, df c, df d) {
  float p1, e1, p2, e2, s, e3;
  two_prod(a.hi, b.hi, p1, e1);
  two_prod(c.hi, d.hi, p2, e2);
  two_sum(p1, p2, s, e3);
  float lo = (e1 + e2) + e3;
  lo = __fmaf_rn(a.hi, b.lo, __fmaf_rn(a.lo, b.hi, lo));
  lo = __fmaf_rn(c.hi, d.lo, __fmaf_rn(c.lo, d.hi, lo));
  return df_make(s, lo);
}

__device__ __forceinline__ cdf c_mul(const cdf &a, const cdf &w) {
  return cdf{df_dot2(a.re, w.re, df_neg(a.im), w.im),
             df_dot2(a.re, w.im, a.im, w.re)};
}

__device__ __forceinline__ cdf c_conj(cdf a) {
  a.im = df_neg(a.im);
  return a;
}

// Forward transform in place, natural order in, digit-reversed out.
__device__ void df_fft_forward(float4 *x, int N, int lg,
                               const float4 *__restrict__ tw) {
  for (int lq = lg - 2; lq >= 0; lq -= 2) {
    const int q = 1 << lq;
    const float4 *T = tw + (N - 4 * q);
    for (int b = threadIdx.x; b < (N >> 2); b += blockDim.x) {
      const int j = b & (q - 1);
      const int base = ((b >> lq) << (lq + 2)) + j;
      const cdf a0 = c_ld(x, base), a1 = c_ld(x, base + q),
                a2 = c_ld(x, base + 2 * q), a3 = c_ld(x, base + 3 * q);
      const cdf b0 = c_add(a0, a2), b1 = c_sub(a0, a2), b2 = c_add(a1, a3),
                b3 = c_sub(a1, a3);
      const cdf mib3{b3.im, df_neg(b3.re)};  // -i b3
      c_st(x, base, c_add(b0, b2));
      c_st(x, base + q, c_mul(c_add(b1, mib3), c_ldg(T, 3 * j)));
      c_st(x, base + 2 * q, c_mul(c_sub(b0, b2), c_ldg(T, 3 * j + 1)));
      c_st(x, base + 3 * q, c_mul(c_sub(b1, mib3), c_ldg(T, 3 * j + 2)));
    }
    __syncthreads();
  }
  if (lg & 1) {
    for (int b = threadIdx.x; b < (N >> 1); b += blockDim.x) {
      const cdf a0 = c_ld(x, 2 * b), a1 = c_ld(x, 2 * b + 1);
      c_st(x, 2 * b, c_add(a0, a1));
      c_st(x, 2 * b + 1, c_sub(a0, a1));
    }
    __syncthreads();
  }
}

// Inverse transform in place (unscaled), digit-reversed in, natural out.
__device__ void df_fft_inverse(float4 *x, int N, int lg,
                               const float4 *__restrict__ tw) {
  if (lg & 1) {
    for (int b = threadIdx.x; b < (N >> 1); b += blockDim.x) {
      const cdf a0 = c_ld(x, 2 * b), a1 = c_ld(x, 2 * b + 1);
      c_st(x, 2 * b, c_add(a0, a1));
      c_st(x, 2 * b + 1, c_sub(a0, a1));
    }
    __syncthreads();
  }
  for (int lq = lg & 1; lq <= lg - 2; lq += 2) {
    const int q = 1 << lq;
    const float4 *T = tw + (N - 4 * q);
    for (int b = threadIdx.x; b < (N >> 2); b += blockDim.x) {
      const int j = b & (q - 1);
      const int base = ((b >> lq) << (lq + 2)) + j;
      const cdf c0 = c_ld(x, base);
      const cdf c1 = c_mul(c_ld(x, base + q), c_conj(c_ldg(T, 3 * j)));
      const cdf c2 = c_mul(c_ld(x, base + 2 * q), c_conj(c_ldg(T, 3 * j + 1)));
      const cdf c3 = c_mul(c_ld(x, base + 3 * q), c_conj(c_ldg(T, 3 * j + 2)));
      const cdf d0 = c_add(c0, c2), d1 = c_sub(c0, c2), d2 = c_add(c1, c3),
                d3 = c_sub(c1, c3);
      const cdf id3{df_neg(d3.im), d3.re};  // +i d3
      c_st(x, base, c_add(d0, d2));
      c_st(x, base + q, c_add(d1, id3));
      c_st(x, base + 2 * q, c_sub(d0, d2));
      c_st(x, base + 3 * q, c_sub(d1, id3));
    }
    __syncthreads();
  }
}

// Twiddle table of the radix-4 stages (float64 sincospi, split to hi + lo).
__global__ void df_twiddle_kernel(int N, int lg, float4 *tw) {
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < N;
       e += gridDim.x * blockDim.x) {
    float4 v = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    for (int lq = lg - 2; lq >= 0; lq -= 2) {
      const int q = 1 << lq;
      if (e >= N - 4 * q && e < N - q) {
        const int r = e - (N - 4 * q), j = r / 3, k = r % 3 + 1;
        const long t = (long)j * k * (N >> (lq + 2));  // w_L^{jk} = w_N^t
        double s, c;
        sincospi(-2.0 * (double)t / (double)N, &s, &c);
        const df dc = df_from_double(c), ds = df_from_double(s);
        v = make_float4(dc.hi, dc.lo, ds.hi, ds.lo);
      }
    }
    tw[e] = v;
  }
}

// Pulse spectrum (digit-reversed order) into the plan.
__global__ void __launch_bounds__(kDfThreads)
df_pulse_kernel(int N, int lg, int n_taps, int power, const double *taps,
                float4 *plan) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float4 *x = reinterpret_cast<float4 *>(smem_raw);
  for (int i = threadIdx.x; i < N; i += blockDim.x) {
    df re{0.0f, 0.0f}, im{0.0f, 0.0f};
    if (i < n_taps) {
      re = df_from_double(power ? taps[i] : taps[2 * i]);
      if (!power) im = df_from_double(taps[2 * i + 1]);
    }
    c_st(x, i, cdf{re, im});
  }
  __syncthreads();
  df_fft_forward(x, N, lg, plan + N);
  for (int i = threadIdx.x; i < N; i += blockDim.x) plan[i] = x[i];
}

template <bool POWER, bool IN_F64>
__global__ void __launch_bounds__(kDfThreads, 2)
range_compress_df_kernel(int B, int L, int N, int lg, int center,
                         const float4 *__restrict__ plan, const void *in,
                         void *out) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float4 *x = reinterpret_cast<float4 *>(smem_raw);
  const int row = blockIdx.x;  // t * L + l
  const int t = row / L, l = row % L;
  for (int i = threadIdx.x; i < N; i += blockDim.x) {
    float vr = 0.0f, vi = 0.0f;
    if (i < B) {
      const size_t e = ((size_t)t * B + i) * L + l;
      // the reference convolves the kernels' complex64 output: the input
      // is rounded to float32 first, as there
      if (POWER) {
        vr = IN_F64 ? (float)static_cast<const double *>(in)[e]
                    : static_cast<const float *>(in)[e];
      } else if (IN_F64) {
        const double *d = static_cast<const double *>(in) + 2 * e;
        vr = (float)d[0];
        vi = (float)d[1];
      } else {
        const float2 f = static_cast<const float2 *>(in)[e];
        vr = f.x;
        vi = f.y;
      }
    }
    x[i] = make_float4(vr, 0.0f, vi, 0.0f);
  }
  __syncthreads();
  df_fft_forward(x, N, lg, plan + N);
  for (int i = threadIdx.x; i < N; i += blockDim.x)
    c_st(x, i, c_mul(c_ld(x, i), c_ldg(plan, i)));
  __syncthreads();
  df_fft_inverse(x, N, lg, plan + N);
  const float inv = 1.0f / (float)N;  // a power of two: exact
  for (int i = threadIdx.x; i < B; i += blockDim.x) {
    const float4 y = x[center + i];
    const size_t e = ((size_t)t * B + i) * L + l;
    // hi + lo rounds the double-float once to float32
    if (POWER)
      static_cast<float *>(out)[e] = fmaxf((y.x + y.y) * inv, 0.0f);
    else
      static_cast<float2 *>(out)[e] =
          make_float2((y.x + y.y) * inv, (y.z + y.w) * inv);
  }
}

static int fft_size(const ss_waveform_opts *o, int *log_n) {
  const long need = (long)o->n_samples + o->n_taps - 1;
  int lg = 1;
  while ((1L << lg) < need) ++lg;
  *log_n = lg;
  return lg <= kFftMaxLog ? (1 << lg) : 0;
}

static int check_opts(const ss_waveform_opts *o) {
  if (o->n_traces <= 0 || o->n_samples <= 0 || o->n_lanes <= 0 ||
      o->n_taps <= 0 || o->center < 0 || o->center >= o->n_taps) {
    set_error("bad waveform sizes (n_traces, n_samples, n_lanes, n_taps > 0;"
              " 0 <= center < n_taps)");
    return SS_ERR_ARG;
  }
  if ((long)o->n_traces * o->n_lanes > 0x7fffffffL) {
    set_error("too many rows");
    return SS_ERR_UNSUPPORTED;
  }
  return SS_OK;
}

static size_t plan_bytes(int N, int precision) {
  return precision == SS_PREC_SPLIT
             ? (size_t)2 * N * sizeof(float4)
             : (size_t)N * sizeof(double2) + (size_t)(N / 2) * sizeof(double2);
}

static int fft_plan(const ss_waveform_opts *o, int precision,
                    const double *taps, void *plan, cudaStream_t st) {
  int lg;
  const int N = fft_size(o, &lg);
  cudaError_t e;
  if (precision == SS_PREC_SPLIT) {
    float4 *p = static_cast<float4 *>(plan);
    df_twiddle_kernel<<<(N + 255) / 256, 256, 0, st>>>(N, lg, p + N);
    const size_t smem = (size_t)N * sizeof(float4);
    e = cudaFuncSetAttribute(df_pulse_kernel,
                             cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)smem);
    if (e != cudaSuccess) return cuda_status(e, "fft smem");
    df_pulse_kernel<<<1, kDfThreads, smem, st>>>(N, lg, o->n_taps, o->power,
                                                 taps, p);
  } else {
    double2 *spec = static_cast<double2 *>(plan);
    double2 *tw = spec + N;
    const size_t smem = (size_t)N * sizeof(double2);
    fft_twiddle_kernel<<<(N / 2 + 255) / 256, 256, 0, st>>>(N, tw);
    e = cudaFuncSetAttribute(fft_pulse_kernel,
                             cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)smem);
    if (e != cudaSuccess) return cuda_status(e, "fft smem");
    fft_pulse_kernel<<<1, kFftThreads, smem, st>>>(N, lg, o->n_taps, o->power,
                                                   taps, tw, spec);
  }
  return cuda_status(cudaGetLastError(), "range compression plan");
}

static int fft_apply(const ss_waveform_opts *o, int precision,
                     const void *plan, const void *in, void *out,
                     cudaStream_t st) {
  int lg;
  const int N = fft_size(o, &lg);
  const unsigned rows = (unsigned)((long)o->n_traces * o->n_lanes);
  cudaError_t e = cudaSuccess;
#define SS_FFT_LAUNCH(KERNEL, THREADS, SMEM, PLAN)                           \
  e = cudaFuncSetAttribute(KERNEL, cudaFuncAttributeMaxDynamicSharedMemorySize, \
                           (int)(SMEM));                                     \
  if (e != cudaSuccess) return cuda_status(e, "fft smem");                   \
  KERNEL<<<rows, THREADS, SMEM, st>>>(o->n_samples, o->n_lanes, N, lg,      \
                                      o->center, PLAN, in, out);
  if (precision == SS_PREC_SPLIT) {
    const float4 *p = static_cast<const float4 *>(plan);
    const size_t smem = (size_t)N * sizeof(float4);
    if (o->power) {
      if (o->in_f64) {
        SS_FFT_LAUNCH((range_compress_df_kernel<true, true>), kDfThreads,
                      smem, p)
      } else {
        SS_FFT_LAUNCH((range_compress_df_kernel<true, false>), kDfThreads,
                      smem, p)
      }
    } else {
      if (o->in_f64) {
        SS_FFT_LAUNCH((range_compress_df_kernel<false, true>), kDfThreads,
                      smem, p)
      } else {
        SS_FFT_LAUNCH((range_compress_df_kernel<false, false>), kDfThreads,
                      smem, p)
      }
    }
  } else {
    const double2 *spec = static_cast<const double2 *>(plan);
    const double2 *tw = spec + N;
    const size_t smem = (size_t)N * sizeof(double2);
#define SS_FFT64(P, F)                                                       \
  e = cudaFuncSetAttribute(range_compress_fft_kernel<P, F>,                  \
                           cudaFuncAttributeMaxDynamicSharedMemorySize,      \
                           (int)smem);                                       \
  if (e != cudaSuccess) return cuda_status(e, "fft smem");                   \
  range_compress_fft_kernel<P, F><<<rows, kFftThreads, smem, st>>>(          \
      o->n_samples, o->n_lanes, N, lg, o->center, tw, spec, in, out);
    if (o->power) {
      if (o->in_f64) { SS_FFT64(true, true) } else { SS_FFT64(true, false) }
    } else {
      if (o->in_f64) { SS_FFT64(false, true) } else { SS_FFT64(false, false) }
    }
#undef SS_FFT64
  }
#undef SS_FFT_LAUNCH
  return cuda_status(cudaGetLastError(), "range compression launch");
}

}  // namespace ss

extern "C" size_t ss_range_compress_fft_scratch_bytes(
    const ss_waveform_opts *o) {
  return ss_range_compress_plan_bytes(o, SS_PREC_FP64);
}

extern "C" int ss_range_compress_fft(const ss_waveform_opts *o,
                                     const double *taps, const void *in,
                                     void *out, void *scratch,
                                     size_t scratch_bytes, void *stream) {
  const int s = ss_range_compress_plan(o, SS_PREC_FP64, taps, scratch,
                                       scratch_bytes, stream);
  if (s != SS_OK) return s;
  return ss_range_compress_apply(o, SS_PREC_FP64, scratch, scratch_bytes, in,
                                 out, stream);
}

extern "C" size_t ss_range_compress_plan_bytes(const ss_waveform_opts *o,
                                               int precision) {
  using namespace ss;
  if (!o || o->n_samples <= 0 || o->n_taps <= 0) return 0;
  if (precision != SS_PREC_FP64 && precision != SS_PREC_SPLIT) return 0;
  int lg;
  const int N = fft_size(o, &lg);
  return N ? plan_bytes(N, precision) : 0;
}

extern "C" int ss_range_compress_plan(const ss_waveform_opts *o,
                                      int precision, const double *taps,
                                      void *plan, size_t plan_size,
                                      void *stream) {
  using namespace ss;
  if (!o || !taps || !plan) {
    set_error("null argument");
    return SS_ERR_ARG;
  }
  int s = check_opts(o);
  if (s != SS_OK) return s;
  if (precision != SS_PREC_FP64 && precision != SS_PREC_SPLIT) {
    set_error("precision must be SS_PREC_FP64 or SS_PREC_SPLIT");
    return SS_ERR_ARG;
  }
  const size_t need = ss_range_compress_plan_bytes(o, precision);
  if (!need) {
    set_error("n_samples + n_taps - 1 above 8192: use ss_range_compress");
    return SS_ERR_UNSUPPORTED;
  }
  if (plan_size < need) {
    set_error("plan buffer too small");
    return SS_ERR_SCRATCH;
  }
  return fft_plan(o, precision, taps, plan, static_cast<cudaStream_t>(stream));
}

extern "C" int ss_range_compress_apply(const ss_waveform_opts *o,
                                       int precision, const void *plan,
                                       size_t plan_size, const void *in,
                                       void *out, void *stream) {
  using namespace ss;
  if (!o || !plan || !in || !out) {
    set_error("null argument");
    return SS_ERR_ARG;
  }
  int s = check_opts(o);
  if (s != SS_OK) return s;
  if (precision != SS_PREC_FP64 && precision != SS_PREC_SPLIT) {
    set_error("precision must be SS_PREC_FP64 or SS_PREC_SPLIT");
    return SS_ERR_ARG;
  }
  const size_t need = ss_range_compress_plan_bytes(o, precision);
  if (!need) {
    set_error("n_samples + n_taps - 1 above 8192: use ss_range_compress");
    return SS_ERR_UNSUPPORTED;
  }
  if (plan_size < need) {
    set_error("plan buffer too small");
    return SS_ERR_SCRATCH;
  }
  return fft_apply(o, precision, plan, in, out,
                   static_cast<cudaStream_t>(stream));
}
