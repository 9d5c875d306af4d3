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

static int fft_size(const ss_waveform_opts *o, int *log_n) {
  const long need = (long)o->n_samples + o->n_taps - 1;
  int lg = 1;
  while ((1L << lg) < need) ++lg;
  *log_n = lg;
  return lg <= kFftMaxLog ? (1 << lg) : 0;
}

}  // namespace ss

extern "C" size_t ss_range_compress_fft_scratch_bytes(
    const ss_waveform_opts *o) {
  using namespace ss;
  if (!o || o->n_samples <= 0 || o->n_taps <= 0) return 0;
  int lg;
  const int N = fft_size(o, &lg);
  if (!N) return 0;
  return (size_t)N * sizeof(double2) + (size_t)(N / 2) * sizeof(double2);
}

extern "C" int ss_range_compress_fft(const ss_waveform_opts *o,
                                     const double *taps, const void *in,
                                     void *out, void *scratch,
                                     size_t scratch_bytes, void *stream) {
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
  int lg;
  const int N = fft_size(o, &lg);
  if (!N) {
    set_error("n_samples + n_taps - 1 above 8192: use ss_range_compress");
    return SS_ERR_UNSUPPORTED;
  }
  const size_t need = ss_range_compress_fft_scratch_bytes(o);
  if (!scratch || scratch_bytes < need) {
    set_error("scratch buffer too small");
    return SS_ERR_SCRATCH;
  }
  const long rows = (long)o->n_traces * o->n_lanes;
  if (rows > 0x7fffffffL) {
    set_error("too many rows");
    return SS_ERR_UNSUPPORTED;
  }
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  double2 *spec = static_cast<double2 *>(scratch);
  double2 *tw = spec + N;
  const size_t smem = (size_t)N * sizeof(double2);
  fft_twiddle_kernel<<<(N / 2 + 255) / 256, 256, 0, st>>>(N, tw);
  cudaError_t e = cudaFuncSetAttribute(
      fft_pulse_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
      (int)smem);
  if (e != cudaSuccess) return cuda_status(e, "fft smem");
  fft_pulse_kernel<<<1, kFftThreads, smem, st>>>(N, lg, o->n_taps, o->power,
                                                 taps, tw, spec);
#define SS_FFT_LAUNCH(P, F)                                                  \
  e = cudaFuncSetAttribute(range_compress_fft_kernel<P, F>,                  \
                           cudaFuncAttributeMaxDynamicSharedMemorySize,      \
                           (int)smem);                                       \
  if (e != cudaSuccess) return cuda_status(e, "fft smem");                   \
  range_compress_fft_kernel<P, F><<<(unsigned)rows, kFftThreads, smem, st>>>( \
      o->n_samples, o->n_lanes, N, lg, o->center, tw, spec, in, out);
  if (o->power) {
    if (o->in_f64) { SS_FFT_LAUNCH(true, true) } else { SS_FFT_LAUNCH(true, false) }
  } else {
    if (o->in_f64) { SS_FFT_LAUNCH(false, true) } else { SS_FFT_LAUNCH(false, false) }
  }
#undef SS_FFT_LAUNCH
  return cuda_status(cudaGetLastError(), "range_compress_fft launch");
}
