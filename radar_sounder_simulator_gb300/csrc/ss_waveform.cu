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
