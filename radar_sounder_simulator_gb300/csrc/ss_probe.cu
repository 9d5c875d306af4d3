// FP32 and FP64 pipe throughput probes.
//
// The facet kernels are bound by the FP32 (FMA) pipe, not by HBM or the
// tensor cores, so their roofline denominator is the FP32 FMA rate this GPU
// sustains at its present clocks (the float64 FFT of the pulse compression
// is bound by the FP64 pipe, measured the same way). Every thread runs
// eight independent fused multiply-add chains (enough to cover the FMA
// latency at full occupancy) and stores their sum so nothing is optimised
// away. FLOP per launch = blocks x threads x 8 chains x iters x 2.
#include "ss_internal.cuh"

namespace ss {

__global__ void __launch_bounds__(256)
fp32_fma_probe_kernel(int iters, float x, float y, float *out) {
  float a[8];
#pragma unroll
  for (int j = 0; j < 8; ++j) a[j] = (float)(threadIdx.x + j);
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int j = 0; j < 8; ++j) a[j] = __fmaf_rn(a[j], x, y);
  }
  float s = 0.0f;
#pragma unroll
  for (int j = 0; j < 8; ++j) s += a[j];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

__global__ void __launch_bounds__(256)
fp64_fma_probe_kernel(int iters, double x, double y, double *out) {
  double a[8];
#pragma unroll
  for (int j = 0; j < 8; ++j) a[j] = (double)(threadIdx.x + j);
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int j = 0; j < 8; ++j) a[j] = __fma_rn(a[j], x, y);
  }
  double s = 0.0;
#pragma unroll
  for (int j = 0; j < 8; ++j) s += a[j];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

// MUFU (special function unit) probe: eight independent chains of the
// base-2 exponential x <- 2^-x (bounded in (0, 1)), one MUFU operation per
// step. Operations per launch = blocks x threads x 8 x iters.
__global__ void __launch_bounds__(256)
mufu_probe_kernel(int iters, float *out) {
  float a[8];
#pragma unroll
  for (int j = 0; j < 8; ++j) a[j] = 0.001f * (float)(threadIdx.x + j);
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int j = 0; j < 8; ++j)
      asm volatile("ex2.approx.ftz.f32 %0, %1;" : "=f"(a[j]) : "f"(-a[j]));
  }
  float s = 0.0f;
#pragma unroll
  for (int j = 0; j < 8; ++j) s += a[j];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

}  // namespace ss

extern "C" int ss_mufu_probe(int32_t blocks, int32_t iters, float *out,
                             void *stream) {
  using namespace ss;
  if (blocks <= 0 || iters <= 0 || !out) {
    set_error("bad probe arguments");
    return SS_ERR_ARG;
  }
  mufu_probe_kernel<<<blocks, 256, 0, static_cast<cudaStream_t>(stream)>>>(
      iters, out);
  return cuda_status(cudaGetLastError(), "mufu probe launch");
}

extern "C" int ss_fp64_fma_probe(int32_t blocks, int32_t iters, double *out,
                                 void *stream) {
  using namespace ss;
  if (blocks <= 0 || iters <= 0 || !out) {
    set_error("bad probe arguments");
    return SS_ERR_ARG;
  }
  fp64_fma_probe_kernel<<<blocks, 256, 0, static_cast<cudaStream_t>(stream)>>>(
      iters, 0.999999, 1e-6, out);
  return cuda_status(cudaGetLastError(), "fp64 probe launch");
}

extern "C" int ss_fp32_fma_probe(int32_t blocks, int32_t iters, float *out,
                                 void *stream) {
  using namespace ss;
  if (blocks <= 0 || iters <= 0 || !out) {
    set_error("bad probe arguments");
    return SS_ERR_ARG;
  }
  fp32_fma_probe_kernel<<<blocks, 256, 0, static_cast<cudaStream_t>(stream)>>>(
      iters, 0.999999f, 1e-6f, out);
  return cuda_status(cudaGetLastError(), "fp32 probe launch");
}
