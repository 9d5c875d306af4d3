// Double-float ("split") arithmetic on the FP32 pipe.
//
// A value is carried as an unevaluated sum hi + lo of two floats
// (|lo| <= ulp(hi)/2 after renormalisation), giving ~48 significant bits at
// FP32-pipe throughput. Error-free transformations used:
//   two_sum       -- Knuth (TAOCP vol. 2, 4.2.2): s + e == a + b exactly
//   fast_two_sum  -- Dekker (1971): same, requires |a| >= |b|
//   two_prod      -- via fused multiply-add: p + e == a * b exactly
// GB300's FP64 rate is a small fraction of its FP32 rate, so the split form
// keeps only these few operations per pair at ~48-bit precision and runs the
// rest in plain float32.
#pragma once

#include <cuda_runtime.h>

namespace ss {

struct df {
  float hi, lo;
};

__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e) {
  s = __fadd_rn(a, b);
  float bb = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

__device__ __forceinline__ void fast_two_sum(float a, float b, float &s,
                                             float &e) {
  s = __fadd_rn(a, b);
  e = __fsub_rn(b, __fsub_rn(s, a));
}

__device__ __forceinline__ void two_prod(float a, float b, float &p,
                                         float &e) {
  p = __fmul_rn(a, b);
  e = __fmaf_rn(a, b, -p);
}

// Split a double into hi + lo floats (host or device).
__host__ __device__ __forceinline__ df df_from_double(double v) {
  df r;
  r.hi = (float)v;
  r.lo = (float)(v - (double)r.hi);
  return r;
}

}  // namespace ss
