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

__device__ __forceinline__ df df_make(float hi, float lo) {
  df r;
  fast_two_sum(hi, lo, r.hi, r.lo);
  return r;
}

// a - b of two floats, exactly.
__device__ __forceinline__ df df_diff(float a, float b) {
  df r;
  two_sum(a, -b, r.hi, r.lo);
  return r;
}

__device__ __forceinline__ df df_add_f(df a, float b) {
  float s, e;
  two_sum(a.hi, b, s, e);
  return df_make(s, e + a.lo);
}

__device__ __forceinline__ df df_add(df a, df b) {
  float s, e;
  two_sum(a.hi, b.hi, s, e);
  return df_make(s, e + (a.lo + b.lo));
}

__device__ __forceinline__ df df_mul_f(df a, float b) {
  float p, e;
  two_prod(a.hi, b, p, e);
  return df_make(p, __fmaf_rn(a.lo, b, e));
}

__device__ __forceinline__ df df_mul(df a, df b) {
  float p, e;
  two_prod(a.hi, b.hi, p, e);
  e = __fmaf_rn(a.hi, b.lo, __fmaf_rn(a.lo, b.hi, e));
  return df_make(p, e);
}

// |v| of a double-float 3-vector: sum of exact squares, then an rsqrt seed
// with one Newton correction (relative error ~1e-14).
__device__ __forceinline__ df df_norm3(df x, df y, df z) {
  float qx, ex, qy, ey, qz, ez;
  two_prod(x.hi, x.hi, qx, ex);
  two_prod(y.hi, y.hi, qy, ey);
  two_prod(z.hi, z.hi, qz, ez);
  float s1, e1, sh, e2;
  two_sum(qx, qy, s1, e1);
  two_sum(s1, qz, sh, e2);
  float sl = (e1 + e2) + (ex + ey + ez) +
             2.0f * (x.hi * x.lo + y.hi * y.lo + z.hi * z.lo);
  fast_two_sum(sh, sl, sh, sl);
  if (!(sh > 0.0f)) return df_make(0.0f, 0.0f);
  const float r = rsqrtf(sh);
  const float r0 = sh * r;
  const float res = __fmaf_rn(-r0, r0, sh) + sl;
  return df_make(r0, res * (0.5f * r));
}

__device__ __forceinline__ df df_neg(df a) { return df{-a.hi, -a.lo}; }

__device__ __forceinline__ df df_sub(df a, df b) { return df_add(a, df_neg(b)); }

__device__ __forceinline__ df df_abs(df a) {
  return a.hi < 0.0f || (a.hi == 0.0f && a.lo < 0.0f) ? df_neg(a) : a;
}

// a < b for renormalised double-floats.
__device__ __forceinline__ bool df_lt(df a, df b) {
  return a.hi < b.hi || (a.hi == b.hi && a.lo < b.lo);
}

__device__ __forceinline__ df df_max(df a, df b) { return df_lt(a, b) ? b : a; }
__device__ __forceinline__ df df_min(df a, df b) { return df_lt(a, b) ? a : b; }

// a / b: a float32 quotient and two corrections against the double-float
// remainder (~2^-46 relative).
__device__ __forceinline__ df df_div(df a, df b) {
  const float q1 = __fdiv_rn(a.hi, b.hi);
  const df r1 = df_sub(a, df_mul_f(b, q1));
  const float q2 = __fdiv_rn(r1.hi, b.hi);
  const df r2 = df_sub(r1, df_mul_f(b, q2));
  const float q3 = __fdiv_rn(r2.hi, b.hi);
  float s, e;
  fast_two_sum(q1, q2, s, e);
  return df_make(s, e + q3);
}

// sqrt(a) for a >= 0: the correctly rounded float32 root of the hi part and
// one Newton correction from the exact remainder (~2^-46 relative).
__device__ __forceinline__ df df_sqrt(df a) {
  if (!(a.hi > 0.0f)) return df_make(0.0f, 0.0f);
  const float x0 = __fsqrt_rn(a.hi);
  float p, e;
  two_prod(x0, x0, p, e);
  const float r = ((a.hi - p) - e) + a.lo;
  return df_make(x0, __fdiv_rn(r, 2.0f * x0));
}

__device__ __forceinline__ df df_dot3(const df *a, const df *b) {
  return df_add(df_add(df_mul(a[0], b[0]), df_mul(a[1], b[1])),
                df_mul(a[2], b[2]));
}

__host__ __device__ __forceinline__ double df_to_double(df a) {
  return (double)a.hi + (double)a.lo;
}

}  // namespace ss
