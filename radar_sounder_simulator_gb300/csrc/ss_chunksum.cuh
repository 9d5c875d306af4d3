// Sum of one output bin's chunk partials, in chunk order.
//
// Float partials (split forms, incoherent power): a float32 two-sum per
// partial with the rounding errors carried alongside -- ~2^-48 relative,
// the float64 sum's value without FP64-pipe additions, which GB300 runs at
// ~1/75 of its FP32 rate. Double partials (FP64 forms): float64 additions,
// as the reference sums.
#pragma once

#include "ss_df.cuh"

namespace ss {

template <typename P>
struct ChunkSum;

template <>
struct ChunkSum<float> {
  float h = 0.0f, l = 0.0f;
  __device__ __forceinline__ void add(float v) {
    float s, e;
    two_sum(h, v, s, e);
    h = s;
    l += e;
  }
  __device__ __forceinline__ double value() const {
    return (double)h + (double)l;
  }
};

template <>
struct ChunkSum<float2> {
  ChunkSum<float> r, i;
  __device__ __forceinline__ void add(float2 v) {
    r.add(v.x);
    i.add(v.y);
  }
  __device__ __forceinline__ double re() const { return r.value(); }
  __device__ __forceinline__ double im() const { return i.value(); }
};

template <>
struct ChunkSum<double2> {
  double r = 0.0, i = 0.0;
  __device__ __forceinline__ void add(double2 v) {
    r += v.x;
    i += v.y;
  }
  __device__ __forceinline__ double re() const { return r; }
  __device__ __forceinline__ double im() const { return i; }
};

}  // namespace ss
