// Double-float arithmetic: a value is the unevaluated sum hi + lo of two FP32 numbers
// (about 48 significant bits), built from FP32 FMAs with the error-free transformations of
// Dekker and Knuth (two-product by FMA, two-sum; the "sloppy" addition of the double-double
// literature).  On a GPU whose FP64 rate is a small fraction of its FP32 rate, the FP64-bound
// residual kernel runs on the FP32 pipe this way at a few FP32 operations per FP64 operation.
#pragma once

#include <cuda_runtime.h>

namespace glgpu
{
struct DF
{
  float h, l;
  __device__ __forceinline__ DF() : h(0.f), l(0.f) {}
  __device__ __forceinline__ explicit DF(float a) : h(a), l(0.f) {}
  __device__ __forceinline__ DF(float a, float b) : h(a), l(b) {}
};

__device__ __forceinline__ DF df_quick(float s, float e) // |s| >= |e|
{
  const float h = s + e;
  return DF(h, e - (h - s));
}
__device__ __forceinline__ DF operator+(DF a, DF b)
{
  const float s = a.h + b.h, bb = s - a.h;
  const float e = (a.h - (s - bb)) + (b.h - bb) + (a.l + b.l);
  return df_quick(s, e);
}
__device__ __forceinline__ DF operator-(DF a) { return DF(-a.h, -a.l); }
__device__ __forceinline__ DF operator-(DF a, DF b) { return a + (-b); }
__device__ __forceinline__ DF operator*(DF a, DF b)
{
  const float p = a.h * b.h;
  float e = fmaf(a.h, b.h, -p);
  e = fmaf(a.h, b.l, fmaf(a.l, b.h, e));
  return df_quick(p, e);
}
__device__ __forceinline__ DF &operator+=(DF &a, DF b) { return a = a + b; }
__device__ __forceinline__ DF &operator-=(DF &a, DF b) { return a = a - b; }

// conversions (one FP64 subtraction each way)
template <typename R> __device__ __forceinline__ R from_d(double v);
template <> __device__ __forceinline__ double from_d<double>(double v) { return v; }
template <> __device__ __forceinline__ DF from_d<DF>(double v)
{
  const float h = __double2float_rn(v);
  return DF(h, __double2float_rn(v - static_cast<double>(h)));
}
__device__ __forceinline__ double to_d(double v) { return v; }
__device__ __forceinline__ double to_d(DF v) { return static_cast<double>(v.h) + static_cast<double>(v.l); }
} // namespace glgpu
