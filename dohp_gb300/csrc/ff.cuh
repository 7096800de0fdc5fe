// Float-float ("double-float") numbers for the FP64-class apply on the FP32 pipe.
//
// A value is hi + lo with two FP32 words. Products use the exact FMA residual (p = a.hi b.hi, e = fma(a.hi,
// b.hi, -p)), sums the branch-free two-sum (Knuth, The Art of Computer Programming vol. 2, 4.2.2; Dekker 1971);
// the cross term a.lo b.lo is dropped. Unit roundoff about 2^-48 (FP64: 2^-53), FP32 exponent range. On GB300
// the FP32 pipe issues ~64x more operations per clock than the FP64 pipe, so ~10 FP32 operations per
// multiply-add still leave the arithmetic several times faster than native FP64.
//
// fma_acc accumulates a dot product without renormalizing the accumulator after every term (10 operations per
// term); fin renormalizes once when a result is stored.
#pragma once

#include <cuda_runtime.h>

namespace dgb {

struct ff {
  float hi, lo;
  ff() = default;
  __host__ __device__ ff(float h, float l) : hi(h), lo(l) {}
  __host__ __device__ ff(double d) : hi((float)d), lo((float)(d - (double)(float)d)) {}
  __host__ __device__ ff(float f) : hi(f), lo(0.0f) {}
  __host__ __device__ ff(int i) : ff((double)i) {}
  __host__ __device__ explicit operator double() const { return (double)hi + (double)lo; }
};

__device__ __forceinline__ ff ff_quick(float s, float e) {  // |s| >= |e|
  const float h = s + e;
  return ff(h, e - (h - s));
}

__device__ __forceinline__ ff operator+(ff a, ff b) {
  const float s = a.hi + b.hi, bb = s - a.hi;
  float e = (a.hi - (s - bb)) + (b.hi - bb);
  e += a.lo + b.lo;
  return ff_quick(s, e);
}
__device__ __forceinline__ ff operator-(ff a) { return ff(-a.hi, -a.lo); }
__device__ __forceinline__ ff operator-(ff a, ff b) { return a + (-b); }
__device__ __forceinline__ ff operator*(ff a, ff b) {
  const float p = a.hi * b.hi;
  float e = fmaf(a.hi, b.hi, -p);
  e = fmaf(a.hi, b.lo, fmaf(a.lo, b.hi, e));
  return ff_quick(p, e);
}
__device__ __forceinline__ ff &operator+=(ff &a, ff b) { return a = a + b; }
__device__ __forceinline__ ff &operator*=(ff &a, ff b) { return a = a * b; }

// s += a b, accumulator left unnormalized
__device__ __forceinline__ void fma_acc(ff &s, ff a, ff b) {
  const float p = a.hi * b.hi;
  float e = fmaf(a.hi, b.hi, -p);
  e = fmaf(a.hi, b.lo, fmaf(a.lo, b.hi, e));
  const float t = s.hi + p, bb = t - s.hi;
  const float err = (s.hi - (t - bb)) + (p - bb);
  s.hi = t;
  s.lo += err + e;
}
__device__ __forceinline__ ff fin(ff s) { return ff_quick(s.hi, s.lo); }

// the same helpers for the native types: exactly the expressions the kernels used before
template <typename T>
__device__ __forceinline__ void fma_acc(T &s, T a, T b) {
  s += a * b;
}
template <typename T>
__device__ __forceinline__ T fin(T s) {
  return s;
}
// s += a0 b0 + a1 b1 + a2 b2
template <typename T>
__device__ __forceinline__ void dot3_acc(T &s, T a0, T b0, T a1, T b1, T a2, T b2) {
  s += a0 * b0 + a1 * b1 + a2 * b2;
}
__device__ __forceinline__ void dot3_acc(ff &s, ff a0, ff b0, ff a1, ff b1, ff a2, ff b2) {
  fma_acc(s, a0, b0);
  fma_acc(s, a1, b1);
  fma_acc(s, a2, b2);
}

}  // namespace dgb
