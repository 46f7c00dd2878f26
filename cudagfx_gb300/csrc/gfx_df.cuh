// gfx_df.cuh -- double-float arithmetic: a value is the unevaluated sum hi + lo of two
// floats with |lo| <= ulp(hi)/2, about 48 significant bits.  GB300 runs FP32 64 times
// faster than FP64, so the FP64-accurate polish sweeps run in this type on the FP32
// units.  The operations are the standard error-free transformations (Dekker 1971,
// Knuth TAOCP vol. 2; as collected by Hida, Li and Bailey, "Library for double-double
// and quad-double arithmetic", 2000), with FMA for the exact product:
//   two_sum(a, b)   = (s, e), s = fl(a + b), a + b = s + e exactly       (6 flops)
//   fast_two_sum    = the same for |a| >= |b|                             (3 flops)
//   two_prod(a, b)  = (p, e), p = fl(a b), e = fma(a, b, -p)              (2 flops)
// Additions and products here are the "sloppy" forms (relative error a few 2^-48),
// which is all the gauge-fixing arithmetic needs; they require IEEE FP32 without
// flush-to-zero, the build default.
#pragma once

#include <cuda_runtime.h>

namespace gfx {

struct dfl {
  float hi, lo;
  dfl() = default;
  __host__ __device__ constexpr dfl(float h, float l) : hi(h), lo(l) {}
  // constants and conversions from double: hi = fl(d), lo = fl(d - hi)
  __host__ __device__ explicit dfl(double d) : hi((float)d), lo((float)(d - (double)(float)d)) {}
  __host__ __device__ explicit dfl(int k) : hi((float)k), lo(0.0f) {}
  __host__ __device__ explicit operator double() const { return (double)hi + (double)lo; }
};

__device__ __forceinline__ dfl fast_two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  return dfl(s, __fsub_rn(b, __fsub_rn(s, a)));
}
__device__ __forceinline__ dfl two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  return dfl(s, __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb)));
}
__device__ __forceinline__ dfl two_prod(float a, float b) {
  const float p = __fmul_rn(a, b);
  return dfl(p, __fmaf_rn(a, b, -p));
}

__device__ __forceinline__ dfl operator+(dfl a, dfl b) {
  dfl s = two_sum(a.hi, b.hi);
  return fast_two_sum(s.hi, __fadd_rn(s.lo, __fadd_rn(a.lo, b.lo)));
}
__device__ __forceinline__ dfl operator-(dfl a) { return dfl(-a.hi, -a.lo); }
__device__ __forceinline__ dfl operator-(dfl a, dfl b) { return a + (-b); }
__device__ __forceinline__ dfl operator*(dfl a, dfl b) {
  dfl p = two_prod(a.hi, b.hi);
  const float e = __fmaf_rn(a.lo, b.hi, __fmaf_rn(a.hi, b.lo, p.lo));
  return fast_two_sum(p.hi, e);
}
__device__ __forceinline__ dfl& operator+=(dfl& a, dfl b) { return a = a + b; }
__device__ __forceinline__ dfl& operator-=(dfl& a, dfl b) { return a = a - b; }
__device__ __forceinline__ dfl& operator*=(dfl& a, dfl b) { return a = a * b; }

// a b + c with one rounding of the low part
__device__ __forceinline__ dfl df_fma(dfl a, dfl b, dfl c) {
  dfl p = two_prod(a.hi, b.hi);
  const float e = __fmaf_rn(a.lo, b.hi, __fmaf_rn(a.hi, b.lo, p.lo));
  dfl s = two_sum(p.hi, c.hi);
  return fast_two_sum(s.hi, __fadd_rn(s.lo, __fadd_rn(e, c.lo)));
}

// 1/sqrt(x): the FP32 estimate refined by one Newton step y (3 - x y^2) / 2 in
// double-float, which doubles its ~23 correct bits
__device__ __forceinline__ dfl df_rsqrt(dfl x) {
  const float y0 = rsqrtf(x.hi);
  const dfl y(y0, 0.0f);
  const dfl r = dfl(1.0f, 0.0f) - x * y * y;  // ~2^-22
  return y + y * dfl(0.5f * r.hi, 0.5f * r.lo);
}

}  // namespace gfx
