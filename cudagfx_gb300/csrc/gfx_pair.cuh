// gfx_pair.cuh -- two gauge copies in one thread with Blackwell's packed FP32 arithmetic.
//
// f2 holds one FP32 value of each of two Gribov copies of the same configuration
// (lane x: the first copy, lane y: the second).  Its operators map to the sm_100+
// packed instructions (__ffma2_rn, __fadd2_rn, __fmul2_rn): one instruction does the
// operation of both copies, with each lane rounded exactly as the scalar FP32
// operation (__fmaf_rn, __fadd_rn, __fmul_rn).  The templated SU(3) code of
// gfx_device.cuh and gfx_common.cuh instantiated with T = f2 therefore gives, lane
// for lane, the bits of the scalar FP32 kernels (the scalar code uses no contracted
// a*b+c: every FMA is an explicit fm()), at about half the instruction issue.  The
// links, shared by both copies, are loaded once and broadcast to both lanes.
#pragma once

#include <cuda_runtime.h>

#include "gfx_device.cuh"

namespace gfx {

struct f2 {
  float2 v;
  __device__ __forceinline__ f2() {}
  __device__ __forceinline__ explicit f2(float a) : v(make_float2(a, a)) {}
  __device__ __forceinline__ f2(float a, float b) : v(make_float2(a, b)) {}
  __device__ __forceinline__ explicit f2(double a) : v(make_float2((float)a, (float)a)) {}
  __device__ __forceinline__ explicit f2(int a) : v(make_float2((float)a, (float)a)) {}
};

__device__ __forceinline__ f2 mkf2(float2 v) {
  f2 r;
  r.v = v;
  return r;
}
__device__ __forceinline__ f2 operator+(f2 a, f2 b) { return mkf2(__fadd2_rn(a.v, b.v)); }
__device__ __forceinline__ f2 operator-(f2 a) { return f2(-a.v.x, -a.v.y); }
// a - b = a + (-b) exactly (IEEE subtraction is addition of the negated operand)
__device__ __forceinline__ f2 operator-(f2 a, f2 b) { return a + (-b); }
__device__ __forceinline__ f2 operator*(f2 a, f2 b) { return mkf2(__fmul2_rn(a.v, b.v)); }
__device__ __forceinline__ f2& operator+=(f2& a, f2 b) { return a = a + b; }
__device__ __forceinline__ f2& operator-=(f2& a, f2 b) { return a = a - b; }
__device__ __forceinline__ f2& operator*=(f2& a, f2 b) { return a = a * b; }

template <>
__device__ __forceinline__ f2 fm<f2>(f2 a, f2 b, f2 c) {
  return mkf2(__ffma2_rn(a.v, b.v, c.v));
}
template <>
__device__ __forceinline__ f2 rsqrt_t<f2>(f2 x) {
  return f2(rsqrtf(x.v.x), rsqrtf(x.v.y));
}

// a pair of gauge-transformation fields: the two copies' FP32 12-real fields
struct GPairPtr {
  const float4* a;
  const float4* b;
  __device__ __forceinline__ GPairPtr operator+(size_t off) const {
    GPairPtr r;
    r.a = a + off;
    r.b = b + off;
    return r;
  }
};

__device__ __forceinline__ cplx<f2> cpair(float ar, float ai, float br, float bi) {
  cplx<f2> z;
  z.re = f2(ar, br);
  z.im = f2(ai, bi);
  return z;
}

// rows 0,1 of both copies' g at site i (planes spaced by stride)
__device__ __forceinline__ void load12_rows01(const GPairPtr& base, size_t stride, int i,
                                              Mat3<f2>& m) {
  const float4 a0 = __ldg(base.a + i), a1 = __ldg(base.a + stride + i),
               a2 = __ldg(base.a + 2 * stride + i);
  const float4 b0 = __ldg(base.b + i), b1 = __ldg(base.b + stride + i),
               b2 = __ldg(base.b + 2 * stride + i);
  m.e[0][0] = cpair(a0.x, a0.y, b0.x, b0.y);
  m.e[0][1] = cpair(a0.z, a0.w, b0.z, b0.w);
  m.e[0][2] = cpair(a1.x, a1.y, b1.x, b1.y);
  m.e[1][0] = cpair(a1.z, a1.w, b1.z, b1.w);
  m.e[1][1] = cpair(a2.x, a2.y, b2.x, b2.y);
  m.e[1][2] = cpair(a2.z, a2.w, b2.z, b2.w);
}

// both copies' g at site i, row 2 rebuilt as conj(row0 x row1) (per lane as unpack12)
__device__ __forceinline__ void load12(const GPairPtr& base, size_t stride, int i, Mat3<f2>& m) {
  load12_rows01(base, stride, i, m);
  row2_from_01(m);
}

// a link shared by both copies, broadcast to both lanes
__device__ __forceinline__ void broadcast(const Mat3<float>& s, Mat3<f2>& m, int rows) {
#pragma unroll
  for (int r = 0; r < 3; r++) {
    if (r >= rows) break;
#pragma unroll
    for (int c = 0; c < 3; c++) {
      m.e[r][c].re = f2(s.e[r][c].re);
      m.e[r][c].im = f2(s.e[r][c].im);
    }
  }
}

// rows 0,1 of both copies' new g, lane x to field a and lane y to field b
__device__ __forceinline__ void store12(float4* a, float4* b, size_t stride, int i,
                                        const Mat3<f2>& m) {
  a[i] = make_float4(m.e[0][0].re.v.x, m.e[0][0].im.v.x, m.e[0][1].re.v.x, m.e[0][1].im.v.x);
  a[stride + i] =
      make_float4(m.e[0][2].re.v.x, m.e[0][2].im.v.x, m.e[1][0].re.v.x, m.e[1][0].im.v.x);
  a[2 * stride + i] =
      make_float4(m.e[1][1].re.v.x, m.e[1][1].im.v.x, m.e[1][2].re.v.x, m.e[1][2].im.v.x);
  b[i] = make_float4(m.e[0][0].re.v.y, m.e[0][0].im.v.y, m.e[0][1].re.v.y, m.e[0][1].im.v.y);
  b[stride + i] =
      make_float4(m.e[0][2].re.v.y, m.e[0][2].im.v.y, m.e[1][0].re.v.y, m.e[1][0].im.v.y);
  b[2 * stride + i] =
      make_float4(m.e[1][1].re.v.y, m.e[1][1].im.v.y, m.e[1][2].re.v.y, m.e[1][2].im.v.y);
}

}  // namespace gfx
