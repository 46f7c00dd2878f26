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
// fields are kept in a pair layout (P12 below) so that the packed operands come
// straight from 16-byte loads, with no register moves to pair them up.
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

// The pair layout of an FP32 12-real field: plane e (e = 0..5, the complex entries of
// rows 0 and 1) holds, per site, the float4 {re of lane x, re of lane y, im of lane x,
// im of lane y}.  One 16-byte load then fills cplx<f2> in register pairs as the packed
// instructions take them.  A pair of gauge copies stores its two g this way (6 planes
// per parity); a link field shared by both copies stores each link in both lanes.
struct P12 {
  float4* p;
  __device__ __forceinline__ P12 operator+(size_t off) const {
    P12 r;
    r.p = p + off;
    return r;
  }
};
constexpr int kPairPlanes = 6;

// rows 0,1 of the pair at site i (planes spaced by stride)
__device__ __forceinline__ void load12_rows01(const P12& base, size_t stride, int i,
                                              Mat3<f2>& m) {
#pragma unroll
  for (int e = 0; e < 6; e++) {
    const float4 v = __ldg(base.p + e * stride + i);
    m.e[e / 3][e % 3].re = f2(v.x, v.y);
    m.e[e / 3][e % 3].im = f2(v.z, v.w);
  }
}

// the pair at site i, row 2 rebuilt as conj(row0 x row1) (lane for lane as unpack12)
__device__ __forceinline__ void load12(const P12& base, size_t stride, int i, Mat3<f2>& m) {
  load12_rows01(base, stride, i, m);
  row2_from_01(m);
}

// rows 0,1 of the pair at site i; with keep_x / keep_y a lane keeps `old` (its copy has
// stopped: its stored bits are written back unchanged)
__device__ __forceinline__ void store12(const P12& base, size_t stride, int i, const Mat3<f2>& m,
                                        const Mat3<f2>& old, bool keep_x, bool keep_y) {
#pragma unroll
  for (int e = 0; e < 6; e++) {
    const cplx<f2> a = m.e[e / 3][e % 3], o = old.e[e / 3][e % 3];
    base.p[e * stride + i] = make_float4(keep_x ? o.re.v.x : a.re.v.x, keep_y ? o.re.v.y : a.re.v.y,
                                         keep_x ? o.im.v.x : a.im.v.x, keep_y ? o.im.v.y : a.im.v.y);
  }
}

// one lane of a pair field read as a scalar FP32 matrix (the per-copy measurement)
struct LaneP12 {
  const float4* p;
  int lane;
  __device__ __forceinline__ LaneP12 operator+(size_t off) const {
    LaneP12 r;
    r.p = p + off;
    r.lane = lane;
    return r;
  }
};
__device__ __forceinline__ void load12_rows01(const LaneP12& base, size_t stride, int i,
                                              Mat3<float>& m) {
#pragma unroll
  for (int e = 0; e < 6; e++) {
    const float4 v = __ldg(base.p + e * stride + i);
    m.e[e / 3][e % 3] = base.lane ? cmk(v.y, v.w) : cmk(v.x, v.z);
  }
}

}  // namespace gfx
