// gfx_narrow.h -- an FP64 value split into a double-float pair hi + lo with integer
// operations only: hi = (float)d and lo = (float)(d - (double)hi), bit for bit.
//
// GB300 runs FP64 and the FP64<->FP32 conversions at 1/64 of its FP32 rate.  The
// rebased polish builds its base from the FP64 links and g; narrowing each real with
// two conversions and an FP64 subtraction kept those kernels on the FP64 pipe.  Here
//
//   d = (-1)^s M 2^(E-52),  M = 2^52 + mantissa (53 bits)
//   hi: M rounded to its top 24 bits, ties to even (a carry out of the top bit
//       moves hi to the next binade), rebiased to FP32
//   lo: d - hi = (-1)^s (M mod 2^29 - 2^29 [if rounded up]) 2^(E-52), an integer of
//       at most 29 bits times a power of two, converted to FP32 by one int-to-float
//       conversion (round to nearest even, as cvt.rn.f32.f64 of the exact difference)
//       and an exact power-of-two scaling
//
// Zeros and values whose hi or lo could leave the FP32 normal range (|d| outside
// [2^-74, 2^127)) take the FP64-conversion route, which gives the same results.  Plain
// C++ with a host twin, so the bit-for-bit agreement is checked on the CPU.
#pragma once

#include <cstdint>
#include <cstring>

#ifndef __CUDACC__
#ifndef __host__
#define __host__
#endif
#ifndef __device__
#define __device__
#endif
#endif

namespace gfx {

__host__ __device__ inline uint64_t narrow_bits_d(double x) {
#ifdef __CUDA_ARCH__
  return (uint64_t)__double_as_longlong(x);
#else
  uint64_t u;
  std::memcpy(&u, &x, 8);
  return u;
#endif
}
__host__ __device__ inline float narrow_float(uint32_t u) {
#ifdef __CUDA_ARCH__
  return __uint_as_float(u);
#else
  float x;
  std::memcpy(&x, &u, 4);
  return x;
#endif
}
__host__ __device__ inline float narrow_i2f(int v) {
#ifdef __CUDA_ARCH__
  return __int2float_rn(v);
#else
  return (float)v;  // round to nearest even under the default floating-point environment
#endif
}

__host__ __device__ inline void narrow_df(double d, float& hi, float& lo) {
  const uint64_t b = narrow_bits_d(d);
  const int e = (int)((b >> 52) & 0x7ff) - 1023;
  if (e < -74 || e > 126) {  // zero, tiny, huge or non-finite: the conversions
    hi = (float)d;
    lo = (float)(d - (double)hi);
    return;
  }
  const uint32_t sign = (uint32_t)(b >> 32) & 0x80000000u;
  const uint64_t m = (b & ((1ull << 52) - 1)) | (1ull << 52);
  uint32_t top = (uint32_t)(m >> 29);                 // 24 bits
  const int rem = (int)(m & ((1u << 29) - 1));        // 29 bits
  int eh = e;
  int low = rem;
  if (rem > (1 << 28) || (rem == (1 << 28) && (top & 1u))) {
    low = rem - (1 << 29);
    if (++top == (1u << 24)) {
      top = 1u << 23;
      eh++;
    }
  }
  hi = narrow_float(sign | ((uint32_t)(eh + 127) << 23) | (top & 0x7fffffu));
  // lo = low 2^(e-52), |low| < 2^29; 2^(e-52) is an FP32 normal for e >= -74
  const float scale = narrow_float((uint32_t)(e - 52 + 127) << 23);
  lo = narrow_i2f(sign ? -low : low) * scale;  // a zero difference is +0, as d - hi
}

}  // namespace gfx
