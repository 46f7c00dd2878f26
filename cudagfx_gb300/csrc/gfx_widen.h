// gfx_widen.h -- a double-float value hi + lo widened to FP64 with integer operations.
//
// GB300 runs FP64 (and the FP32<->FP64 conversions) at 1/64 of its FP32 rate.  The FP32
// thermalization reunitarizes each new link in double-float and stores it in FP64 and
// FP32; (double)hi + (double)lo and (float) of that took two conversions, an FP64 add
// and a conversion back per real, about 40% of that kernel's cycles on the FP64 pipe.
// Here hi's bits are rebiased into an FP64 pattern and lo is added to it as an integer
// count of FP64 ulps:
//
//   hi = (1 + m/2^23) 2^Eh   ->   FP64 pattern: sign, exponent Eh, mantissa m 2^29
//   lo = Ml 2^(El-23)        ->   Ml 2^(El-Eh+29) ulps of 2^(Eh-52), truncated
//
// For a normalized pair (|lo| <= ulp(hi)/2, as every double-float operation leaves it)
// the count is below 2^29 and the mantissa m 2^29 is at most 2^52 - 2^29, so the add
// never carries into the exponent.  It borrows from it only when hi is a power of two
// and lo is negative; then the result lies in the binade below, where an ulp is
// 2^(Eh-53), and lo is counted in those units.  The result is within one FP64 ulp of
// the exact hi + lo (exactly it, unless lo has bits below 2^(Eh-53)); the double-float
// value itself is only good to ~2^-48.
//
// The nearest FP32 to the result is hi itself: a pair out of a round-to-nearest-even
// two-sum has |lo| < ulp(hi)/2, or = ulp(hi)/2 with hi's last bit even, and the
// truncation happens only for lo far below that tie.
//
// A zero or subnormal hi gives a signed zero (the pair is then below 2^-126 in size),
// an infinite or NaN hi a NaN.  Plain C++ with a host twin, so the same code is
// checked on the CPU.
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

__host__ __device__ inline uint32_t widen_bits_f(float x) {
#ifdef __CUDA_ARCH__
  return __float_as_uint(x);
#else
  uint32_t u;
  std::memcpy(&u, &x, 4);
  return u;
#endif
}
__host__ __device__ inline double widen_double(uint64_t u) {
#ifdef __CUDA_ARCH__
  return __longlong_as_double((long long)u);
#else
  double x;
  std::memcpy(&x, &u, 8);
  return x;
#endif
}

__host__ __device__ inline double widen_df(float hi, float lo) {
  const uint32_t hb = widen_bits_f(hi), lb = widen_bits_f(lo);
  const uint32_t sign = hb & 0x80000000u;
  const int eh = (int)((hb >> 23) & 0xffu), el = (int)((lb >> 23) & 0xffu);
  const bool opp = ((hb ^ lb) & 0x80000000u) != 0u && (lb & 0x7fffffffu) != 0u;
  const int down = ((hb & 0x7fffffu) == 0u && opp) ? 1 : 0;
  int k = el - eh + 29 + down;  // lo's significand shift onto the ulp grid
  k = k > 7 ? 7 : k;
  const uint32_t ml = el != 0 ? ((lb & 0x7fffffu) | 0x800000u) : 0u;
  const uint32_t lu = k >= 0 ? ml << k : ml >> (k < -31 ? 31 : -k);
  const uint32_t whi = ((((hb & 0x7fffffffu) >> 3) + 0x38000000u) | sign);
  uint64_t pat = ((uint64_t)whi << 32) | (uint64_t)(hb << 29);
  pat = opp ? pat - lu : pat + lu;
  if (eh == 0) pat = (uint64_t)sign << 32;
  if (eh == 255) pat = 0x7ff8000000000000ull;
  return widen_double(pat);
}

}  // namespace gfx
