// gfx_mt.cu -- bank of 4096 MT607 Mersenne Twisters (w = 32, n = 19, m = 9, r = 1,
// tempering shifts 12/7/15/18), restated from the published Mersenne Twister
// recurrence (Matsumoto & Nishimura 1998) with per-generator parameters
// (matrix_a, mask_b, mask_c) read from the twister-parameter file.
//
// Call semantics reproduce the reference bank (MersenneTwister.cu:142-229,
// 236-323) bit for bit:
//   * output j of twister r goes to out[r + 4096*j], as ((float)x + 1) / 2^32;
//   * every call restarts at ring slot 0 of the saved 19-word state, and saves
//     the state and seed = state[0] at the end;
//   * initialized == 0 re-seeds the state from seed with the MT init recurrence;
//   * gaussian fields: Box-Muller on the pairs (2k, 2k+1) of each twister's lane,
//     fused into the generator.
// This translation unit is compiled with -prec-sqrt=false -prec-div=false,
// the flags of the reference build, so the Box-Muller arithmetic matches it.
#include "gfx_internal.h"

namespace gfx {

namespace {
constexpr uint32_t kUMask = 0xFFFFFFFEu;
constexpr uint32_t kLMask = 0x1u;
constexpr float kInv2p32 = 2.3283064365386963e-10f;  // 2^-32, exact
}  // namespace

__device__ __forceinline__ void box_muller(float u1, float u2, float& g1, float& g2) {
  const float PIf = 3.14159265358979f;
  const float r = sqrtf(-2.0f * logf(u1));
  const float phi = 2 * PIf * u2;
  g1 = r * __cosf(phi);
  g2 = r * __sinf(phi);
}

template <bool GAUSS>
__global__ void __launch_bounds__(128) mt_generate_kernel(MTBank bank, float* __restrict__ out,
                                                          int nper, int initialized) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= kMTCount) return;
  uint32_t mt[kMTN];
  if (!initialized) {
    mt[0] = bank.seed[r];
#pragma unroll
    for (int k = 1; k < kMTN; k++) mt[k] = 1812433253u * (mt[k - 1] ^ (mt[k - 1] >> 30)) + (uint32_t)k;
  } else {
#pragma unroll
    for (int k = 0; k < kMTN; k++) mt[k] = bank.status[k * kMTCount + r];
  }
  const uint32_t A = bank.a[r], B = bank.b[r], C = bank.c[r];
  uint32_t mti1 = mt[0];
  float pending = 0.0f;

  auto emit = [&](int j, uint32_t x) {
    x ^= (x >> 12);
    x ^= (x << 7) & B;
    x ^= (x << 15) & C;
    x ^= (x >> 18);
    const float u = ((float)x + 1.0f) * kInv2p32;
    if (GAUSS) {
      if ((j & 1) == 0) {
        pending = u;
      } else {
        float g1, g2;
        box_muller(pending, u, g1, g2);
        out[r + (size_t)(j - 1) * kMTCount] = g1;
        out[r + (size_t)j * kMTCount] = g2;
      }
    } else {
      out[r + (size_t)j * kMTCount] = u;
    }
  };

  int o = 0;
  // full rounds of the 19-word ring with static slot indices (registers only)
  for (; o + kMTN <= nper; o += kMTN) {
#pragma unroll
    for (int k = 0; k < kMTN; k++) {
      const int k1 = (k + 1) % kMTN, kM = (k + 9) % kMTN;
      const uint32_t mti = mti1;
      mti1 = mt[k1];
      uint32_t x = (mti & kUMask) | (mti1 & kLMask);
      x = mt[kM] ^ (x >> 1) ^ ((x & 1u) ? A : 0u);
      mt[k] = x;
      emit(o + k, x);
    }
  }
#pragma unroll
  for (int k = 0; k < kMTN; k++) {
    if (o + k < nper) {
      const int k1 = (k + 1) % kMTN, kM = (k + 9) % kMTN;
      const uint32_t mti = mti1;
      mti1 = mt[k1];
      uint32_t x = (mti & kUMask) | (mti1 & kLMask);
      x = mt[kM] ^ (x >> 1) ^ ((x & 1u) ? A : 0u);
      mt[k] = x;
      emit(o + k, x);
    }
  }
  bank.seed[r] = mt[0];
#pragma unroll
  for (int k = 0; k < kMTN; k++) bank.status[k * kMTCount + r] = mt[k];
}

void launch_mt_generate(const MTBank& bank, float* out, int nper, int initialized, int gauss,
                        cudaStream_t s) {
  if (gauss)
    mt_generate_kernel<true><<<kMTCount / 128, 128, 0, s>>>(bank, out, nper, initialized);
  else
    mt_generate_kernel<false><<<kMTCount / 128, 128, 0, s>>>(bank, out, nper, initialized);
}

}  // namespace gfx
