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
//   * gaussian fields: Box-Muller on the pairs (2k, 2k+1) of each twister's outputs,
//     applied in the generator before the outputs are stored.
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

// One warp per twister: lane k (< 19) holds word k of the ring.  A round of 19
// outputs updates word k from words k, k+1 and k+9 (mod 19) as they stand at its turn,
// which splits into two dependent steps: words 0..9 read only words not yet updated in
// the round, and words 10..18 read words 0..9 (k+9 mod 19 = k-10, and word 0 for
// k = 18) -- two shuffle steps per round instead of 19 sequential updates.  A block of
// 32 warps (32 twisters) collects kTileRounds rounds of outputs in shared memory and
// writes them row by row, 32 consecutive twisters per row, so the stores stay
// coalesced; the Box-Muller pairs (2k, 2k+1) of each twister are formed there.
constexpr int kTwistersPerBlock = 32;
constexpr int kTileRounds = 8;                     // even: pairs never straddle a tile
constexpr int kTileRows = kTileRounds * kMTN;      // 152 outputs per twister and tile

__device__ __forceinline__ uint32_t mt_step(uint32_t mti, uint32_t mti1, uint32_t mtm, uint32_t A) {
  const uint32_t x = (mti & kUMask) | (mti1 & kLMask);
  return mtm ^ (x >> 1) ^ ((x & 1u) ? A : 0u);
}

__device__ __forceinline__ float mt_temper(uint32_t x, uint32_t B, uint32_t C) {
  x ^= (x >> 12);
  x ^= (x << 7) & B;
  x ^= (x << 15) & C;
  x ^= (x >> 18);
  return ((float)x + 1.0f) * kInv2p32;
}

template <bool GAUSS>
__global__ void __launch_bounds__(kTwistersPerBlock * 32) mt_generate_kernel(MTBank bank,
                                                                             float* __restrict__ out,
                                                                             int nper,
                                                                             int initialized) {
  __shared__ float tile[kTileRows][kTwistersPerBlock + 1];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int r0 = blockIdx.x * kTwistersPerBlock;
  const int r = r0 + w;  // this warp's twister (the grid covers exactly kMTCount)
  uint32_t mt = 0;
  if (!initialized) {
    uint32_t v = bank.seed[r];
    for (int k = 1; k <= lane && k < kMTN; k++) v = 1812433253u * (v ^ (v >> 30)) + (uint32_t)k;
    mt = v;
  } else if (lane < kMTN) {
    mt = bank.status[lane * kMTCount + r];
  }
  const uint32_t A = bank.a[r], B = bank.b[r], C = bank.c[r];
  const int src1a = lane + 1 < 32 ? lane + 1 : lane, src9a = lane + 9 < 32 ? lane + 9 : lane;
  const int src1b = lane == kMTN - 1 ? 0 : src1a, src9b = lane >= 10 ? lane - 10 : lane;
  for (int o = 0; o < nper; o += kTileRows) {
    const int cnt = min(kTileRows, nper - o);
    for (int k0 = 0; k0 < cnt; k0 += kMTN) {
      const int rem = min(kMTN, cnt - k0);
      // words 0..9 from the round's old words
      uint32_t n1 = __shfl_sync(0xffffffffu, mt, src1a);
      uint32_t n9 = __shfl_sync(0xffffffffu, mt, src9a);
      if (lane < 10 && lane < rem) mt = mt_step(mt, n1, n9, A);
      // words 10..18 from old word k+1 (new word 0 for k = 18) and new word k-10
      n1 = __shfl_sync(0xffffffffu, mt, src1b);
      n9 = __shfl_sync(0xffffffffu, mt, src9b);
      if (lane >= 10 && lane < kMTN && lane < rem) mt = mt_step(mt, n1, n9, A);
      if (lane < rem) tile[k0 + lane][w] = mt_temper(mt, B, C);
    }
    __syncthreads();
    // rows j of the tile -> out[(o + j) * kMTCount + r0 + col]
    const int col = threadIdx.x & (kTwistersPerBlock - 1);
    if (GAUSS) {
      // an unpaired last output (odd nper) is not written, as in the sequential form
      for (int pr = threadIdx.x / kTwistersPerBlock; 2 * pr + 1 < cnt;
           pr += blockDim.x / kTwistersPerBlock) {
        float g1, g2;
        box_muller(tile[2 * pr][col], tile[2 * pr + 1][col], g1, g2);
        out[(size_t)(o + 2 * pr) * kMTCount + r0 + col] = g1;
        out[(size_t)(o + 2 * pr + 1) * kMTCount + r0 + col] = g2;
      }
    } else {
      for (int row = threadIdx.x / kTwistersPerBlock; row < cnt;
           row += blockDim.x / kTwistersPerBlock)
        out[(size_t)(o + row) * kMTCount + r0 + col] = tile[row][col];
    }
    __syncthreads();
  }
  if (lane < kMTN) bank.status[lane * kMTCount + r] = mt;
  if (lane == 0) bank.seed[r] = mt;
}

void launch_mt_generate(const MTBank& bank, float* out, int nper, int initialized, int gauss,
                        cudaStream_t s) {
  const int grid = kMTCount / kTwistersPerBlock, block = kTwistersPerBlock * 32;
  if (gauss)
    mt_generate_kernel<true><<<grid, block, 0, s>>>(bank, out, nper, initialized);
  else
    mt_generate_kernel<false><<<grid, block, 0, s>>>(bank, out, nper, initialized);
}

}  // namespace gfx
