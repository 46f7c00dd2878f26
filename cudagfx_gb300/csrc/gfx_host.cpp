// gfx_host.cpp -- host-side generators of libgfx: the glibc rand() stream that seeds
// the twister bank, the reference's Park-Miller SU(3) initializer, Haar-random
// SU(3) for Gribov copies, unit fields, and the status strings.
#include <cmath>
#include <cstdint>
#include <cstring>

#include "../../include/gfx.h"

extern "C" {

int gfx_abi_version(void) { return GFX_ABI_VERSION; }

const char* gfx_status_string(int s) {
  switch (s) {
    case GFX_OK: return "ok";
    case GFX_ERR_BAD_VOLUME: return "lattice extents not supported (all extents must be even)";
    case GFX_ERR_OOM: return "device memory allocation failed";
    case GFX_ERR_NOT_CONVERGED: return "gauge condition not reached within maxit";
    case GFX_ERR_IO: return "i/o error";
    case GFX_ERR_CUDA: return "CUDA error";
    case GFX_ERR_ARG: return "invalid argument";
    case GFX_ERR_STATE: return "call out of order";
    default: return "unknown status";
  }
}

// glibc srandom()/random() with the default TYPE_3 state (31 words, separation 3):
// r[0] = seed; r[i] = 16807 r[i-1] mod (2^31 - 1) (Schrage), then the additive
// feedback r[f] += r[r] over a 31-word ring with 310 outputs discarded; each output
// is (new word) >> 1.  srand/rand are the same stream in glibc.
void gfx_glibc_rand(unsigned int seed, int n, int32_t* out) {
  int32_t ring[31];
  if (seed == 0) seed = 1;
  ring[0] = (int32_t)seed;
  int32_t word = (int32_t)seed;
  for (int i = 1; i < 31; i++) {
    const long hi = word / 127773, lo = word % 127773;
    word = (int32_t)(16807 * lo - 2836 * hi);
    if (word < 0) word += 2147483647;
    ring[i] = word;
  }
  int f = 3, r = 0;
  for (int k = -310; k < n; k++) {
    const uint32_t v = (uint32_t)ring[f] + (uint32_t)ring[r];
    ring[f] = (int32_t)v;
    if (k >= 0) out[k] = (int32_t)(v >> 1);
    f = f == 30 ? 0 : f + 1;
    r = r == 30 ? 0 : r + 1;
  }
}

// Park-Miller Lehmer generator, stream 0 after PlantSeeds (rngs.c:51-98)
namespace {
struct ParkMiller {
  long s;
  double next() {
    const long M = 2147483647L, A = 48271L, Q = M / A, R = M % A;
    const long t = A * (s % Q) - R * (s / Q);
    s = t > 0 ? t : t + M;
    return (double)s / M;
  }
};

inline void su3_row2(double* g) {
  // row 2 = conj(row0 x row1); g is complex[3][3] as 18 doubles
  auto re = [&](int r, int c) { return g[(r * 3 + c) * 2]; };
  auto im = [&](int r, int c) { return g[(r * 3 + c) * 2 + 1]; };
  auto cross = [&](int a, int b, int c, int d, double& xr, double& xi) {
    // (row0[a] row1[b] - row0[c] row1[d])
    xr = (re(0, a) * re(1, b) - im(0, a) * im(1, b)) - (re(0, c) * re(1, d) - im(0, c) * im(1, d));
    xi = (re(0, a) * im(1, b) + im(0, a) * re(1, b)) - (re(0, c) * im(1, d) + im(0, c) * re(1, d));
  };
  double xr, xi;
  cross(1, 2, 2, 1, xr, xi);
  g[12] = xr; g[13] = -xi;
  cross(2, 0, 0, 2, xr, xi);
  g[14] = xr; g[15] = -xi;
  cross(0, 1, 1, 0, xr, xi);
  g[16] = xr; g[17] = -xi;
}

uint64_t splitmix(uint64_t& x) {
  uint64_t z = (x += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
double unit_open(uint64_t& x) {  // (0, 1)
  return ((double)(splitmix(x) >> 11) + 0.5) * (1.0 / 9007199254740992.0);
}
}  // namespace

// random_init_trafo / random_init_gauge (su3manip.c:539-767) after PlantSeeds(seed)
void gfx_random_init_reference(long seed, double* su3, long n) {
  ParkMiller pm;
  pm.s = seed % 2147483647L;
  for (long i = 0; i < n; i++) {
    double* g = su3 + 18 * i;
    for (int r = 0; r < 2; r++) {
      double v[6];
      double h = pm.next(), norm;
      v[0] = h;
      norm = h * h;
      for (int k = 1; k < 5; k++) {
        h = (1.0 - norm) * pm.next();
        v[k] = h;
        norm += h * h;
      }
      v[5] = std::sqrt(1.0 - norm);
      for (int k = 0; k < 6; k++) g[r * 6 + k] = v[k];
    }
    // Gram-Schmidt of row 1 against row 0
    double pr = 0.0, pi = 0.0;
    for (int j = 0; j < 3; j++) {
      const double br = g[6 + 2 * j], bi = g[6 + 2 * j + 1], ar = g[2 * j], ai = -g[2 * j + 1];
      pr += br * ar - bi * ai;
      pi += br * ai + bi * ar;
    }
    for (int j = 0; j < 3; j++) {
      const double ar = g[2 * j], ai = g[2 * j + 1];
      g[6 + 2 * j] -= pr * ar - pi * ai;
      g[6 + 2 * j + 1] -= pr * ai + pi * ar;
    }
    double len = 0.0;
    for (int k = 6; k < 12; k++) len += g[k] * g[k];
    len = 1.0 / std::sqrt(len);
    for (int k = 6; k < 12; k++) g[k] *= len;
    su3_row2(g);
  }
}

// Haar SU(3): complex Gaussian rows 0,1, Gram-Schmidt, row 2 = conj(row0 x row1).
// Stream for matrix i is splitmix64 seeded with (seed, i), so any subset can be
// regenerated independently.
void gfx_random_init_haar(uint64_t seed, double* su3, long n) {
  for (long i = 0; i < n; i++) {
    uint64_t st = seed * 0xD1B54A32D192ED03ull + (uint64_t)i * 0x8CB92BA72F3D8DD7ull;
    double* g = su3 + 18 * i;
    for (int k = 0; k < 12; k += 2) {
      const double u1 = unit_open(st), u2 = unit_open(st);
      const double r = std::sqrt(-2.0 * std::log(u1));
      g[k] = r * std::cos(6.283185307179586 * u2);
      g[k + 1] = r * std::sin(6.283185307179586 * u2);
    }
    double len = 0.0;
    for (int k = 0; k < 6; k++) len += g[k] * g[k];
    len = 1.0 / std::sqrt(len);
    for (int k = 0; k < 6; k++) g[k] *= len;
    double pr = 0.0, pi = 0.0;
    for (int j = 0; j < 3; j++) {
      const double br = g[6 + 2 * j], bi = g[6 + 2 * j + 1], ar = g[2 * j], ai = -g[2 * j + 1];
      pr += br * ar - bi * ai;
      pi += br * ai + bi * ar;
    }
    for (int j = 0; j < 3; j++) {
      const double ar = g[2 * j], ai = g[2 * j + 1];
      g[6 + 2 * j] -= pr * ar - pi * ai;
      g[6 + 2 * j + 1] -= pr * ai + pi * ar;
    }
    len = 0.0;
    for (int k = 6; k < 12; k++) len += g[k] * g[k];
    len = 1.0 / std::sqrt(len);
    for (int k = 6; k < 12; k++) g[k] *= len;
    su3_row2(g);
  }
}

void gfx_unit_init(double* su3, long n) {
  std::memset(su3, 0, sizeof(double) * 18 * (size_t)n);
  for (long i = 0; i < n; i++) {
    su3[18 * i + 0] = 1.0;
    su3[18 * i + 8] = 1.0;
    su3[18 * i + 16] = 1.0;
  }
}

}  // extern "C"
