// Checks gfx::narrow_df (cudagfx_gb300/csrc/gfx_narrow.h) on the CPU: for random doubles
// across the FP32 range, ties at half an FP32 ulp, binade edges, zeros and the
// fallback range, hi and lo must equal (float)d and (float)(d - (double)hi) bit for
// bit.  Prints the counts and exits non-zero on any difference.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <random>

#include "gfx_narrow.h"

static unsigned bits(float x) {
  unsigned u;
  std::memcpy(&u, &x, 4);
  return u;
}

int main(int argc, char** argv) {
  const long n_rand = argc > 1 ? std::atol(argv[1]) : 1000000;
  std::mt19937_64 rng(20261204);
  std::uniform_real_distribution<double> u(-1.0, 1.0);
  long n = 0, bad = 0;
  auto check = [&](double d) {
    float h, l;
    gfx::narrow_df(d, h, l);
    const float h0 = (float)d;
    const float l0 = (float)(d - (double)h0);
    n++;
    if (bits(h) != bits(h0) || bits(l) != bits(l0)) {
      if (bad < 5) std::printf("mismatch d=%.17g: %a %a vs %a %a\n", d, h, l, h0, l0);
      bad++;
    }
  };
  for (long i = 0; i < n_rand; i++) {
    check(u(rng) * std::ldexp(1.0, (int)(rng() % 200) - 100));
    // FP32 values plus half an ulp (ties), and just off the tie
    const float f = (float)(u(rng) * std::ldexp(1.0, (int)(rng() % 60) - 30));
    const double ulp = std::ldexp(1.0, std::ilogb(f) - 23);
    check((double)f + 0.5 * ulp);
    check((double)f - 0.5 * ulp);
    check((double)f + 0.5 * ulp * (1.0 + 1e-12));
    // just below a power of two (carry into the next binade)
    const double p2 = std::ldexp(1.0, (int)(rng() % 60) - 30);
    check(p2 - std::ldexp(p2, -26) * u(rng) * 0.5);
  }
  const double edge[] = {0.0, -0.0, 1.0, -1.0, 1e-30, 3e-23, 6e-23, 1e38, 3.4e38, 1e-300,
                         std::ldexp(1.0, -74), std::ldexp(1.0, -75), std::ldexp(1.0, 126),
                         std::ldexp(1.0, 127) * 1.9, INFINITY, -INFINITY, NAN};
  for (double d : edge) check(d);
  std::printf("values %ld  mismatches %ld\n", n, bad);
  return bad ? 1 : 0;
}
