// Checks gfx::widen_df (cudagfx_gb300/csrc/gfx_widen.h) on the CPU against FP64:
// normalized double-float pairs from random doubles, pairs with a low part far below
// the FP64 grid of the high part (truncated), ties at half an FP32 ulp, powers of two
// with a negative low part (the binade below) and zeros.  Prints the counts and exits
// non-zero on a result more than one FP64 ulp from hi + lo, or, for a pair a
// round-to-nearest-even two-sum can give, on (float) of the result other than hi.
#include <cmath>
#include <cstdio>
#include <algorithm>
#include <cstdlib>
#include <random>

#include "gfx_widen.h"

int main(int argc, char** argv) {
  const long n_rand = argc > 1 ? std::atol(argv[1]) : 1000000;
  std::mt19937_64 rng(20261204);
  std::uniform_real_distribution<double> u(-1.0, 1.0);
  long n = 0, bad = 0, badf = 0;
  double maxulp = 0.0;
  auto check = [&](float h, float l) {
    const double w = gfx::widen_df(h, l);
    const double ex = (double)h + (double)l;
    const double a = std::fabs(ex);
    const double ulp = a > 0.0 ? std::nextafter(a, INFINITY) - a : 0.0;
    // a subnormal lo (below 2^-126) is dropped
    const double tol = std::fpclassify(l) == FP_SUBNORMAL ? std::max(ulp, (double)std::fabs(l)) : ulp;
    const double e = tol > 0.0 ? std::fabs(w - ex) / tol : (w == ex ? 0.0 : 2.0);
    n++;
    if (e > maxulp) maxulp = e;
    if (e > 1.0) bad++;
    if ((float)ex == h && (float)w != h) badf++;
  };
  for (long i = 0; i < n_rand; i++) {
    const double d = u(rng) * std::ldexp(1.0, (int)(rng() % 40) - 30);
    const float h = (float)d;
    check(h, (float)(d - (double)h));
    const float hp = std::ldexp(1.0f, (int)(rng() % 20) - 10) * ((rng() & 1) ? 1.0f : -1.0f);
    const float ul = std::ldexp(1.0f, std::ilogb(hp) - 23);
    check(hp, -0.5f * ul);
    check(hp, -0.25f * ul);
    check(std::fabs(hp), -0.25f * ul * (float)(0.5 + 0.5 * std::fabs(u(rng))));
    check(hp, 0.5f * ul);
    check(std::nextafter(hp, 0.0f), 0.5f * ul * ((rng() & 1) ? 1.0f : -1.0f));
    const float hr = (float)u(rng);
    const float ur = std::ldexp(1.0f, std::ilogb(hr) - 23);
    check(hr, (float)(u(rng) * 0.5 * ur * std::ldexp(1.0, -(int)(rng() % 45))));
  }
  const float edge[][2] = {{0.0f, 0.0f}, {-0.0f, 0.0f}, {1e-30f, 1e-38f}, {1.0f, 0.0f},
                           {-1.0f, -0.0f}, {1.0f, 1e-45f}, {3e20f, 1e10f}, {-0.5f, 1e-9f},
                           {0.5f, -1e-9f}, {-2.0f, 5e-8f}};
  for (const auto& p : edge) check(p[0], p[1]);
  std::printf("pairs %ld  beyond one ulp %ld  fp32 mismatches %ld  max ulp %.3f\n", n, bad,
              badf, maxulp);
  return bad || badf ? 1 : 0;
}
