// gfx_heatbath.cu -- stochastic updates for sm_103a:
//   * simulated-annealing heatbath of the gauge transformation g
//     (simulated_annealing.cu:5-257),
//   * microcanonical (SU(2)-reflection) sweep of g,
//   * Cabibbo-Marinari heatbath of the links for thermalization
//     (heatbath_thermalization.cu:235-550), storing the result at link (x, nu).
// Random numbers are read from the Mersenne-Twister fields with the reference's
// indexing: gauss[k], unif[4k..4k+3] with k = eo index (SA) or 4*eo + nu (links).
#include "gfx_common.cuh"
#include "gfx_internal.h"
#include "gfx_widen.h"

namespace gfx {

// dev_get_a0 (simulated_annealing.cu:5-27): one single-precision trial
__device__ __forceinline__ int get_a0(double& a0, double kb, float gauss, float4 u) {
  float a = fabsf(gauss);
  float b = -logf(1.0f - u.x);
  float y = a * a + b;
  y = (float)((double)y / kb);
  const float help = u.y;
  if ((2.0f * (help * help)) <= (2.0f - y)) {
    a0 = (double)(1.0f - y);
    return 1;
  }
  a0 = 0.0;
  return 0;
}

// dev_heatbath_su2 in FP32 arithmetic, for the FP32 sweeps of g: the same trial,
// acceptance and construction as below, with the SU(2) parameters formed in float
// (g is stored in FP32, and GB300's FP64 rate is 1/64 of its FP32 rate, so the FP64
// form made this kernel FP64-pipe bound)
__device__ __forceinline__ Su2<float> heatbath_su2_f32(const Su2<float>& w, double beta,
                                                       float gauss, float4 u) {
  const float k = fm(w.v[3], w.v[3], fm(w.v[2], w.v[2], fm(w.v[1], w.v[1], w.v[0] * w.v[0])));
  const float rdet = rsqrtf(k);
  // dev_get_a0 with y / (k beta) in float
  const float a = fabsf(gauss);
  const float y = __fdiv_rn(fm(a, a, -logf(1.0f - u.x)), (float)((double)k * beta));
  if (!((2.0f * (u.y * u.y)) <= (2.0f - y))) return w;
  const float a0 = 1.0f - y;
  const float norm = sqrtf(1.0f - a0 * a0);
  const float cos_theta = 2.0f * u.z - 1.0f;
  const float sin_theta = sqrtf(1.0f - cos_theta * cos_theta);
  float sphi, cphi;
  sincospif(2.0f * u.w, &sphi, &cphi);
  const float a1 = norm * sin_theta * cphi, a2 = norm * sin_theta * sphi, a3 = norm * cos_theta;
  const float v0 = w.v[0] * rdet, v1 = w.v[1] * rdet, v2 = w.v[2] * rdet, v3 = w.v[3] * rdet;
  Su2<float> al;
  al.v[0] = a0 * v0 - a1 * v1 - a2 * v2 - a3 * v3;
  al.v[1] = a0 * v1 + a1 * v0 - a2 * v3 + a3 * v2;
  al.v[2] = a0 * v2 + a2 * v0 - a3 * v1 + a1 * v3;
  al.v[3] = a0 * v3 + a3 * v0 - a1 * v2 + a2 * v1;
  return al;
}

// dev_heatbath_su2 (simulated_annealing.cu:33-73).  k = |w|^2 as in the reference;
// on rejection alpha = w (unnormalized), which the final reunitarization absorbs.
template <typename T>
__device__ __forceinline__ Su2<T> heatbath_su2(const Su2<T>& wt, double beta, float gauss,
                                               float4 u) {
  if constexpr (sizeof(T) == 4) return heatbath_su2_f32(wt, beta, gauss, u);
  double w[4] = {(double)wt.v[0], (double)wt.v[1], (double)wt.v[2], (double)wt.v[3]};
  const double k = w[0] * w[0] + w[1] * w[1] + w[2] * w[2] + w[3] * w[3];
  const double rdet = rsqrt(k);
  double v[4];
#pragma unroll
  for (int i = 0; i < 4; i++) v[i] = w[i] * rdet;
  double a[4];
  const int ret = get_a0(a[0], k * beta, gauss, u);
  Su2<T> al;
  if (ret == 1) {
    const double norm = sqrt(1.0 - a[0] * a[0]);
    const double cos_theta = 2.0 * (double)u.z - 1.0;
    const double sin_theta = sqrt(1.0 - cos_theta * cos_theta);
    const double phi = 6.2831853071795862 * (double)u.w;
    double sphi, cphi;
    sincos(phi, &sphi, &cphi);
    a[1] = norm * sin_theta * cphi;
    a[2] = norm * sin_theta * sphi;
    a[3] = norm * cos_theta;
    // dev_su2_ti_su2(alpha, a, v) (dev_su3.cu:1385-1399)
    al.v[0] = (T)(a[0] * v[0] - a[1] * v[1] - a[2] * v[2] - a[3] * v[3]);
    al.v[1] = (T)(a[0] * v[1] + a[1] * v[0] - a[2] * v[3] + a[3] * v[2]);
    al.v[2] = (T)(a[0] * v[2] + a[2] * v[0] - a[3] * v[1] + a[1] * v[3]);
    al.v[3] = (T)(a[0] * v[3] + a[3] * v[0] - a[1] * v[2] + a[2] * v[1]);
  } else {
    al = wt;
  }
  return al;
}

// cabibbo_marinari_heatbath (simulated_annealing.cu:81-142): the three subgroups use
// the same random numbers
template <typename T>
__device__ __forceinline__ void cm_heatbath(Mat3<T>& g, const Mat3<T>& star, double beta,
                                            float gauss, float4 u) {
#pragma unroll
  for (int s = 0; s < 3; s++) {
    const int a = sub_a(s), b = sub_b(s);
    Su2<T> w = su2_extract(g, star, a, b);
    Su2<T> al = heatbath_su2(w, beta, gauss, u);
    su2_rotate(g, a, b, al);
  }
}

// Kennedy-Pendleton SU(2) heatbath for the Wilson action: the subgroup weight is
// exp(beta * alpha.w) with beta = beta_lattice/3, so a0 has density
// sqrt(1-a0^2) exp(beta |w| a0).  One trial: 2 lambda^2 = (E + g^2/2) / (beta |w|)
// with E exponential and g standard normal, a0 = 1 - 2 lambda^2, accepted when
// u^2 <= 1 - lambda^2; a rejected trial leaves the subgroup unchanged (the chain
// still has the Wilson-action distribution as its fixed point).
template <typename T>
__device__ __forceinline__ Su2<T> heatbath_su2_kp(const Su2<T>& wt, double beta, float gauss,
                                                  float4 u) {
  const double w[4] = {(double)wt.v[0], (double)wt.v[1], (double)wt.v[2], (double)wt.v[3]};
  const double k = sqrt(w[0] * w[0] + w[1] * w[1] + w[2] * w[2] + w[3] * w[3]);
  Su2<T> al;
  al.v[0] = T(1);
  al.v[1] = al.v[2] = al.v[3] = T(0);
  if (!(k > 0.0)) return al;
  const double rk = 1.0 / k;
  const double E = -log(1.0 - (double)u.x);
  const double y = (E + 0.5 * (double)gauss * (double)gauss) / (beta * k);
  if (!((double)u.y * (double)u.y <= 1.0 - 0.5 * y)) return al;
  double v[4];
#pragma unroll
  for (int i = 0; i < 4; i++) v[i] = w[i] * rk;
  double a[4];
  a[0] = 1.0 - y;
  const double norm = sqrt(fmax(0.0, 1.0 - a[0] * a[0]));
  const double cos_theta = 2.0 * (double)u.z - 1.0;
  const double sin_theta = sqrt(fmax(0.0, 1.0 - cos_theta * cos_theta));
  double sphi, cphi;
  sincospi(2.0 * (double)u.w, &sphi, &cphi);
  a[1] = norm * sin_theta * cphi;
  a[2] = norm * sin_theta * sphi;
  a[3] = norm * cos_theta;
  al.v[0] = (T)(a[0] * v[0] - a[1] * v[1] - a[2] * v[2] - a[3] * v[3]);
  al.v[1] = (T)(a[0] * v[1] + a[1] * v[0] - a[2] * v[3] + a[3] * v[2]);
  al.v[2] = (T)(a[0] * v[2] + a[2] * v[0] - a[3] * v[1] + a[1] * v[3]);
  al.v[3] = (T)(a[0] * v[3] + a[3] * v[0] - a[1] * v[2] + a[2] * v[1]);
  return al;
}

// the same Kennedy-Pendleton trial in FP32 arithmetic (the FP32 thermalization)
__device__ __forceinline__ Su2<float> heatbath_su2_kp_f32(const Su2<float>& w, double beta,
                                                          float gauss, float4 u) {
  const float k = sqrtf(fm(w.v[3], w.v[3], fm(w.v[2], w.v[2], fm(w.v[1], w.v[1], w.v[0] * w.v[0]))));
  Su2<float> al;
  al.v[0] = 1.f;
  al.v[1] = al.v[2] = al.v[3] = 0.f;
  if (!(k > 0.f)) return al;
  const float rk = 1.f / k;
  const float E = -logf(1.f - u.x);
  const float y = __fdiv_rn(fm(0.5f * gauss, gauss, E), (float)beta * k);
  if (!(u.y * u.y <= 1.f - 0.5f * y)) return al;
  const float a0 = 1.f - y;
  const float norm = sqrtf(fmaxf(0.f, 1.f - a0 * a0));
  const float cos_theta = 2.f * u.z - 1.f;
  const float sin_theta = sqrtf(fmaxf(0.f, 1.f - cos_theta * cos_theta));
  float sphi, cphi;
  sincospif(2.f * u.w, &sphi, &cphi);
  const float a1 = norm * sin_theta * cphi, a2 = norm * sin_theta * sphi, a3 = norm * cos_theta;
  const float v0 = w.v[0] * rk, v1 = w.v[1] * rk, v2 = w.v[2] * rk, v3 = w.v[3] * rk;
  al.v[0] = a0 * v0 - a1 * v1 - a2 * v2 - a3 * v3;
  al.v[1] = a0 * v1 + a1 * v0 - a2 * v3 + a3 * v2;
  al.v[2] = a0 * v2 + a2 * v0 - a3 * v1 + a1 * v3;
  al.v[3] = a0 * v3 + a3 * v0 - a1 * v2 + a2 * v1;
  return al;
}

// star for the gauge-transformation update (same as the OR kernel; FP32 with 12-real
// links in the OR sweep's reduced form)
template <typename T, int NRU, int NDIR>
__device__ __forceinline__ void g_star(const Lattice& L, const Site& c, int parity,
                                       const typename VecOf<T>::type* __restrict__ U,
                                       const typename VecOf<T>::type* __restrict__ G,
                                       Mat3<T>& star) {
  if constexpr (sizeof(T) == 4 && NRU == 12) {
    compute_star_f32<NDIR>(L, c, parity, U, G, star);
    return;
  }
  constexpr int NCU = Field<T, NRU>::NCHUNK;
  constexpr int NCG = Field<T, 12>::NCHUNK;
  const size_t vh = (size_t)L.vh;
  const int q = 1 - parity;
  const typename VecOf<T>::type* Gq = G + (size_t)q * NCG * vh;
  mzero(star);
#pragma unroll
  for (int mu = 0; mu < NDIR; mu++) {
    Mat3<T> a, b;
    Field<T, NRU>::load(U + (size_t)(parity * 4 + mu) * NCU * vh, vh, c.i, a);
    Field<T, 12>::load(Gq, vh, nb_fwd(L, c, mu), b);
    addmul_nd(star, a, b);
    const int jb = nb_bwd(L, c, mu);
    Field<T, NRU>::load(U + (size_t)(q * 4 + mu) * NCU * vh, vh, jb, a);
    Field<T, 12>::load(Gq, vh, jb, b);
    addmul_dd(star, a, b);
  }
}

template <typename T, int NRU>
__global__ void __launch_bounds__(256) sa_heatbath_kernel(Lattice L,
                                                           const typename VecOf<T>::type* U,
                                                           typename VecOf<T>::type* G, int parity,
                                                           double beta, const float* gauss,
                                                           const float4* unif4) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= L.vh) return;
  const size_t vh = (size_t)L.vh;
  const Site c = site_of(L, i, parity);
  Mat3<T> star, g;
  g_star<T, NRU, 4>(L, c, parity, U, G, star);
  typename VecOf<T>::type* Gp = G + (size_t)parity * Field<T, 12>::NCHUNK * vh;
  Field<T, 12>::load(Gp, vh, i, g);
  cm_heatbath(g, star, beta, __ldg(gauss + i), __ldg(unif4 + i));
  normalize<T, false>(g);
  Field<T, 12>::store(Gp, vh, i, g);
}

template <typename T, int NRU, int NDIR>
__global__ void __launch_bounds__(256) micro_kernel(Lattice L, const typename VecOf<T>::type* U,
                                                     typename VecOf<T>::type* G, int parity) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= L.vh) return;
  const size_t vh = (size_t)L.vh;
  const Site c = site_of(L, i, parity);
  Mat3<T> star, g;
  g_star<T, NRU, NDIR>(L, c, parity, U, G, star);
  typename VecOf<T>::type* Gp = G + (size_t)parity * Field<T, 12>::NCHUNK * vh;
  Field<T, 12>::load(Gp, vh, i, g);
  cm_micro(g, star);
  normalize<T, false>(g);
  Field<T, 12>::store(Gp, vh, i, g);
}

void launch_sa_heatbath(int prec, int link_nr, const Lattice& L, const void* U, void* G,
                        int parity, double beta, const float* gauss, const float* unif, int block,
                        cudaStream_t s) {
  dim3 grid((L.vh + block - 1) / block);
  const float4* u4 = (const float4*)unif;
  if (prec == 0 && link_nr == 8)
    sa_heatbath_kernel<float, 8><<<grid, block, 0, s>>>(L, (const float4*)U, (float4*)G, parity,
                                                         beta, gauss, u4);
  else if (prec == 0)
    sa_heatbath_kernel<float, 12><<<grid, block, 0, s>>>(L, (const float4*)U, (float4*)G, parity,
                                                          beta, gauss, u4);
  else if (link_nr == 18)
    sa_heatbath_kernel<double, 18><<<grid, block, 0, s>>>(L, (const double2*)U, (double2*)G,
                                                           parity, beta, gauss, u4);
  else
    sa_heatbath_kernel<double, 12><<<grid, block, 0, s>>>(L, (const double2*)U, (double2*)G,
                                                           parity, beta, gauss, u4);
}

void launch_micro(int prec, int link_nr, int ndir, const Lattice& L, const void* U, void* G,
                  int parity, int block, cudaStream_t s) {
  dim3 grid((L.vh + block - 1) / block);
#define MICRO(T, NR, ND)                                                        \
  micro_kernel<T, NR, ND><<<grid, block, 0, s>>>(L, (const typename VecOf<T>::type*)U, \
                                                   (typename VecOf<T>::type*)G, parity)
  if (prec == 0 && link_nr == 8) {
    if (ndir == 4) MICRO(float, 8, 4);
    else MICRO(float, 8, 3);
  } else if (prec == 0) {
    if (ndir == 4) MICRO(float, 12, 4);
    else MICRO(float, 12, 3);
  } else if (link_nr == 18) {
    if (ndir == 4) MICRO(double, 18, 4);
    else MICRO(double, 18, 3);
  } else {
    if (ndir == 4) MICRO(double, 12, 4);
    else MICRO(double, 12, 3);
  }
#undef MICRO
}

// ---------------------------------------------------------------------------
// link heatbath (heatbath_thermalization.cu:235-308, 493-550)
// ---------------------------------------------------------------------------
struct Coord {
  int x, y, z, t;
};
// one step (d = +-1) with periodic wrap, without an integer division
__device__ __forceinline__ int wrap_step(int v, int d, int n) {
  v += d;
  return v < 0 ? v + n : (v >= n ? v - n : v);
}
__device__ __forceinline__ Coord cshift(const Lattice& L, Coord c, int mu, int d) {
  if (mu == 0) c.x = wrap_step(c.x, d, L.lx);
  else if (mu == 1) c.y = wrap_step(c.y, d, L.ly);
  else if (mu == 2) c.z = wrap_step(c.z, d, L.lz);
  else c.t = wrap_step(c.t, d, L.lt);
  return c;
}

template <int NR>
__device__ __forceinline__ void ld_link(const Lattice& L, const double2* __restrict__ U, Coord c,
                                        int mu, Mat3<double>& m) {
  constexpr int NC = Field<double, NR>::NCHUNK;
  const int p = (c.x + c.y + c.z + c.t) & 1;
  const int i = (c.x >> 1) + L.lxh * (c.y + L.ly * (c.z + L.lz * c.t));
  Field<double, NR>::load(U + (size_t)(p * 4 + mu) * NC * L.vh, (size_t)L.vh, i, m);
}

// VARIANT 0: the reference's update (one random set per link, all subgroups);
// VARIANT 1: Kennedy-Pendleton, subgroup s draws slot 4*i + ((nu + s) & 3) of the
// fields, so the three subgroups use independent numbers.
template <int NR, int VARIANT>
__global__ void __launch_bounds__(128) link_heatbath_kernel(Lattice L, double2* U, int parity,
                                                             int nu, double beta3,
                                                             const float* gauss,
                                                             const float4* unif4) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= L.vh) return;
  const Site s = site_of(L, i, parity);
  const Coord x = {2 * s.xh + s.s, s.y, s.z, s.t};
  Mat3<double> staple, h1, h2, h3;
  mzero(staple);
#pragma unroll 1
  for (int mu = 0; mu < 4; mu++) {
    if (mu == nu) continue;
    const Coord xpn = cshift(L, x, nu, 1);
    const Coord xpm = cshift(L, x, mu, 1);
    const Coord xmm = cshift(L, x, mu, -1);
    const Coord xpnmm = cshift(L, xpn, mu, -1);
    // U_mu(x+nu) U_nu^+(x+mu) U_mu^+(x)
    ld_link<NR>(L, U, xpn, mu, h1);
    ld_link<NR>(L, U, xpm, nu, h2);
    mzero(h3);
    addmul_nd(h3, h1, h2);
    ld_link<NR>(L, U, x, mu, h1);
    addmul_nd(staple, h3, h1);
    // U_mu^+(x+nu-mu) U_nu^+(x-mu) U_mu(x-mu)
    ld_link<NR>(L, U, xpnmm, mu, h1);
    ld_link<NR>(L, U, xmm, nu, h2);
    mzero(h3);
    addmul_dd(h3, h1, h2);  // h1^+ h2^+
    ld_link<NR>(L, U, xmm, mu, h1);
    addmul(staple, h3, h1);
  }
  constexpr int NC = Field<double, NR>::NCHUNK;
  double2* blk = U + (size_t)(parity * 4 + nu) * NC * L.vh;
  Mat3<double> link;
  Field<double, NR>::load(blk, (size_t)L.vh, i, link);
  if (VARIANT == 0) {
    const int r = 4 * i + nu;
    cm_heatbath(link, staple, beta3, __ldg(gauss + r), __ldg(unif4 + r));
  } else {
#pragma unroll
    for (int sg = 0; sg < 3; sg++) {
      const int r = 4 * i + ((nu + sg) & 3);
      const int a = sub_a(sg), b = sub_b(sg);
      Su2<double> w = su2_extract(link, staple, a, b);
      su2_rotate(link, a, b, heatbath_su2_kp(w, beta3, __ldg(gauss + r), __ldg(unif4 + r)));
    }
  }
  normalize<double, true>(link);
  Field<double, NR>::store(blk, (size_t)L.vh, i, link);
}

// The same update in FP32 arithmetic, for thermalization: staples from the FP32 link
// copy (12 reals), the SU(2) heatbath steps on an FP32 copy of the link, then the new
// link is reunitarized in double-float arithmetic (~48 bits, about 1e-14 from
// unitary), widened to FP64 and stored in both copies (the FP32 one as the rounding of
// the FP64 one), so they stay in step.  A heatbath draws the new link at random; FP32
// arithmetic moves the drawn link by ~1e-7, far below the spread of the draw, so the
// chain samples the same distribution, while the kernel runs on the FP32 units
// instead of the FP64 pipe.
__device__ __forceinline__ const float4* link_plane32(const Lattice& L,
                                                     const float4* __restrict__ U32, Coord c,
                                                     int mu, int& i) {
  const int p = (c.x + c.y + c.z + c.t) & 1;
  i = (c.x >> 1) + L.lxh * (c.y + L.ly * (c.z + L.lz * c.t));
  return U32 + (size_t)(p * 4 + mu) * 3 * L.vh;
}
__device__ __forceinline__ void ld_link32(const Lattice& L, const float4* __restrict__ U32,
                                          Coord c, int mu, Mat3<float>& m) {
  const int p = (c.x + c.y + c.z + c.t) & 1;
  const int i = (c.x >> 1) + L.lxh * (c.y + L.ly * (c.z + L.lz * c.t));
  Field<float, 12>::load(U32 + (size_t)(p * 4 + mu) * 3 * L.vh, (size_t)L.vh, i, m);
}

// Six blocks of 128 per SM (80 registers, a few bytes spilled): 3% faster per
// thermalization sweep on GB300 than the 90-register build at five.
template <int NR, int VARIANT>
__global__ void __launch_bounds__(128, 6) link_heatbath_f32_kernel(Lattice L, double2* U,
                                                                 float4* U32, int parity, int nu,
                                                                 double beta3, const float* gauss,
                                                                 const float4* unif4) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= L.vh) return;
  const Site s = site_of(L, i, parity);
  const Coord x = {2 * s.xh + s.s, s.y, s.z, s.t};
  // Each staple term is an SU(3) product: its rows 0, 1 need rows 0, 1 of the first
  // factor only, and its row 2 is conj(row 0 x row 1), as in the FP32 OR star.
  const size_t vh = (size_t)L.vh;
  Mat3<float> staple, a, b;
  mzero(staple);
#pragma unroll
  for (int mu = 0; mu < 4; mu++) {
    if (mu == nu) continue;
    const Coord xpn = cshift(L, x, nu, 1);
    const Coord xpm = cshift(L, x, mu, 1);
    const Coord xmm = cshift(L, x, mu, -1);
    const Coord xpnmm = cshift(L, xpn, mu, -1);
    cplx<float> P[2][3], T[2][3];
    int j;
    // U_mu(x+nu) U_nu^+(x+mu) U_mu^+(x): P = rows 0,1 of A B^+, T = rows 0,1 of P C^+
    const float4* pl = link_plane32(L, U32, xpn, mu, j);
    link_rows01(pl, vh, j, a);
    pl = link_plane32(L, U32, xpm, nu, j);
    link_full(pl, vh, j, b);
#pragma unroll
    for (int r = 0; r < 2; r++)
#pragma unroll
      for (int k = 0; k < 3; k++) {
        cplx<float> y = cmulc(a.e[r][0], b.e[k][0]);
        cmacc(y, a.e[r][1], b.e[k][1]);
        cmacc(y, a.e[r][2], b.e[k][2]);
        P[r][k] = y;
      }
    pl = link_plane32(L, U32, x, mu, j);
    link_full(pl, vh, j, b);
#pragma unroll
    for (int r = 0; r < 2; r++)
#pragma unroll
      for (int k = 0; k < 3; k++) {
        cplx<float> y = cmulc(P[r][0], b.e[k][0]);
        cmacc(y, P[r][1], b.e[k][1]);
        cmacc(y, P[r][2], b.e[k][2]);
        T[r][k] = y;
        staple.e[r][k] = cadd(staple.e[r][k], y);
      }
    acc_cross_conj(staple.e[2][0], T[0][1], T[1][2], T[0][2], T[1][1]);
    acc_cross_conj(staple.e[2][1], T[0][2], T[1][0], T[0][0], T[1][2]);
    acc_cross_conj(staple.e[2][2], T[0][0], T[1][1], T[0][1], T[1][0]);
    // U_mu^+(x+nu-mu) U_nu^+(x-mu) U_mu(x-mu) = Q^+ F with Q = E D, E = U_nu(x-mu),
    // D = U_mu(x+nu-mu); Y = conj of its rows 0,1, so its row 2 is Y_0 x Y_1
    pl = link_plane32(L, U32, xmm, nu, j);
    link_rows01(pl, vh, j, a);
    pl = link_plane32(L, U32, xpnmm, mu, j);
    link_full(pl, vh, j, b);
    Mat3<float> q;
#pragma unroll
    for (int r = 0; r < 2; r++)
#pragma unroll
      for (int k = 0; k < 3; k++) {
        cplx<float> y = cmul(a.e[r][0], b.e[0][k]);
        cmac(y, a.e[r][1], b.e[1][k]);
        cmac(y, a.e[r][2], b.e[2][k]);
        q.e[r][k] = y;
      }
    row2_from_01(q);
    pl = link_plane32(L, U32, xmm, mu, j);
    link_full(pl, vh, j, b);
#pragma unroll
    for (int r = 0; r < 2; r++)
#pragma unroll
      for (int k = 0; k < 3; k++) {
        cplx<float> y = cmulc(q.e[0][r], b.e[0][k]);
        cmacc(y, q.e[1][r], b.e[1][k]);
        cmacc(y, q.e[2][r], b.e[2][k]);
        T[r][k] = y;
        staple.e[r][k] = cadd(staple.e[r][k], cconj(y));
      }
    acc_cross(staple.e[2][0], T[0][1], T[1][2], T[0][2], T[1][1]);
    acc_cross(staple.e[2][1], T[0][2], T[1][0], T[0][0], T[1][2]);
    acc_cross(staple.e[2][2], T[0][0], T[1][1], T[0][1], T[1][0]);
  }
  Mat3<float> link;
  ld_link32(L, U32, x, nu, link);
  if (VARIANT == 0) {
    const int r = 4 * i + nu;
    cm_heatbath(link, staple, beta3, __ldg(gauss + r), __ldg(unif4 + r));
  } else {
#pragma unroll
    for (int sg = 0; sg < 3; sg++) {
      const int r = 4 * i + ((nu + sg) & 3);
      const int a = sub_a(sg), b = sub_b(sg);
      Su2<float> w = su2_extract(link, staple, a, b);
      su2_rotate(link, a, b, heatbath_su2_kp_f32(w, beta3, __ldg(gauss + r), __ldg(unif4 + r)));
    }
  }
  // Reunitarize in double-float (~48 bits, on the FP32 units; FP64 Gram-Schmidt made
  // this kernel FP64-pipe bound on GB300) and widen: the FP64 link is unitary to ~1e-14
  Mat3<dfl> lf;
#pragma unroll
  for (int r = 0; r < 2; r++)
#pragma unroll
    for (int c = 0; c < 3; c++)
      lf.e[r][c] = cmk<dfl>(dfl(link.e[r][c].re, 0.0f), dfl(link.e[r][c].im, 0.0f));
  normalize<dfl, NR == 18>(lf);
  // widened on the integer units (gfx_widen.h) to one FP64 ulp of the double-float;
  // the FP32 copy, hi, is the FP32 rounding of the FP64 one
  Mat3<double> ld;
  mzero(ld);
#pragma unroll
  for (int r = 0; r < (NR == 18 ? 3 : 2); r++)
#pragma unroll
    for (int c = 0; c < 3; c++) {
      const dfl re = lf.e[r][c].re, im = lf.e[r][c].im;
      ld.e[r][c] = cmk<double>(widen_df(re.hi, re.lo), widen_df(im.hi, im.lo));
      if (r < 2) link.e[r][c] = cmk<float>(re.hi, im.hi);
    }
  constexpr int NC = Field<double, NR>::NCHUNK;
  Field<double, NR>::store(U + (size_t)(parity * 4 + nu) * NC * L.vh, (size_t)L.vh, i, ld);
  Field<float, 12>::store(U32 + (size_t)(parity * 4 + nu) * 3 * L.vh, (size_t)L.vh, i, link);
}

void launch_link_heatbath_f32(int link_nr, const Lattice& L, void* U, void* U32, int parity,
                              int nu, double beta3, const float* gauss, const float* unif,
                              int variant, cudaStream_t s) {
  dim3 grid((L.vh + 127) / 128);
#define LHB32(NR, VAR)                                                                      \
  link_heatbath_f32_kernel<NR, VAR><<<grid, 128, 0, s>>>(L, (double2*)U, (float4*)U32, parity, \
                                                         nu, beta3, gauss, (const float4*)unif)
  if (link_nr == 18) {
    if (variant) LHB32(18, 1);
    else LHB32(18, 0);
  } else {
    if (variant) LHB32(12, 1);
    else LHB32(12, 0);
  }
#undef LHB32
}

void launch_link_heatbath(int link_nr, const Lattice& L, void* U, int parity, int nu, double beta3,
                          const float* gauss, const float* unif, int variant, int block,
                          cudaStream_t s) {
  dim3 grid((L.vh + block - 1) / block);
#define LHB(NR, VAR)                                                                \
  link_heatbath_kernel<NR, VAR><<<grid, block, 0, s>>>(L, (double2*)U, parity, nu, beta3, \
                                                       gauss, (const float4*)unif)
  if (link_nr == 18) {
    if (variant) LHB(18, 1);
    else LHB(18, 0);
  } else {
    if (variant) LHB(12, 1);
    else LHB(12, 0);
  }
#undef LHB
}

}  // namespace gfx
