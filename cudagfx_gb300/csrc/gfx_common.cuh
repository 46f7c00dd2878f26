// gfx_common.cuh -- device code shared by the single-lattice and batched kernels:
// precision-converting loads, the star w(x), the per-site functional and the FP64
// block reduction.  Sharing them keeps the batched results bit-identical per copy.
#pragma once

#include <type_traits>

#include "gfx_device.cuh"
#include "gfx_internal.h"
#include "gfx_narrow.h"
#include "gfx_pair.cuh"

namespace gfx {

// ---------------------------------------------------------------------------
// generic loads with precision conversion
// ---------------------------------------------------------------------------
template <typename TC, typename TS, int NR>
struct Load {
  typedef typename VecOf<TS>::type V;
  __device__ static __forceinline__ void go(const V* base, size_t stride, int i, Mat3<TC>& m) {
    Field<TC, NR>::load(base, stride, i, m);
  }
};
// FP64 compute on FP32-stored g: widen rows 0,1 and reunitarize in FP64
template <>
struct Load<double, float, 12> {
  __device__ static __forceinline__ void go(const float4* base, size_t stride, int i,
                                            Mat3<double>& m) {
    Mat3<float> f;
    Field<float, 12>::load(base, stride, i, f);
#pragma unroll
    for (int r = 0; r < 2; r++)
#pragma unroll
      for (int c = 0; c < 3; c++) m.e[r][c] = cmk<double>(f.e[r][c].re, f.e[r][c].im);
    normalize<double, true>(m);
  }
};

// an FP64 matrix of NC double2 planes (6: rows 0,1, row 2 rebuilt; 9: all rows) as
// double-float pairs, split on the integer units (gfx_narrow.h)
template <int NC>
__device__ __forceinline__ void load_narrow(const double2* __restrict__ base, size_t stride,
                                            int i, Mat3<dfl>& m) {
#pragma unroll
  for (int k = 0; k < NC; k++) {
    const double2 v = __ldg(base + k * stride + i);
    float rh, rl, ih, il;
    narrow_df(v.x, rh, rl);
    narrow_df(v.y, ih, il);
    m.e[k / 3][k % 3] = cmk<dfl>(dfl(rh, rl), dfl(ih, il));
  }
  if (NC == 6) row2_from_01(m);
}

// ---------------------------------------------------------------------------
// L2 warm-up for one block of checkerboard sites [i0, i0 + n) of one parity.
// In the even/odd SoA layout everything such a block reads lies in contiguous
// ranges of 16-byte plane elements: its forward links and its own g at the block's
// indices, and the other parity's g and backward links at the index shifts
// 0/+-1 (x), +-sy, +-sz, +-st.  One cp.async.bulk.prefetch.L2 per range and plane,
// issued by the first threads of the block before any load, puts all of the
// block's DRAM requests in flight at once; the regular loads then hit L2.  It is a
// hint: the neighbours that wrap around the lattice fall outside the ranges and
// are fetched by the regular loads, and every range is clamped to its plane.
// A tuner candidate (staging = 1): on GB300 the extra L2 traffic makes the FP32
// sweep slower, and the FP64 sweeps are compute-bound either way.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void l2_prefetch_range(const void* plane, int vh, int a, int b) {
  a = max(a, 0);
  b = min(b, vh);
  if (b > a)
    asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"((const char*)plane +
                                                                     (size_t)a * 16),
                 "r"((b - a) * 16)
                 : "memory");
}

// NCU / NCG: 16-byte planes per link / per g.  U and G are the field bases.
template <int NCU, int NCG, int NDIR>
__device__ __forceinline__ void prefetch_range_k(const Lattice& L, int parity, int i0, int n,
                                                 const void* U, const void* G, int k) {
  constexpr int NSHIFT = 2 * NDIR - 1;  // x (both sides merged), then +-y, +-z, +-t
  constexpr int N_FWD = NDIR * NCU, N_OWN = NCG, N_NB = NSHIFT * NCG;
  const int vh = L.vh, q = 1 - parity;
  const char* u = (const char*)U;
  const char* g = (const char*)G;
  const size_t plane = (size_t)vh * 16;
  const int strides[4] = {0, L.sy, L.sz, L.st};
  if (k < N_FWD) {
    const int mu = k / NCU, c = k - mu * NCU;
    l2_prefetch_range(u + ((size_t)(parity * 4 + mu) * NCU + c) * plane, vh, i0, i0 + n);
    return;
  }
  k -= N_FWD;
  if (k < N_OWN) {
    l2_prefetch_range(g + ((size_t)parity * NCG + k) * plane, vh, i0, i0 + n);
    return;
  }
  k -= N_OWN;
  if (k < N_NB) {
    const int r = k / NCG, c = k - r * NCG;
    const char* p = g + ((size_t)q * NCG + c) * plane;
    if (r == 0) {
      l2_prefetch_range(p, vh, i0 - 1, i0 + n + 1);
    } else {
      const int s = strides[(r + 1) >> 1] * ((r & 1) ? 1 : -1);
      l2_prefetch_range(p, vh, i0 + s, i0 + n + s);
    }
    return;
  }
  k -= N_NB;
  const int mu = k / NCU, c = k - mu * NCU;
  const int s = strides[mu];
  l2_prefetch_range(u + ((size_t)(q * 4 + mu) * NCU + c) * plane, vh, i0 - s - (mu == 0),
                    i0 + n - s);
}

template <int NCU, int NCG, int NDIR>
__device__ __forceinline__ void prefetch_block(const Lattice& L, int parity, int i0, int n,
                                               const void* U, const void* G) {
  constexpr int NTOT = 2 * NDIR * NCU + 2 * NDIR * NCG;  // fwd + own + neighbours + bwd
  for (int k = threadIdx.x; k < NTOT; k += blockDim.x)
    prefetch_range_k<NCU, NCG, NDIR>(L, parity, i0, n, U, G, k);
}


// star w(x) = sum_mu U_mu(x) g^+(x+mu) + U_mu^+(x-mu) g^+(x-mu)   (overrelax.cu:350-394)
template <typename TC, typename TSU, int NRU, typename TSG, int NRG, int NDIR>
__device__ __forceinline__ void compute_star(const Lattice& L, const Site& c, int parity,
                                             const typename VecOf<TSU>::type* __restrict__ U,
                                             const typename VecOf<TSG>::type* __restrict__ G,
                                             Mat3<TC>& star) {
  constexpr int NCU = Field<TSU, NRU>::NCHUNK;
  constexpr int NCG = Field<TSG, NRG>::NCHUNK;
  const size_t vh = (size_t)L.vh;
  const int q = 1 - parity;
  const typename VecOf<TSG>::type* Gq = G + (size_t)q * NCG * vh;
  mzero(star);
#pragma unroll
  for (int mu = 0; mu < NDIR; mu++) {
    Mat3<TC> a, b;
    Load<TC, TSU, NRU>::go(U + (size_t)(parity * 4 + mu) * NCU * vh, vh, c.i, a);
    const int jf = nb_fwd(L, c, mu);
    Load<TC, TSG, NRG>::go(Gq, vh, jf, b);
    addmul_nd(star, a, b);
    const int jb = nb_bwd(L, c, mu);
    Load<TC, TSU, NRU>::go(U + (size_t)(q * 4 + mu) * NCU * vh, vh, jb, a);
    Load<TC, TSG, NRG>::go(Gq, vh, jb, b);
    addmul_dd(star, a, b);
  }
}

// ---------------------------------------------------------------------------
// FP32 star with fewer operations.  Each term is an SU(3) product P; its rows 0, 1
// need only rows 0, 1 of one factor, and its row 2 is conj(P_0 x P_1):
//   forward  P = U_mu(x) g^+(x+mu):  rows 0,1 of U, all of g
//   backward Q = g(x-mu) U_mu(x-mu): rows 0,1 of g, all of U;  w += Q^+
// so one factor per term is never reconstructed and a third of its products is
// replaced by a cross product.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void load12_rows01(const float4* __restrict__ base, size_t stride,
                                              int i, Mat3<float>& m) {
  const float4 a = __ldg(base + i), b = __ldg(base + stride + i), c = __ldg(base + 2 * stride + i);
  m.e[0][0] = cmk(a.x, a.y);
  m.e[0][1] = cmk(a.z, a.w);
  m.e[0][2] = cmk(b.x, b.y);
  m.e[1][0] = cmk(b.z, b.w);
  m.e[1][1] = cmk(c.x, c.y);
  m.e[1][2] = cmk(c.z, c.w);
}
// acc += conj(p q - r s)  and  acc += p q - r s
template <typename T>
__device__ __forceinline__ void acc_cross_conj(cplx<T>& acc, cplx<T> p, cplx<T> q, cplx<T> r,
                                               cplx<T> s) {
  acc.re = fm(p.re, q.re, fm(-p.im, q.im, fm(-r.re, s.re, fm(r.im, s.im, acc.re))));
  acc.im = fm(-p.re, q.im, fm(-p.im, q.re, fm(r.re, s.im, fm(r.im, s.re, acc.im))));
}
template <typename T>
__device__ __forceinline__ void acc_cross(cplx<T>& acc, cplx<T> p, cplx<T> q, cplx<T> r,
                                          cplx<T> s) {
  acc.re = fm(p.re, q.re, fm(-p.im, q.im, fm(-r.re, s.re, fm(r.im, s.im, acc.re))));
  acc.im = fm(p.re, q.im, fm(p.im, q.re, fm(-r.re, s.im, fm(-r.im, s.re, acc.im))));
}

// An FP32 12-real field read (and written) with an L2 eviction priority: pol is a
// createpolicy handle, evict_last for g (48 MB for 32^4, so it can stay resident in
// L2 while the 192 MB of links stream past it), evict_first for links.
struct HintP {
  const float4* p;
  uint64_t pol;
  __device__ __forceinline__ HintP operator+(size_t off) const { return {p + off, pol}; }
};
__device__ __forceinline__ uint64_t l2_policy_evict_last() {
  uint64_t pol;
  asm volatile("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(pol));
  return pol;
}
__device__ __forceinline__ uint64_t l2_policy_evict_first() {
  uint64_t pol;
  asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(pol));
  return pol;
}
__device__ __forceinline__ float4 ldg_hint(const float4* p, uint64_t pol) {
  float4 v;
  asm("ld.global.nc.L2::cache_hint.v4.f32 {%0, %1, %2, %3}, [%4], %5;"
      : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w)
      : "l"(p), "l"(pol));
  return v;
}
__device__ __forceinline__ void stg_hint(float4* p, float4 v, uint64_t pol) {
  asm volatile("st.global.L2::cache_hint.v4.f32 [%0], {%1, %2, %3, %4}, %5;" ::"l"(p), "f"(v.x),
               "f"(v.y), "f"(v.z), "f"(v.w), "l"(pol)
               : "memory");
}
__device__ __forceinline__ void load12_rows01(const HintP& base, size_t stride, int i,
                                              Mat3<float>& m) {
  const float4 a = ldg_hint(base.p + i, base.pol), b = ldg_hint(base.p + stride + i, base.pol),
               c = ldg_hint(base.p + 2 * stride + i, base.pol);
  m.e[0][0] = cmk(a.x, a.y);
  m.e[0][1] = cmk(a.z, a.w);
  m.e[0][2] = cmk(b.x, b.y);
  m.e[1][0] = cmk(b.z, b.w);
  m.e[1][1] = cmk(c.x, c.y);
  m.e[1][2] = cmk(c.z, c.w);
}
__device__ __forceinline__ void load12_hint(const HintP& base, size_t stride, int i,
                                            Mat3<float>& m) {
  unpack12(ldg_hint(base.p + i, base.pol), ldg_hint(base.p + stride + i, base.pol),
           ldg_hint(base.p + 2 * stride + i, base.pol), m);
}
__device__ __forceinline__ void store12_hint(float4* base, size_t stride, int i,
                                             const Mat3<float>& m, uint64_t pol) {
  stg_hint(base + i, make_float4(m.e[0][0].re, m.e[0][0].im, m.e[0][1].re, m.e[0][1].im), pol);
  stg_hint(base + stride + i,
           make_float4(m.e[0][2].re, m.e[0][2].im, m.e[1][0].re, m.e[1][0].im), pol);
  stg_hint(base + 2 * stride + i,
           make_float4(m.e[1][1].re, m.e[1][1].im, m.e[1][2].re, m.e[1][2].im), pol);
}

// loads of the FP32 star.  Scalar: one copy, 3 planes of float4 per matrix.  Pairs
// (T = f2, gfx_pair.cuh): the P12 layout, 6 planes per matrix, for the two copies' g
// and for the links held in both lanes; LaneP12 reads one copy of a pair field.
__device__ __forceinline__ void link_rows01(const float4* base, size_t stride, int i,
                                            Mat3<float>& m) {
  load12_rows01(base, stride, i, m);
}
__device__ __forceinline__ void link_full(const float4* base, size_t stride, int i,
                                          Mat3<float>& m) {
  Field<float, 12>::load(base, stride, i, m);
}
template <typename P, typename M>
__device__ __forceinline__ void g_rows01(const P& base, size_t stride, int i, M& m) {
  load12_rows01(base, stride, i, m);
}
__device__ __forceinline__ void g_full(const float4* base, size_t stride, int i, Mat3<float>& m) {
  Field<float, 12>::load(base, stride, i, m);
}
__device__ __forceinline__ void g_full(const LaneP12& base, size_t stride, int i,
                                       Mat3<float>& m) {
  load12_rows01(base, stride, i, m);
  row2_from_01(m);
}
__device__ __forceinline__ void link_rows01(const P12& base, size_t stride, int i, Mat3<f2>& m) {
  load12_rows01(base, stride, i, m);
}
__device__ __forceinline__ void link_full(const P12& base, size_t stride, int i, Mat3<f2>& m) {
  load12(base, stride, i, m);
}
__device__ __forceinline__ void g_full(const P12& base, size_t stride, int i, Mat3<f2>& m) {
  load12(base, stride, i, m);
}
__device__ __forceinline__ void link_rows01(const HintP& base, size_t stride, int i,
                                            Mat3<float>& m) {
  load12_rows01(base, stride, i, m);
}
__device__ __forceinline__ void link_full(const HintP& base, size_t stride, int i,
                                          Mat3<float>& m) {
  load12_hint(base, stride, i, m);
}
__device__ __forceinline__ void g_full(const HintP& base, size_t stride, int i, Mat3<float>& m) {
  load12_hint(base, stride, i, m);
}
template <typename P>
struct Planes {
  static constexpr int n = 3;
};
template <>
struct Planes<P12> {
  static constexpr int n = kPairPlanes;
};
template <>
struct Planes<LaneP12> {
  static constexpr int n = kPairPlanes;
};

// T = float with UP = GP = const float4* (one copy) or GP = LaneP12 (one copy of a pair
// field), or T = f2 with UP = GP = P12 (two copies of one configuration): the same
// operations lane for lane
template <typename T, typename UP, typename GP, int NDIR>
__device__ __forceinline__ void compute_star_12(const Lattice& L, const Site& c, int parity,
                                                UP U, GP G, Mat3<T>& star) {
  constexpr int NPU = Planes<UP>::n, NPG = Planes<GP>::n;
  const size_t vh = (size_t)L.vh;
  const int q = 1 - parity;
  const GP Gq = G + (size_t)q * NPG * vh;
  mzero(star);
#pragma unroll
  for (int mu = 0; mu < NDIR; mu++) {
    Mat3<T> a, b;
    cplx<T> P[2][3];
    // forward: P = U g^+
    link_rows01(U + (size_t)(parity * 4 + mu) * NPU * vh, vh, c.i, a);
    g_full(Gq, vh, nb_fwd(L, c, mu), b);
#pragma unroll
    for (int r = 0; r < 2; r++)
#pragma unroll
      for (int j = 0; j < 3; j++) {
        cplx<T> x = cmulc(a.e[r][0], b.e[j][0]);
        cmacc(x, a.e[r][1], b.e[j][1]);
        cmacc(x, a.e[r][2], b.e[j][2]);
        P[r][j] = x;
        star.e[r][j] = cadd(star.e[r][j], x);
      }
    acc_cross_conj(star.e[2][0], P[0][1], P[1][2], P[0][2], P[1][1]);
    acc_cross_conj(star.e[2][1], P[0][2], P[1][0], P[0][0], P[1][2]);
    acc_cross_conj(star.e[2][2], P[0][0], P[1][1], P[0][1], P[1][0]);
    // backward: Q = g(x-mu) U_mu(x-mu), w += Q^+
    const int jb = nb_bwd(L, c, mu);
    g_rows01(Gq, vh, jb, b);
    link_full(U + (size_t)(q * 4 + mu) * NPU * vh, vh, jb, a);
#pragma unroll
    for (int r = 0; r < 2; r++)
#pragma unroll
      for (int j = 0; j < 3; j++) {
        cplx<T> x = cmul(b.e[r][0], a.e[0][j]);
        cmac(x, b.e[r][1], a.e[1][j]);
        cmac(x, b.e[r][2], a.e[2][j]);
        P[r][j] = x;
        star.e[j][r] = cadd(star.e[j][r], cconj(x));
      }
    // (Q^+)_{j2} = conj(Q_{2j}) = (Q_0 x Q_1)_j
    acc_cross(star.e[0][2], P[0][1], P[1][2], P[0][2], P[1][1]);
    acc_cross(star.e[1][2], P[0][2], P[1][0], P[0][0], P[1][2]);
    acc_cross(star.e[2][2], P[0][0], P[1][1], P[0][1], P[1][0]);
  }
}

template <int NDIR>
__device__ __forceinline__ void compute_star_f32(const Lattice& L, const Site& c, int parity,
                                                 const float4* __restrict__ U,
                                                 const float4* __restrict__ G,
                                                 Mat3<float>& star) {
  compute_star_12<float, const float4*, const float4*, NDIR>(L, c, parity, U, G, star);
}

// One overrelaxation site update (overrelax.cu:335-446) of site i of parity `parity`
// in place: FP64 in the reference's operation order; FP32 and double-float with the
// reduced forms.
template <typename T, int NRU, int NDIR>
__device__ __forceinline__ void or_site_update(const Lattice& L, const Site& c, int parity,
                                               const typename VecOf<T>::type* __restrict__ U,
                                               typename VecOf<T>::type* __restrict__ G, int i,
                                               T omega) {
  constexpr int NCG = Field<T, 12>::NCHUNK;
  const size_t vh = (size_t)L.vh;
  typename VecOf<T>::type* Gp = G + (size_t)parity * NCG * vh;
  Mat3<T> star, gold, gn;
  if constexpr (sizeof(T) == 4 && NRU == 12)
    compute_star_f32<NDIR>(L, c, parity, U, G, star);
  else
    compute_star<T, T, NRU, T, 12, NDIR>(L, c, parity, U, G, star);
  Field<T, 12>::load(Gp, vh, i, gold);
  if constexpr (!std::is_same<T, double>::value) {
    or_update_composed(gold, star, omega, gn);  // FP32 and double-float
  } else {
    Mat3<T> g = gold;
    cm_relax(g, star);
    normalize<T, true>(g);
    overrelax_rows01(gn, gold, g, omega);
  }
  Field<T, 12>::store(Gp, vh, i, gn);
}

// The FP32 12-real update with L2 eviction priorities (staging modes 3 and 4): g read
// and written as evict_last, so the 48 MB of a 32^4 g can stay in L2 while the links
// stream; the links as evict_first (LINKS_FIRST) or with the default priority.  The
// operations are those of or_site_update<float, 12, NDIR>.
template <int NDIR, bool LINKS_FIRST>
__device__ __forceinline__ void or_site_update_hint(const Lattice& L, const Site& c, int parity,
                                                    const float4* U, float4* G, int i,
                                                    float omega) {
  const size_t vh = (size_t)L.vh;
  const uint64_t pg = l2_policy_evict_last();
  const HintP Gh{G, pg};
  Mat3<float> star, gold, gn;
  if constexpr (LINKS_FIRST)
    compute_star_12<float, HintP, HintP, NDIR>(L, c, parity, HintP{U, l2_policy_evict_first()},
                                               Gh, star);
  else
    compute_star_12<float, const float4*, HintP, NDIR>(L, c, parity, U, Gh, star);
  float4* Gp = G + (size_t)parity * 3 * vh;
  load12_hint(HintP{Gp, pg}, vh, i, gold);
  or_update_composed(gold, star, omega, gn);
  store12_hint(Gp, vh, i, gn, pg);
}

// The FP32 update of site i for two copies of one configuration at once (T = f2):
// lane for lane the operations of or_site_update<float, 12, NDIR>.  U: the links in
// both lanes, G: the pair's g, both in the P12 layout.  A lane whose copy has stopped
// (run_x / run_y false) is computed but its stored bits are written back unchanged.
template <int NDIR>
__device__ __forceinline__ void or_site_update_pair(const Lattice& L, const Site& c, int parity,
                                                    P12 U, P12 G, int i, float omega, bool run_x,
                                                    bool run_y) {
  const size_t vh = (size_t)L.vh;
  Mat3<f2> star, gold, gn;
  compute_star_12<f2, P12, P12, NDIR>(L, c, parity, U, G, star);
  const P12 Gp = G + (size_t)parity * kPairPlanes * vh;
  load12(Gp, vh, i, gold);
  or_update_composed(gold, star, f2(omega), gn);
  store12(Gp, vh, i, gn, gold, !run_x, !run_y);
}

// Per-site functional from X = g w (overrelax.cu:451-605, see measure_kernel):
// f = Re tr X, d = tr[Delta Delta^+] = sum_ij |AH(X)_ij|^2.
template <typename TC>
__device__ __forceinline__ void site_functional(const Mat3<TC>& g, const Mat3<TC>& star,
                                                double& f, double& d) {
  Mat3<TC> X;
  mul(X, g, star);
  f = (double)X.e[0][0].re + (double)X.e[1][1].re + (double)X.e[2][2].re;
  const TC tim = (X.e[0][0].im + X.e[1][1].im + X.e[2][2].im) * TC(1.0 / 3.0);
  TC acc = TC(0);
#pragma unroll
  for (int a = 0; a < 3; a++) {
    const TC di = X.e[a][a].im - tim;
    acc += di * di;
  }
  TC off = TC(0);
#pragma unroll
  for (int a = 0; a < 3; a++)
#pragma unroll
    for (int b = a + 1; b < 3; b++) {
      const TC re = (X.e[a][b].re - X.e[b][a].re) * TC(0.5);
      const TC im = (X.e[a][b].im + X.e[b][a].im) * TC(0.5);
      off += re * re + im * im;
    }
  d = (double)acc + 2.0 * (double)off;
}

// FP64 sums of f and d and max of m over the block, in a fixed order
__device__ __forceinline__ void block_reduce3(double f, double d, double m, double* out) {
  __shared__ double sh[3][32];
  f = warp_sum(f);
  d = warp_sum(d);
  m = warp_max(m);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) {
    sh[0][w] = f;
    sh[1][w] = d;
    sh[2][w] = m;
  }
  __syncthreads();
  if (w == 0) {
    const int nw = blockDim.x >> 5;
    f = l < nw ? sh[0][l] : 0.0;
    d = l < nw ? sh[1][l] : 0.0;
    m = l < nw ? sh[2][l] : 0.0;
    f = warp_sum(f);
    d = warp_sum(d);
    m = warp_max(m);
    if (l == 0) {
      out[0] = f;
      out[1] = d;
      out[2] = m;
    }
  }
}

// The FP32 checks' per-site values in FP32: GB300 runs FP64 at a small fraction of its
// FP32 rate, and the FP64 conversions and shuffles of the general path cost a check on
// the FP32 links about as much as a sweep.  The sums over the 32 sites of a warp are
// FP32 (relative rounding ~3e-7, well inside what the FP32 phase's plateau test
// resolves); every sum above the warp -- warps of a block, blocks, slices -- is FP64.
__device__ __forceinline__ void site_functional_f32(const Mat3<float>& g, const Mat3<float>& star,
                                                    float& f, float& d) {
  Mat3<float> X;
  mul(X, g, star);
  f = X.e[0][0].re + X.e[1][1].re + X.e[2][2].re;
  const float tim = (X.e[0][0].im + X.e[1][1].im + X.e[2][2].im) * (1.0f / 3.0f);
  float acc = 0.0f;
#pragma unroll
  for (int a = 0; a < 3; a++) {
    const float di = X.e[a][a].im - tim;
    acc = fm(di, di, acc);
  }
  float off = 0.0f;
#pragma unroll
  for (int a = 0; a < 3; a++)
#pragma unroll
    for (int b = a + 1; b < 3; b++) {
      const float re = (X.e[a][b].re - X.e[b][a].re) * 0.5f;
      const float im = (X.e[a][b].im + X.e[b][a].im) * 0.5f;
      off = fm(im, im, fm(re, re, off));
    }
  d = fm(2.0f, off, acc);
}

// block sums of the FP32 per-site values: FP32 within each warp (fixed butterfly),
// FP64 across the warps in the order of block_reduce3; the max in FP32 (exact)
__device__ __forceinline__ void block_reduce3_f32(float f, float d, double* out) {
  __shared__ double sh[3][32];
  float m = d;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    f += __shfl_xor_sync(0xffffffffu, f, o);
    d += __shfl_xor_sync(0xffffffffu, d, o);
    m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
  }
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) {
    sh[0][w] = (double)f;
    sh[1][w] = (double)d;
    sh[2][w] = (double)m;
  }
  __syncthreads();
  if (w == 0) {
    const int nw = blockDim.x >> 5;
    double fs = l < nw ? sh[0][l] : 0.0;
    double ds = l < nw ? sh[1][l] : 0.0;
    double ms = l < nw ? sh[2][l] : 0.0;
    fs = warp_sum(fs);
    ds = warp_sum(ds);
    ms = warp_max(ms);
    if (l == 0) {
      out[0] = fs;
      out[1] = ds;
      out[2] = ms;
    }
  }
}

enum { CRIT_MAXDADA = 0, CRIT_THETA = 1, CRIT_THETA_SLICES = 2 };

// Totals over the slices, then (when loop is given) one check of the convergence loop:
// record, compare with the criterion, decide done (0 run on, 1 converged, 2 leave the
// FP32 phase, 3 iteration cap, 4 shorter check interval, 5 renew the rebased base).  Called by all threads of one block; returns done on
// thread 0 (and -1 elsewhere).
__device__ __forceinline__ int reduce_and_check(const double* slice_sums, int lt, double vol,
                                                double v3, int ndir, Reduced* out,
                                                LoopState* loop, CheckRecord* hist,
                                                int advance) {
  double f = 0.0, d = 0.0, m = 0.0, tmax = 0.0;
  for (int t = threadIdx.x; t < lt; t += blockDim.x) {
    f += slice_sums[3 * t];
    d += slice_sums[3 * t + 1];
    m = fmax(m, slice_sums[3 * t + 2]);
    tmax = fmax(tmax, slice_sums[3 * t + 1] / (3.0 * v3));
  }
  // one warp suffices for lt <= 32*k; reduce in a fixed order
  __shared__ double sh[4][32];
  f = warp_sum(f);
  d = warp_sum(d);
  m = warp_max(m);
  tmax = warp_max(tmax);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) {
    sh[0][w] = f;
    sh[1][w] = d;
    sh[2][w] = m;
    sh[3][w] = tmax;
  }
  __syncthreads();
  if (threadIdx.x != 0) return -1;
  f = d = m = tmax = 0.0;
  for (int k = 0; k < (int)(blockDim.x >> 5); k++) {
    f += sh[0][k];
    d += sh[1][k];
    m = fmax(m, sh[2][k]);
    tmax = fmax(tmax, sh[3][k]);
  }
  Reduced r;
  r.F = f / (2.0 * ndir * vol);
  r.dAdA = d / vol;
  r.maxdAdA = m;
  r.theta = r.dAdA / 3.0;
  r.theta_slice_max = tmax;
  *out = r;
  if (!loop) return 0;
  LoopState& S = *loop;
  S.iter += advance;
  const double value = S.criterion == CRIT_MAXDADA ? r.maxdAdA
                       : S.criterion == CRIT_THETA ? r.theta
                                                   : r.theta_slice_max;
  if (S.nhist < S.hist_cap && hist) {
    CheckRecord& h = hist[S.nhist];
    h.iter = S.iter;
    h.phase = S.phase;
    h.F = r.F;
    h.dAdA = r.dAdA;
    h.maxdAdA = r.maxdAdA;
    h.theta = r.theta;
    h.theta_slice_max = r.theta_slice_max;
  }
  S.nhist++;
  S.last_F = r.F;
  S.last_dAdA = r.dAdA;
  S.last_max = r.maxdAdA;
  S.last_theta = r.theta;
  S.last_theta_slice_max = r.theta_slice_max;
  int done = 0;
  if (S.phase == 0) {
    // single-precision phase: hand over to the double-precision phase when the target
    // is reached (the FP64 phase verifies it), or when, below switch_eps, the value
    // stops decreasing -- the FP32 rounding floor, which a few FP64 sweeps remove
    // (the plateau threshold corresponds to the same decrease per sweep on either
    // check interval)
    const double plateau = S.ck_near > 0 && S.ck == S.ck_near ? S.plateau_near : S.plateau_ratio;
    if (value < S.eps || (value < S.switch_eps && S.prev > 0.0 && value > plateau * S.prev))
      done = 2;
  } else if (value < S.eps) {
    done = 1;
  }
  // close to the end: shorter intervals cut the sweeps run past convergence (or past
  // the FP32 floor) while the long interval keeps the checks cheap before that
  if (!done && S.ck_near > 0 && S.ck > S.ck_near && value < S.switch_eps) done = 4;
  if (!done && S.iter + S.ck >= S.maxit) done = 3;
  if (!done && S.rebase_at > 0 && S.iter >= S.rebase_at) done = 5;
  S.prev = value;
  S.done = done;
  return done;
}


}  // namespace gfx
