// gfx_rebased.cuh -- device code of the rebased FP32 sweeps, shared by the
// single-lattice kernels (gfx_rebased.cu) and the batched ones (gfx_batch.cu).
//
// The gauge transformation is written g(x) = (1 + a(x)) g_c(x): g_c is a fixed FP64
// field (the base) and a is small and held in FP32.  With the rebased links
//   U'_mu(x) = g_c(x) U_mu(x) g_c(x+mu)^+
// the matrix the update and the functional are built from is
//   X(x) = g(x) w(x) = (1 + a(x)) [ w0(x) + C(x) ],
//   w0(x) = sum_mu U'_mu(x) + U'_mu(x-mu)^+                       (fixed with the base)
//   C(x)  = sum_mu U'_mu(x) a(x+mu)^+ + [a(x-mu) U'_mu(x-mu)]^+    (proportional to a)
// and g_new = (1 + a_new) g_c, because the overrelaxation step acts on g from the
// left and its reunitarization commutes with right-multiplication by g_c.
// Every term that changes from sweep to sweep is proportional to a, so FP32 errs on
// it by about 1e-7 |a| in absolute terms.  w0 is formed once per base in FP64 and
// kept as its FP32 value plus the FP32 remainder of its anti-hermitian part (the part
// that the subgroup elements and theta need to full accuracy) and of its real trace.
// The subgroup elements, R = S - 1, the step a + T (1 + a) and the reunitarization
// are evaluated on the small quantities (p - 1, q, R, a) directly, never as a
// difference against 1.  Near convergence |a| stays far below 1e-3, so these sweeps
// follow the FP64 iteration to about 1e-12 and share its fixed point, while every
// operation runs on the FP32 units (64 times the FP64 rate on GB300).  The base is
// renewed (g_c <- (1 + a) g_c in FP64, a <- 0) at the start of each polish and every
// 1000 polish sweeps.
#pragma once

#include "gfx_common.cuh"

namespace gfx {

// w0 per site: 7 float4 planes = 28 floats:
//   0..17  FP32 value of w0, row-major (re, im)
//   18..20 Im of the diagonal of AH(lo), lo = w0 - hi      (AH(M) = (M - M^+)/2)
//   21..26 AH(lo)_01, AH(lo)_02, AH(lo)_12                  (re, im); AH(lo)_ba = -conj(AH(lo)_ab)
//   27     Re tr lo
constexpr int kW0Planes = 7;

// row 2 of a = g_hat - 1 for g_hat = 1 + a in SU(3): g_hat_2 = conj(g_hat_0 x g_hat_1),
// and (e0 + a0) x (e1 + a1) = e2 + (-a02, -a12, a00 + a11) + a0 x a1
__device__ __forceinline__ void small_row2(Mat3<float>& a) {
  a.e[2][0] = cadd(cross_conj(a.e[0][1], a.e[1][2], a.e[0][2], a.e[1][1]), cmk(-a.e[0][2].re, a.e[0][2].im));
  a.e[2][1] = cadd(cross_conj(a.e[0][2], a.e[1][0], a.e[0][0], a.e[1][2]), cmk(-a.e[1][2].re, a.e[1][2].im));
  a.e[2][2] = cadd(cross_conj(a.e[0][0], a.e[1][1], a.e[0][1], a.e[1][0]),
                   cconj(cadd(a.e[0][0], a.e[1][1])));
}

__device__ __forceinline__ void load_w0(const float4* __restrict__ W, size_t vh, int i,
                                        Mat3<float>& hi, Mat3<float>& lo, float& trlo) {
  float f[28];
#pragma unroll
  for (int p = 0; p < kW0Planes; p++) {
    const float4 v = __ldg(W + p * vh + i);
    f[4 * p] = v.x, f[4 * p + 1] = v.y, f[4 * p + 2] = v.z, f[4 * p + 3] = v.w;
  }
#pragma unroll
  for (int r = 0; r < 3; r++)
#pragma unroll
    for (int k = 0; k < 3; k++) hi.e[r][k] = cmk(f[2 * (3 * r + k)], f[2 * (3 * r + k) + 1]);
  lo.e[0][0] = cmk(0.f, f[18]);
  lo.e[1][1] = cmk(0.f, f[19]);
  lo.e[2][2] = cmk(0.f, f[20]);
  lo.e[0][1] = cmk(f[21], f[22]);
  lo.e[1][0] = cmk(-f[21], f[22]);
  lo.e[0][2] = cmk(f[23], f[24]);
  lo.e[2][0] = cmk(-f[23], f[24]);
  lo.e[1][2] = cmk(f[25], f[26]);
  lo.e[2][1] = cmk(-f[25], f[26]);
  trlo = f[27];
}

// X(x) = Xh + Xd = (1 + a(x)) (w0(x) + C(x)); a is a(x), rows 0..2
template <int NDIR>
__device__ __forceinline__ void rebased_x(const Lattice& L, const Site& c, int parity,
                                          const float4* __restrict__ Ur,
                                          const float4* __restrict__ W0,
                                          const float4* __restrict__ A, Mat3<float>& Xh,
                                          Mat3<float>& Xd, Mat3<float>& a, float& trlo) {
  const size_t vh = (size_t)L.vh;
  const int q = 1 - parity;
  const float4* Aq = A + (size_t)q * 3 * vh;
  Mat3<float> W;  // AH(lo) + C: small
  load_w0(W0 + (size_t)parity * kW0Planes * vh, vh, c.i, Xh, W, trlo);
#pragma unroll
  for (int mu = 0; mu < NDIR; mu++) {
    Mat3<float> u, b;
    cplx<float> P[2][3], v[3];
    // forward: P = U'_mu(x) a(x+mu)^+, rows 0,1 directly; row 2 from
    // (U' g_hat^+)_2 = conj((U'_0 + P_0) x (U'_1 + P_1)) minus U'_2 = conj(U'_0 x U'_1)
    load12_rows01(Ur + (size_t)(parity * 4 + mu) * 3 * vh, vh, c.i, u);
    load12_rows01(Aq, vh, nb_fwd(L, c, mu), b);
    small_row2(b);
#pragma unroll
    for (int r = 0; r < 2; r++)
#pragma unroll
      for (int j = 0; j < 3; j++) {
        cplx<float> x = cmulc(u.e[r][0], b.e[j][0]);
        cmacc(x, u.e[r][1], b.e[j][1]);
        cmacc(x, u.e[r][2], b.e[j][2]);
        P[r][j] = x;
        W.e[r][j] = cadd(W.e[r][j], x);
      }
#pragma unroll
    for (int j = 0; j < 3; j++) v[j] = cadd(u.e[1][j], P[1][j]);
    acc_cross_conj(W.e[2][0], u.e[0][1], P[1][2], u.e[0][2], P[1][1]);
    acc_cross_conj(W.e[2][0], P[0][1], v[2], P[0][2], v[1]);
    acc_cross_conj(W.e[2][1], u.e[0][2], P[1][0], u.e[0][0], P[1][2]);
    acc_cross_conj(W.e[2][1], P[0][2], v[0], P[0][0], v[2]);
    acc_cross_conj(W.e[2][2], u.e[0][0], P[1][1], u.e[0][1], P[1][0]);
    acc_cross_conj(W.e[2][2], P[0][0], v[1], P[0][1], v[0]);
    // backward: Q = a(x-mu) U'_mu(x-mu), W += Q^+; row 2 of Q by the same identity
    const int jb = nb_bwd(L, c, mu);
    load12_rows01(Aq, vh, jb, b);
    Field<float, 12>::load(Ur + (size_t)(q * 4 + mu) * 3 * vh, vh, jb, u);
#pragma unroll
    for (int r = 0; r < 2; r++)
#pragma unroll
      for (int j = 0; j < 3; j++) {
        cplx<float> x = cmul(b.e[r][0], u.e[0][j]);
        cmac(x, b.e[r][1], u.e[1][j]);
        cmac(x, b.e[r][2], u.e[2][j]);
        P[r][j] = x;
        W.e[j][r] = cadd(W.e[j][r], cconj(x));
      }
#pragma unroll
    for (int j = 0; j < 3; j++) v[j] = cadd(u.e[1][j], P[1][j]);
    // (Q^+)_{j2} = conj(Q_2j) = (U'_0 x Q_1 + Q_0 x (U'_1 + Q_1))_j
    acc_cross(W.e[0][2], u.e[0][1], P[1][2], u.e[0][2], P[1][1]);
    acc_cross(W.e[0][2], P[0][1], v[2], P[0][2], v[1]);
    acc_cross(W.e[1][2], u.e[0][2], P[1][0], u.e[0][0], P[1][2]);
    acc_cross(W.e[1][2], P[0][2], v[0], P[0][0], v[2]);
    acc_cross(W.e[2][2], u.e[0][0], P[1][1], u.e[0][1], P[1][0]);
    acc_cross(W.e[2][2], P[0][0], v[1], P[0][1], v[0]);
  }
  load12_rows01(A + (size_t)parity * 3 * vh, vh, c.i, a);
  small_row2(a);
  // Xd = W + a (Xh + W)
#pragma unroll
  for (int r = 0; r < 3; r++)
#pragma unroll
    for (int j = 0; j < 3; j++) {
      cplx<float> x = W.e[r][j];
#pragma unroll
      for (int k = 0; k < 3; k++) cmac(x, a.e[r][k], cadd(Xh.e[k][j], W.e[k][j]));
      Xd.e[r][j] = x;
    }
}

struct HD {
  cplx<float> h, d;  // the value h + d; h is an entry of w0's FP32 value
};
__device__ __forceinline__ HD hd(const Mat3<float>& Xh, const Mat3<float>& Xd, int r, int k) {
  HD v;
  v.h = Xh.e[r][k];
  v.d = Xd.e[r][k];
  return v;
}
__device__ __forceinline__ cplx<float> hd_full(const HD& x) { return cadd(x.h, x.d); }
// p x + q y with p = 1 + dp
__device__ __forceinline__ HD hd_high(cplx<float> dp, cplx<float> q, const HD& x, const HD& y) {
  HD o = x;
  cmac(o.d, dp, hd_full(x));
  cmac(o.d, q, hd_full(y));
  return o;
}
// -conj(q) x + conj(p) y
__device__ __forceinline__ HD hd_low(cplx<float> dp, cplx<float> q, const HD& x, const HD& y) {
  HD o = y;
  cmac(o.d, cmk(-q.re, q.im), hd_full(x));
  cmac(o.d, cconj(dp), hd_full(y));
  return o;
}

// the subgroup element of su2_pq as (p - 1, q): p - 1 = (w0 - n + i w3) / n with
// w0 - n = -(w1^2 + w2^2 + w3^2) / (w0 + n), free of cancellation for w0 > 0
__device__ __forceinline__ void su2_small(const HD& xaa, const HD& xbb, const HD& xab,
                                          const HD& xba, cplx<float>& dp, cplx<float>& q) {
  const float w0 = (xaa.h.re + xbb.h.re) + (xaa.d.re + xbb.d.re);
  const float w3 = (xbb.h.im - xaa.h.im) + (xbb.d.im - xaa.d.im);
  const float w1 = -(xab.h.im + xba.h.im) - (xab.d.im + xba.d.im);
  const float w2 = (xba.h.re - xab.h.re) + (xba.d.re - xab.d.re);
  const float s2 = fm(w3, w3, fm(w2, w2, w1 * w1));
  const float n2 = fm(w0, w0, s2);
  const float r = rsqrtf(n2);
  const float n = n2 * r;
  dp = cmk(w0 > 0.f ? __fdividef(-s2 * r, w0 + n) : fm(w0, r, -1.f), w3 * r);
  q = cmk(w2 * r, w1 * r);
}

// 1/sqrt(1 + s) - 1 = -s y^2 / (1 + y), y = 1/sqrt(1 + s)
__device__ __forceinline__ float rsqrt1p_m1(float s) {
  const float y = rsqrtf(1.f + s);
  return __fdividef(-s * y * y, 1.f + y);
}

// one overrelaxation step on a: rows 0,1 of the new a, from X = Xh + Xd
__device__ __forceinline__ void or_update_small(const Mat3<float>& Xh, const Mat3<float>& Xd,
                                                const Mat3<float>& a, float omega,
                                                Mat3<float>& b) {
  cplx<float> dp1, q1, dp2, q2, dp3, q3;
  su2_small(hd(Xh, Xd, 0, 0), hd(Xh, Xd, 1, 1), hd(Xh, Xd, 0, 1), hd(Xh, Xd, 1, 0), dp1, q1);
  const HD x00 = hd_high(dp1, q1, hd(Xh, Xd, 0, 0), hd(Xh, Xd, 1, 0));
  const HD x01 = hd_high(dp1, q1, hd(Xh, Xd, 0, 1), hd(Xh, Xd, 1, 1));
  const HD x02 = hd_high(dp1, q1, hd(Xh, Xd, 0, 2), hd(Xh, Xd, 1, 2));
  const HD x11 = hd_low(dp1, q1, hd(Xh, Xd, 0, 1), hd(Xh, Xd, 1, 1));
  const HD x12 = hd_low(dp1, q1, hd(Xh, Xd, 0, 2), hd(Xh, Xd, 1, 2));
  su2_small(x00, hd(Xh, Xd, 2, 2), x02, hd(Xh, Xd, 2, 0), dp2, q2);
  const HD y21 = hd_low(dp2, q2, x01, hd(Xh, Xd, 2, 1));
  const HD y22 = hd_low(dp2, q2, x02, hd(Xh, Xd, 2, 2));
  su2_small(x11, y22, x12, y21, dp3, q3);
  // R = S3 S2 S1 - 1 (or_update_composed's S) from the small parameters
  const cplx<float> one = cmk(1.f, 0.f);
  const cplx<float> p1 = cadd(one, dp1), p2 = cadd(one, dp2), p3 = cadd(one, dp3);
  const cplx<float> q1c = cconj(q1), q2c = cconj(q2), q3c = cconj(q3);
  const cplx<float> t0 = cmul(q2c, p1), t1 = cmul(q2c, q1);
  Mat3<float> R;
  R.e[0][0] = cadd(cadd(dp2, dp1), cmul(dp2, dp1));
  R.e[0][1] = cmul(p2, q1);
  R.e[0][2] = q2;
  R.e[1][0] = cmk(0.f, 0.f);
  cmac(R.e[1][0], p3, q1c);
  cmac(R.e[1][0], q3, t0);
  R.e[1][0] = cmk(-R.e[1][0].re, -R.e[1][0].im);
  R.e[1][1] = csub(cadd(cadd(dp3, cconj(dp1)), cmul(dp3, cconj(dp1))), cmul(q3, t1));
  R.e[1][2] = cmul(q3, cconj(p2));
  R.e[2][0] = csub(cmul(q3c, q1c), cmul(cconj(p3), t0));
  R.e[2][1] = cmk(0.f, 0.f);
  cmac(R.e[2][1], q3c, cconj(p1));
  cmac(R.e[2][1], cconj(p3), t1);
  R.e[2][1] = cmk(-R.e[2][1].re, -R.e[2][1].im);
  R.e[2][2] = cadd(cadd(cconj(dp3), cconj(dp2)), cmul(cconj(dp3), cconj(dp2)));
  // T = w R + c2 R^2 and b = a + T (1 + a), rows 0,1
  const float c2 = omega * (omega - 1.f) * 0.5f;
#pragma unroll
  for (int r = 0; r < 2; r++) {
    cplx<float> T[3];
#pragma unroll
    for (int j = 0; j < 3; j++) {
      const cplx<float> r2 = mul_entry(R, R, r, j);
      T[j] = cmk(fm(omega, R.e[r][j].re, c2 * r2.re), fm(omega, R.e[r][j].im, c2 * r2.im));
    }
#pragma unroll
    for (int j = 0; j < 3; j++) {
      cplx<float> o = cadd(a.e[r][j], T[j]);
#pragma unroll
      for (int k = 0; k < 3; k++) cmac(o, T[k], a.e[k][j]);
      b.e[r][j] = o;
    }
  }
  // Gram-Schmidt on the rows of 1 + b, in terms of b
  float t = rsqrt1p_m1(fm(2.f, b.e[0][0].re, row_norm2<float>(b.e[0])));
#pragma unroll
  for (int k = 0; k < 3; k++) b.e[0][k] = cmk(fm(t, b.e[0][k].re, b.e[0][k].re), fm(t, b.e[0][k].im, b.e[0][k].im));
  b.e[0][0].re += t;
  cplx<float> proj = cadd(b.e[1][0], cconj(b.e[0][1]));  // conj(row0) . row1
#pragma unroll
  for (int k = 0; k < 3; k++) cmacc(proj, b.e[1][k], b.e[0][k]);
  b.e[1][0] = csub(b.e[1][0], proj);
#pragma unroll
  for (int k = 0; k < 3; k++) {
    const cplx<float> x = cmul(proj, b.e[0][k]);
    b.e[1][k] = csub(b.e[1][k], x);
  }
  t = rsqrt1p_m1(fm(2.f, b.e[1][1].re, row_norm2<float>(b.e[1])));
#pragma unroll
  for (int k = 0; k < 3; k++) b.e[1][k] = cmk(fm(t, b.e[1][k].re, b.e[1][k].re), fm(t, b.e[1][k].im, b.e[1][k].im));
  b.e[1][1].re += t;
}

// One overrelaxation site update of a at site c (parity `parity`): the body of
// or_rebased_kernel and of the batched kernel, which share it so that a batched copy
// stays bit-identical to its single-lattice solve
template <int NDIR>
__device__ __forceinline__ void rebased_site_update(const Lattice& L, const Site& c, int parity,
                                                    const float4* __restrict__ Ur,
                                                    const float4* __restrict__ W0,
                                                    float4* __restrict__ A, float omega) {
  Mat3<float> Xh, Xd, a, b;
  float trlo;
  rebased_x<NDIR>(L, c, parity, Ur, W0, A, Xh, Xd, a, trlo);
  or_update_small(Xh, Xd, a, omega, b);
  Field<float, 12>::store(A + (size_t)parity * 3 * L.vh, (size_t)L.vh, c.i, b);
}

// functional and theta terms of site c (site_functional on X = Xh + Xd): the
// anti-hermitian combinations are formed on the FP32 value and the small part apart
template <int NDIR>
__device__ __forceinline__ void rebased_site_functional(const Lattice& L, const Site& c,
                                                        int parity, const float4* __restrict__ Ur,
                                                        const float4* __restrict__ W0,
                                                        const float4* __restrict__ A, double& f,
                                                        double& d) {
  Mat3<float> Xh, Xd, a;
  float trlo;
  rebased_x<NDIR>(L, c, parity, Ur, W0, A, Xh, Xd, a, trlo);
  f = (double)Xh.e[0][0].re + (double)Xh.e[1][1].re + (double)Xh.e[2][2].re + (double)trlo +
      (double)(Xd.e[0][0].re + Xd.e[1][1].re + Xd.e[2][2].re);
  const float tim = ((Xh.e[0][0].im + Xh.e[1][1].im + Xh.e[2][2].im) +
                     (Xd.e[0][0].im + Xd.e[1][1].im + Xd.e[2][2].im)) * (1.f / 3.f);
  float acc = 0.f, off = 0.f;
#pragma unroll
  for (int m = 0; m < 3; m++) {
    const float di = (Xh.e[m][m].im + Xd.e[m][m].im) - tim;
    acc = fm(di, di, acc);
  }
#pragma unroll
  for (int m = 0; m < 3; m++)
#pragma unroll
    for (int n = m + 1; n < 3; n++) {
      const float re = ((Xh.e[m][n].re - Xh.e[n][m].re) + (Xd.e[m][n].re - Xd.e[n][m].re)) * 0.5f;
      const float im = ((Xh.e[m][n].im + Xh.e[n][m].im) + (Xd.e[m][n].im + Xd.e[n][m].im)) * 0.5f;
      off = fm(re, re, fm(im, im, off));
    }
  d = (double)acc + 2.0 * (double)off;
}

}  // namespace gfx
