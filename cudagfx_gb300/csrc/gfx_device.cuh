// gfx_device.cuh -- device-side building blocks for the sm_103a gauge-fixing kernels.
//
//  * SU(3) algebra on register-resident 3x3 complex matrices, templated on the
//    arithmetic type (float for the bulk sweeps, double for the polish sweeps and
//    the reference-precision path).  The update formulas follow the reference's
//    device library (dev_su3.cu:1321-1634) and overrelax.cu:149-269.
//  * Even/odd structure-of-arrays field layout (see Field below).
//  * Site <-> coordinate arithmetic for the checkerboard index, with neighbours
//    computed on the fly instead of the reference's gathered nn[] table
//    (cudagaugefix.cu:72-196).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "gfx_df.cuh"

namespace gfx {

// ---------------------------------------------------------------------------
// complex / matrix types
// ---------------------------------------------------------------------------
template <typename T>
struct cplx {
  T re, im;
};

template <typename T>
struct Mat3 {
  cplx<T> e[3][3];
};

template <typename T>
__device__ __forceinline__ cplx<T> cmk(T re, T im) {
  cplx<T> r;
  r.re = re;
  r.im = im;
  return r;
}
// a*b + c with a single rounding: the algebra below is written as explicit FMA
// chains (a complex multiply-accumulate is four FMAs), which halves the FP32/FP64
// instruction count compared to separately rounded products and sums.
template <typename T>
__device__ __forceinline__ T fm(T a, T b, T c);
template <>
__device__ __forceinline__ float fm<float>(float a, float b, float c) {
  return __fmaf_rn(a, b, c);
}
template <>
__device__ __forceinline__ double fm<double>(double a, double b, double c) {
  return __fma_rn(a, b, c);
}
template <>
__device__ __forceinline__ dfl fm<dfl>(dfl a, dfl b, dfl c) {
  return df_fma(a, b, c);
}

template <typename T>
__device__ __forceinline__ cplx<T> cmul(cplx<T> a, cplx<T> b) {
  return cmk<T>(fm(a.re, b.re, -a.im * b.im), fm(a.re, b.im, a.im * b.re));
}
// a * conj(b)
template <typename T>
__device__ __forceinline__ cplx<T> cmulc(cplx<T> a, cplx<T> b) {
  return cmk<T>(fm(a.re, b.re, a.im * b.im), fm(a.im, b.re, -a.re * b.im));
}
// acc += a * b
template <typename T>
__device__ __forceinline__ void cmac(cplx<T>& acc, cplx<T> a, cplx<T> b) {
  acc.re = fm(-a.im, b.im, fm(a.re, b.re, acc.re));
  acc.im = fm(a.im, b.re, fm(a.re, b.im, acc.im));
}
// acc += a * conj(b)
template <typename T>
__device__ __forceinline__ void cmacc(cplx<T>& acc, cplx<T> a, cplx<T> b) {
  acc.re = fm(a.im, b.im, fm(a.re, b.re, acc.re));
  acc.im = fm(-a.re, b.im, fm(a.im, b.re, acc.im));
}
// acc += conj(a * b)
template <typename T>
__device__ __forceinline__ void cmac_conj(cplx<T>& acc, cplx<T> a, cplx<T> b) {
  acc.re = fm(-a.im, b.im, fm(a.re, b.re, acc.re));
  acc.im = fm(-a.im, b.re, fm(-a.re, b.im, acc.im));
}
template <typename T>
__device__ __forceinline__ cplx<T> cadd(cplx<T> a, cplx<T> b) {
  return cmk<T>(a.re + b.re, a.im + b.im);
}
template <typename T>
__device__ __forceinline__ cplx<T> csub(cplx<T> a, cplx<T> b) {
  return cmk<T>(a.re - b.re, a.im - b.im);
}
template <typename T>
__device__ __forceinline__ cplx<T> cconj(cplx<T> a) {
  return cmk<T>(a.re, -a.im);
}

template <typename T>
__device__ __forceinline__ T rsqrt_t(T x);
template <>
__device__ __forceinline__ float rsqrt_t<float>(float x) {
  return rsqrtf(x);
}
template <>
__device__ __forceinline__ double rsqrt_t<double>(double x) {
  return rsqrt(x);
}
template <>
__device__ __forceinline__ dfl rsqrt_t<dfl>(dfl x) {
  return df_rsqrt(x);
}

template <typename T>
__device__ __forceinline__ void mzero(Mat3<T>& m) {
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++) m.e[i][j] = cmk<T>(T(0), T(0));
}

// conj(p q - r s), one entry of the cross product row
template <typename T>
__device__ __forceinline__ cplx<T> cross_conj(cplx<T> p, cplx<T> q, cplx<T> r, cplx<T> s) {
  const T re = fm(p.re, q.re, fm(-p.im, q.im, fm(-r.re, s.re, r.im * s.im)));
  const T im = fm(-p.re, q.im, fm(-p.im, q.re, fm(r.re, s.im, r.im * s.re)));
  return cmk<T>(re, im);
}

// row 2 = conj(row0 x row1): the 12-real reconstruction (dev_su3.cu:288-305)
template <typename T>
__device__ __forceinline__ void row2_from_01(Mat3<T>& g) {
  g.e[2][0] = cross_conj(g.e[0][1], g.e[1][2], g.e[0][2], g.e[1][1]);
  g.e[2][1] = cross_conj(g.e[0][2], g.e[1][0], g.e[0][0], g.e[1][2]);
  g.e[2][2] = cross_conj(g.e[0][0], g.e[1][1], g.e[0][1], g.e[1][0]);
}

// s += a * b
template <typename T>
__device__ __forceinline__ void addmul(Mat3<T>& s, const Mat3<T>& a, const Mat3<T>& b) {
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++)
#pragma unroll
      for (int k = 0; k < 3; k++) cmac(s.e[i][j], a.e[i][k], b.e[k][j]);
}

// s += a * b^+
template <typename T>
__device__ __forceinline__ void addmul_nd(Mat3<T>& s, const Mat3<T>& a, const Mat3<T>& b) {
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++)
#pragma unroll
      for (int k = 0; k < 3; k++) cmacc(s.e[i][j], a.e[i][k], b.e[j][k]);
}

// s += a^+ b^+ = (b a)^+ ; the backward star term U^+(x-mu) g^+(x-mu)
template <typename T>
__device__ __forceinline__ void addmul_dd(Mat3<T>& s, const Mat3<T>& a, const Mat3<T>& b) {
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++)
#pragma unroll
      for (int k = 0; k < 3; k++) cmac_conj(s.e[i][j], a.e[k][i], b.e[j][k]);
}

// (a*b)_ij for one entry
template <typename T>
__device__ __forceinline__ cplx<T> mul_entry(const Mat3<T>& a, const Mat3<T>& b, int i, int j) {
  cplx<T> r = cmul(a.e[i][0], b.e[0][j]);
  cmac(r, a.e[i][1], b.e[1][j]);
  cmac(r, a.e[i][2], b.e[2][j]);
  return r;
}

// r = a * b
template <typename T>
__device__ __forceinline__ void mul(Mat3<T>& r, const Mat3<T>& a, const Mat3<T>& b) {
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++) r.e[i][j] = mul_entry(a, b, i, j);
}

template <typename T>
__device__ __forceinline__ T row_norm2(const cplx<T>* r) {
  return fm(r[2].im, r[2].im, fm(r[2].re, r[2].re, fm(r[1].im, r[1].im, fm(r[1].re, r[1].re,
         fm(r[0].im, r[0].im, r[0].re * r[0].re)))));
}

// Gram-Schmidt on rows 0,1 (dev_su3.cu:1569-1615); row 2 only when asked
template <typename T, bool ROW2>
__device__ __forceinline__ void normalize(Mat3<T>& u) {
  T len = rsqrt_t<T>(row_norm2<T>(u.e[0]));
#pragma unroll
  for (int i = 0; i < 3; i++) {
    u.e[0][i].re *= len;
    u.e[0][i].im *= len;
  }
  cplx<T> proj = cmulc(u.e[1][0], u.e[0][0]);
  cmacc(proj, u.e[1][1], u.e[0][1]);
  cmacc(proj, u.e[1][2], u.e[0][2]);
#pragma unroll
  for (int i = 0; i < 3; i++) {
    const cplx<T> b = u.e[1][i], a = u.e[0][i];
    u.e[1][i].re = fm(proj.im, a.im, fm(-proj.re, a.re, b.re));
    u.e[1][i].im = fm(-proj.im, a.re, fm(-proj.re, a.im, b.im));
  }
  len = rsqrt_t<T>(row_norm2<T>(u.e[1]));
#pragma unroll
  for (int i = 0; i < 3; i++) {
    u.e[1][i].re *= len;
    u.e[1][i].im *= len;
  }
  if (ROW2) row2_from_01(u);
}

// ---------------------------------------------------------------------------
// SU(2) subgroup updates.  A subgroup element is the 4-vector
// (w0, w1, w2, w3) = (a.x, a.y, b.x, b.y) of the reference (overrelax.cu:184-198).
// ---------------------------------------------------------------------------
template <typename T>
struct Su2 {
  T v[4];
};

// w of subgroup (a,b) of X = g * star (overrelax.cu:217-223); only four entries of X
template <typename T>
__device__ __forceinline__ Su2<T> su2_extract(const Mat3<T>& g, const Mat3<T>& star, int a, int b) {
  cplx<T> xaa = mul_entry(g, star, a, a);
  cplx<T> xbb = mul_entry(g, star, b, b);
  cplx<T> xab = mul_entry(g, star, a, b);
  cplx<T> xba = mul_entry(g, star, b, a);
  Su2<T> w;
  w.v[0] = xaa.re + xbb.re;
  w.v[3] = -xaa.im + xbb.im;
  w.v[1] = -xab.im - xba.im;
  w.v[2] = -xab.re + xba.re;
  return w;
}

// rows a,b of g <- alpha acting from the left (overrelax.cu:244-265):
//   row_a' = (a0 + i a3) row_a + (a2 + i a1) row_b
//   row_b' = (-a2 + i a1) row_a + (a0 - i a3) row_b
template <typename T>
__device__ __forceinline__ void su2_rotate(Mat3<T>& g, int a, int b, const Su2<T>& al) {
  const T a0 = al.v[0], a1 = al.v[1], a2 = al.v[2], a3 = al.v[3];
#pragma unroll
  for (int c = 0; c < 3; c++) {
    const cplx<T> ga = g.e[a][c], gb = g.e[b][c];
    g.e[a][c].re = fm(-a1, gb.im, fm(a2, gb.re, fm(-a3, ga.im, a0 * ga.re)));
    g.e[a][c].im = fm(a1, gb.re, fm(a2, gb.im, fm(a3, ga.re, a0 * ga.im)));
    g.e[b][c].re = fm(a3, gb.im, fm(a0, gb.re, fm(-a1, ga.im, -a2 * ga.re)));
    g.e[b][c].im = fm(-a3, gb.re, fm(a0, gb.im, fm(a1, ga.re, -a2 * ga.im)));
  }
}

// SU(2) subgroups in the reference's order: (0,1), (0,2), (1,2)
__device__ __forceinline__ int sub_a(int s) { return s == 2 ? 1 : 0; }
__device__ __forceinline__ int sub_b(int s) { return s == 0 ? 1 : 2; }

// Cabibbo-Marinari relaxation (overrelax.cu:203-269)
template <typename T>
__device__ __forceinline__ void cm_relax(Mat3<T>& g, const Mat3<T>& star) {
#pragma unroll
  for (int s = 0; s < 3; s++) {
    const int a = sub_a(s), b = sub_b(s);
    Su2<T> w = su2_extract(g, star, a, b);
    T det = rsqrt_t<T>(w.v[0] * w.v[0] + w.v[1] * w.v[1] + w.v[2] * w.v[2] + w.v[3] * w.v[3]);
#pragma unroll
    for (int k = 0; k < 4; k++) w.v[k] *= det;
    su2_rotate(g, a, b, w);
  }
}

// Micro-overrelaxation: alpha = (2 w0/|w|^2) w - 1, i.e. the square of the relaxed
// subgroup element (heatbath_thermalization.cu:318-401)
template <typename T>
__device__ __forceinline__ void cm_micro(Mat3<T>& g, const Mat3<T>& star) {
#pragma unroll
  for (int s = 0; s < 3; s++) {
    const int a = sub_a(s), b = sub_b(s);
    Su2<T> w = su2_extract(g, star, a, b);
    T tr = w.v[0] * w.v[0] + w.v[1] * w.v[1] + w.v[2] * w.v[2] + w.v[3] * w.v[3];
    Su2<T> al;
    if (fabs((double)tr) < 1.0e-9) {
      al.v[0] = T(1);
      al.v[1] = al.v[2] = al.v[3] = T(0);
    } else {
      T fac = T(2) * w.v[0] / tr;
#pragma unroll
      for (int k = 0; k < 4; k++) al.v[k] = fac * w.v[k];
      al.v[0] -= T(1);
    }
    su2_rotate(g, a, b, al);
  }
}

// Overrelaxation step of overrelax.cu:149-177, 411-417:
//   g_new = normalize( normalize(Rw) g_old ),  Rw = 1 + w R + w(w-1)/2 R^2,
//   R = g_relax g_old^+ - 1.
// For g_old in SU(3), normalize(Rw) g_old = normalize(Rw g_old), and
//   Rw g_old = g_old + w D + w(w-1)/2 (D g_old^+) D,  D = g_relax - g_old,
// so only rows 0,1 of the result are formed (they are all that is stored).
template <typename T>
__device__ __forceinline__ void overrelax_rows01(Mat3<T>& gout, const Mat3<T>& gold,
                                                 const Mat3<T>& grelax, T omega) {
  Mat3<T> D;
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++) D.e[i][j] = csub(grelax.e[i][j], gold.e[i][j]);
  const T c2 = omega * (omega - T(1)) * T(0.5);
#pragma unroll
  for (int r = 0; r < 2; r++) {
    // c2 * R_rk with R = D gold^+
    cplx<T> R[3];
#pragma unroll
    for (int k = 0; k < 3; k++) {
      cplx<T> x = cmulc(D.e[r][0], gold.e[k][0]);
      cmacc(x, D.e[r][1], gold.e[k][1]);
      cmacc(x, D.e[r][2], gold.e[k][2]);
      R[k] = cmk<T>(c2 * x.re, c2 * x.im);
    }
#pragma unroll
    for (int j = 0; j < 3; j++) {
      cplx<T> o = cmk<T>(fm(omega, D.e[r][j].re, gold.e[r][j].re),
                         fm(omega, D.e[r][j].im, gold.e[r][j].im));
#pragma unroll
      for (int k = 0; k < 3; k++) cmac(o, R[k], D.e[k][j]);
      gout.e[r][j] = o;
    }
  }
  normalize<T, false>(gout);
}

// ---------------------------------------------------------------------------
// The same overrelaxation update with fewer operations (used for FP32 sweeps; the
// FP64 sweeps keep the reference's operation order above).
// The three subgroup steps act from the left, g_relax = S g_old with
// S = S3 S2 S1, so R = g_relax g_old^+ - 1 = S - 1, and
//   Rw g_old = g_old + (w R + w(w-1)/2 R^2) g_old        (rows 0, 1 only).
// Each subgroup needs four entries of X = S_k..S_1 g_old w; they are carried
// along by rotating only the entries later subgroups read.
// ---------------------------------------------------------------------------
// the unit SU(2) element of subgroup (a,b) from Xaa, Xbb, Xab, Xba as (p, q):
// rows a,b <- (p row_a + q row_b, -conj(q) row_a + conj(p) row_b)   (overrelax.cu:184-198)
template <typename T>
__device__ __forceinline__ void su2_pq(cplx<T> xaa, cplx<T> xbb, cplx<T> xab, cplx<T> xba,
                                       cplx<T>& p, cplx<T>& q) {
  const T w0 = xaa.re + xbb.re, w3 = xbb.im - xaa.im, w1 = -xab.im - xba.im,
          w2 = xba.re - xab.re;
  const T r = rsqrt_t<T>(fm(w3, w3, fm(w2, w2, fm(w1, w1, w0 * w0))));
  p = cmk<T>(w0 * r, w3 * r);
  q = cmk<T>(w2 * r, w1 * r);
}
// -conj(q) x + conj(p) y
template <typename T>
__device__ __forceinline__ cplx<T> su2_low(cplx<T> p, cplx<T> q, cplx<T> x, cplx<T> y) {
  cplx<T> r = cmk<T>(-q.re, q.im);  // -conj(q)
  cplx<T> o = cmul(r, x);
  cmac(o, cconj(p), y);
  return o;
}
// p x + q y
template <typename T>
__device__ __forceinline__ cplx<T> su2_high(cplx<T> p, cplx<T> q, cplx<T> x, cplx<T> y) {
  cplx<T> o = cmul(p, x);
  cmac(o, q, y);
  return o;
}

template <typename T>
__device__ __forceinline__ void or_update_composed(const Mat3<T>& gold, const Mat3<T>& star,
                                                   T omega, Mat3<T>& gn) {
  Mat3<T> X;
  mul(X, gold, star);
  cplx<T> p1, q1, p2, q2, p3, q3;
  su2_pq(X.e[0][0], X.e[1][1], X.e[0][1], X.e[1][0], p1, q1);  // subgroup (0,1)
  const cplx<T> x00 = su2_high(p1, q1, X.e[0][0], X.e[1][0]);
  const cplx<T> x01 = su2_high(p1, q1, X.e[0][1], X.e[1][1]);
  const cplx<T> x02 = su2_high(p1, q1, X.e[0][2], X.e[1][2]);
  const cplx<T> x11 = su2_low(p1, q1, X.e[0][1], X.e[1][1]);
  const cplx<T> x12 = su2_low(p1, q1, X.e[0][2], X.e[1][2]);
  su2_pq(x00, X.e[2][2], x02, X.e[2][0], p2, q2);  // subgroup (0,2)
  const cplx<T> y21 = su2_low(p2, q2, x01, X.e[2][1]);
  const cplx<T> y22 = su2_low(p2, q2, x02, X.e[2][2]);
  su2_pq(x11, y22, x12, y21, p3, q3);  // subgroup (1,2)
  // S = S3 S2 S1; S1 = [[p1, q1, 0], [-q1*, p1*, 0], [0, 0, 1]]
  const cplx<T> zero = cmk<T>(T(0), T(0));
  const cplx<T> s0[3] = {cmul(p2, p1), cmul(p2, q1), q2};
  const cplx<T> t2[3] = {cmul(cmk<T>(-q2.re, q2.im), p1), cmul(cmk<T>(-q2.re, q2.im), q1),
                         cconj(p2)};
  const cplx<T> r1[3] = {cmk<T>(-q1.re, q1.im), cconj(p1), zero};
  Mat3<T> R;  // S - 1
#pragma unroll
  for (int j = 0; j < 3; j++) {
    R.e[0][j] = s0[j];
    R.e[1][j] = su2_high(p3, q3, r1[j], t2[j]);
    R.e[2][j] = su2_low(p3, q3, r1[j], t2[j]);
  }
#pragma unroll
  for (int k = 0; k < 3; k++) R.e[k][k].re -= T(1);
  const T c2 = omega * (omega - T(1)) * T(0.5);
#pragma unroll
  for (int r = 0; r < 2; r++) {
    cplx<T> M[3];  // w R + c2 R^2, row r
#pragma unroll
    for (int j = 0; j < 3; j++) {
      const cplx<T> r2 = mul_entry(R, R, r, j);
      M[j] = cmk<T>(fm(omega, R.e[r][j].re, c2 * r2.re), fm(omega, R.e[r][j].im, c2 * r2.im));
    }
#pragma unroll
    for (int j = 0; j < 3; j++) {
      cplx<T> o = gold.e[r][j];
#pragma unroll
      for (int k = 0; k < 3; k++) cmac(o, M[k], gold.e[k][j]);
      gn.e[r][j] = o;
    }
  }
  normalize<T, false>(gn);
}

// ---------------------------------------------------------------------------
// Field layout in HBM
// ---------------------------------------------------------------------------
// A field of n matrices per (parity, slot) is stored as NCHUNK planes of 16-byte
// vectors: plane c holds chunk c of every matrix, so consecutive threads
// (consecutive checkerboard sites) read consecutive 16-byte words -- one
// fully coalesced 128-bit load per chunk.
//   FP32, 12 reals: 3 chunks of float4  (row0 = c0.xyzw, c1.xy; row1 = c1.zw, c2.xyzw)
//   FP64, 12 reals: 6 chunks of double2 (one complex number per chunk)
//   FP64, 18 reals: 9 chunks of double2 (rows 0..2, no reconstruction)
template <typename T>
struct VecOf;
template <>
struct VecOf<float> {
  typedef float4 type;
};
template <>
struct VecOf<double> {
  typedef double2 type;
};
// a double-float complex number: (re.hi, re.lo, im.hi, im.lo)
template <>
struct VecOf<dfl> {
  typedef float4 type;
};

template <typename T, int NR>
struct Field {
  typedef typename VecOf<T>::type V;
  // FP32 8-real links keep their exact 12-real rows in three more planes for the
  // links the 8-parameter form cannot hold accurately (see reconstruct8): 5 planes
  static constexpr int NCHUNK = NR == 8 ? 5 : NR * (int)sizeof(T) / 16;

  // load matrix i of the block starting at base (planes spaced by stride vectors)
  __device__ static __forceinline__ void load(const V* __restrict__ base, size_t stride, int i,
                                              Mat3<T>& m);
  __device__ static __forceinline__ void store(V* __restrict__ base, size_t stride, int i,
                                               const Mat3<T>& m);
};

template <typename T>
__device__ __forceinline__ T* mat_scalar(Mat3<T>& m, int k) {
  // k in [0,18): row-major complex entries, re/im interleaved
  return (&m.e[0][0].re) + k;
}

__device__ __forceinline__ float4 ldg_stream(const float4* p) { return __ldg(p); }
__device__ __forceinline__ double2 ldg_stream(const double2* p) { return __ldg(p); }

// rows 0,1 from the three 16-byte chunks of an FP32 12-real matrix; row 2 rebuilt
__device__ __forceinline__ void unpack12(float4 a, float4 b, float4 c, Mat3<float>& m) {
  m.e[0][0] = cmk(a.x, a.y);
  m.e[0][1] = cmk(a.z, a.w);
  m.e[0][2] = cmk(b.x, b.y);
  m.e[1][0] = cmk(b.z, b.w);
  m.e[1][1] = cmk(c.x, c.y);
  m.e[1][2] = cmk(c.z, c.w);
  row2_from_01(m);
}

template <>
__device__ __forceinline__ void Field<float, 12>::load(const float4* __restrict__ base,
                                                       size_t stride, int i, Mat3<float>& m) {
  unpack12(__ldg(base + i), __ldg(base + stride + i), __ldg(base + 2 * stride + i), m);
}

// 8-real links (the reference's GF_8 parameters, su3manip.c:234-276):
//   p = (a2, a3), q = (arg a1, arg c1, b1) for rows a, b, c.
// |a1| = sqrt(1 - |a2|^2 - |a3|^2) and |c1| = sqrt(1 - |a1|^2 - |b1|^2) from the unit
// first row and column.  b2, b3 follow from b orthogonal to a and conj(c1) = a2 b3 - a3 b2
// (c = conj(a x b)); c2, c3 from c orthogonal to a and conj(b1) = c2 a3 - c3 a2; each a 2x2
// system with determinant |a2|^2 + |a3|^2.  The layout cannot hold links with
// |a2|^2 + |a3|^2 near 0 (e.g. unit links; the FP32 error grows like 6e-8 over it):
// returns false below kMinN2For8, and the caller reads the exact 12-real rows.
constexpr float kMinN2For8 = 1e-2f;
__device__ __forceinline__ bool reconstruct8(float4 p, float4 q, Mat3<float>& m) {
  const cplx<float> a2 = cmk(p.x, p.y), a3 = cmk(p.z, p.w), b1 = cmk(q.z, q.w);
  const float n2 = fm(p.w, p.w, fm(p.z, p.z, fm(p.y, p.y, p.x * p.x)));
  if (n2 < kMinN2For8) return false;
  // hardware approximations (a few FP32 ulp): this copy only feeds the FP32 sweeps
  const float x1 = fmaxf(1.0f - n2, 0.0f);
  const float xc = fmaxf(n2 - fm(b1.im, b1.im, b1.re * b1.re), 0.0f);
  const float r1 = x1 > 0.0f ? x1 * rsqrtf(x1) : 0.0f;
  const float rc = xc > 0.0f ? xc * rsqrtf(xc) : 0.0f;
  float s1, c1s, s3, c3s;
  __sincosf(q.x, &s1, &c1s);
  __sincosf(q.y, &s3, &c3s);
  const cplx<float> a1 = cmk(r1 * c1s, r1 * s1), c1 = cmk(rc * c3s, rc * s3);
  const float inv = __fdividef(1.0f, n2);
  const cplx<float> ca1b1 = cmulc(b1, a1);  // conj(a1) b1
  const cplx<float> ca1c1 = cmulc(c1, a1);  // conj(a1) c1
  const cplx<float> cc1 = cconj(c1), cb1 = cconj(b1), ca2 = cconj(a2), ca3 = cconj(a3);
  cplx<float> t;
  t = cmul(a2, ca1b1);
  cmac(t, ca3, cc1);
  const cplx<float> b2 = cmk(-t.re * inv, -t.im * inv);
  t = cmul(ca2, cc1);
  t = csub(t, cmul(a3, ca1b1));
  const cplx<float> b3 = cmk(t.re * inv, t.im * inv);
  t = cmul(ca3, cb1);
  t = csub(t, cmul(a2, ca1c1));
  const cplx<float> c2 = cmk(t.re * inv, t.im * inv);
  t = cmul(ca2, cb1);
  cmac(t, a3, ca1c1);
  const cplx<float> c3 = cmk(-t.re * inv, -t.im * inv);
  m.e[0][0] = a1;
  m.e[0][1] = a2;
  m.e[0][2] = a3;
  m.e[1][0] = b1;
  m.e[1][1] = b2;
  m.e[1][2] = b3;
  m.e[2][0] = c1;
  m.e[2][1] = c2;
  m.e[2][2] = c3;
  return true;
}

// planes 0, 1: the 8 parameters; planes 2-4: rows 0, 1 as in the 12-real layout,
// read only for the rare links reconstruct8 declines
template <>
__device__ __forceinline__ void Field<float, 8>::load(const float4* __restrict__ base,
                                                      size_t stride, int i, Mat3<float>& m) {
  if (!reconstruct8(__ldg(base + i), __ldg(base + stride + i), m))
    unpack12(__ldg(base + 2 * stride + i), __ldg(base + 3 * stride + i),
             __ldg(base + 4 * stride + i), m);
}


template <>
__device__ __forceinline__ void Field<float, 12>::store(float4* __restrict__ base, size_t stride,
                                                        int i, const Mat3<float>& m) {
  base[i] = make_float4(m.e[0][0].re, m.e[0][0].im, m.e[0][1].re, m.e[0][1].im);
  base[stride + i] = make_float4(m.e[0][2].re, m.e[0][2].im, m.e[1][0].re, m.e[1][0].im);
  base[2 * stride + i] = make_float4(m.e[1][1].re, m.e[1][1].im, m.e[1][2].re, m.e[1][2].im);
}
template <>
__device__ __forceinline__ void Field<double, 12>::load(const double2* __restrict__ base,
                                                        size_t stride, int i, Mat3<double>& m) {
#pragma unroll
  for (int k = 0; k < 6; k++) {
    double2 v = __ldg(base + k * stride + i);
    m.e[k / 3][k % 3] = cmk(v.x, v.y);
  }
  row2_from_01(m);
}
template <>
__device__ __forceinline__ void Field<double, 12>::store(double2* __restrict__ base,
                                                         size_t stride, int i,
                                                         const Mat3<double>& m) {
#pragma unroll
  for (int k = 0; k < 6; k++) base[k * stride + i] = make_double2(m.e[k / 3][k % 3].re, m.e[k / 3][k % 3].im);
}
template <>
__device__ __forceinline__ void Field<double, 18>::load(const double2* __restrict__ base,
                                                        size_t stride, int i, Mat3<double>& m) {
#pragma unroll
  for (int k = 0; k < 9; k++) {
    double2 v = __ldg(base + k * stride + i);
    m.e[k / 3][k % 3] = cmk(v.x, v.y);
  }
}
template <>
__device__ __forceinline__ void Field<double, 18>::store(double2* __restrict__ base,
                                                         size_t stride, int i,
                                                         const Mat3<double>& m) {
#pragma unroll
  for (int k = 0; k < 9; k++) base[k * stride + i] = make_double2(m.e[k / 3][k % 3].re, m.e[k / 3][k % 3].im);
}

// double-float fields: one complex entry per 16-byte chunk, rows 0..1 (12 reals,
// row 2 rebuilt) or rows 0..2 (18 reals)
template <int NR>
__device__ __forceinline__ void load_df(const float4* __restrict__ base, size_t stride, int i,
                                        Mat3<dfl>& m) {
#pragma unroll
  for (int k = 0; k < NR / 2; k++) {
    const float4 v = __ldg(base + k * stride + i);
    m.e[k / 3][k % 3] = cmk<dfl>(dfl(v.x, v.y), dfl(v.z, v.w));
  }
  if (NR == 12) row2_from_01(m);
}
template <int NR>
__device__ __forceinline__ void store_df(float4* __restrict__ base, size_t stride, int i,
                                         const Mat3<dfl>& m) {
#pragma unroll
  for (int k = 0; k < NR / 2; k++) {
    const cplx<dfl> z = m.e[k / 3][k % 3];
    base[k * stride + i] = make_float4(z.re.hi, z.re.lo, z.im.hi, z.im.lo);
  }
}
template <>
__device__ __forceinline__ void Field<dfl, 12>::load(const float4* __restrict__ base, size_t stride,
                                                     int i, Mat3<dfl>& m) {
  load_df<12>(base, stride, i, m);
}
template <>
__device__ __forceinline__ void Field<dfl, 12>::store(float4* __restrict__ base, size_t stride,
                                                      int i, const Mat3<dfl>& m) {
  store_df<12>(base, stride, i, m);
}
template <>
__device__ __forceinline__ void Field<dfl, 18>::load(const float4* __restrict__ base, size_t stride,
                                                     int i, Mat3<dfl>& m) {
  load_df<18>(base, stride, i, m);
}

// ---------------------------------------------------------------------------
// Lattice geometry
// ---------------------------------------------------------------------------
// Division by a runtime constant d <= 2^31 for dividends n < 2^31:
// q = (n * m) >> s with m = ceil(2^s / d), s = 31 + ceil(log2 d)  (round-up method).
struct FastDiv {
  uint32_t d, m, s;
};

__device__ __forceinline__ uint32_t fdiv(uint32_t n, const FastDiv& f) {
  return (uint32_t)(((unsigned long long)n * f.m) >> f.s);
}

// Checkerboard index of parity p: i = xh + LXh*(y + LY*(z + LZ*t)), x = 2*xh + ((p+y+z+t)&1).
// It equals the reference's lexic2eo numbering (cudagaugefix.cu:129-196) for even LX.
struct Lattice {
  int lx, ly, lz, lt;  // extents (all even)
  int lxh;             // lx/2
  int vh;              // V/2
  int sy, sz, st;      // eo-index strides of y, z, t
  FastDiv d_lxh, d_ly, d_lz;
};

struct Site {
  int i, xh, y, z, t, s;  // s = x & 1
};

__device__ __forceinline__ Site site_of(const Lattice& L, int i, int parity) {
  Site c;
  c.i = i;
  uint32_t r = fdiv((uint32_t)i, L.d_lxh);
  c.xh = i - (int)r * L.lxh;
  uint32_t r2 = fdiv(r, L.d_ly);
  c.y = (int)r - (int)r2 * L.ly;
  uint32_t r3 = fdiv(r2, L.d_lz);
  c.z = (int)r2 - (int)r3 * L.lz;
  c.t = (int)r3;
  c.s = (parity + c.y + c.z + c.t) & 1;
  return c;
}

// eo index of the neighbour x + mu (fwd) or x - mu (bwd); it has the opposite parity
__device__ __forceinline__ int nb_fwd(const Lattice& L, const Site& c, int mu) {
  switch (mu) {
    case 0: {
      int xh = c.xh + c.s;
      if (xh == L.lxh) xh = 0;
      return c.i - c.xh + xh;
    }
    case 1:
      return c.y == L.ly - 1 ? c.i - (L.ly - 1) * L.sy : c.i + L.sy;
    case 2:
      return c.z == L.lz - 1 ? c.i - (L.lz - 1) * L.sz : c.i + L.sz;
    default:
      return c.t == L.lt - 1 ? c.i - (L.lt - 1) * L.st : c.i + L.st;
  }
}
__device__ __forceinline__ int nb_bwd(const Lattice& L, const Site& c, int mu) {
  switch (mu) {
    case 0: {
      int xh = c.xh - (1 - c.s);
      if (xh < 0) xh = L.lxh - 1;
      return c.i - c.xh + xh;
    }
    case 1:
      return c.y == 0 ? c.i + (L.ly - 1) * L.sy : c.i - L.sy;
    case 2:
      return c.z == 0 ? c.i + (L.lz - 1) * L.sz : c.i - L.sz;
    default:
      return c.t == 0 ? c.i + (L.lt - 1) * L.st : c.i - L.st;
  }
}

// Pointers to one lattice's fields.  Links: block (p, mu) at U + (p*4+mu)*NCHUNK*vh,
// plane c of it at +c*vh.  Gauge transformation: block p at G + p*NCHUNK*vh.
template <typename T, int NRU, int NRG>
struct FieldPtrs {
  typedef typename VecOf<T>::type V;
  const V* U;
  V* G;
};

// ---------------------------------------------------------------------------
// block reductions (FP64 accumulation)
// ---------------------------------------------------------------------------
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ double warp_max(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

}  // namespace gfx
