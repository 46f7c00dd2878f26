/*
 * gfx_oracle.c -- CPU oracle for the cudagfx gauge-fixing hot path.
 *
 * TEST INFRASTRUCTURE ONLY: the checker for the CUDA implementation, never
 * part of the product.  Each routine restates one piece of the reference's
 * algorithm in plain C, following the reference's order of operations so that
 * FP64 results agree with the reference to rounding.  Citations are
 * file:line in the reference (kpetrov/cudagfx).
 *
 * Build: gcc -O2 -ffp-contract=off -fopenmp -shared -fPIC (no FMA contraction,
 * so the results are identical on x86-64 and aarch64).
 */
#include "gfx_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

/* ------------------------------------------------------------------ */
/* complex and 3x3 helpers, same operation order as dev_su3.cu:17-83   */
/* ------------------------------------------------------------------ */
typedef struct { double re, im; } cx;
typedef cx m3[3][3];

static inline cx c_mk(double re, double im) { cx r; r.re = re; r.im = im; return r; }
static inline cx c_conj(cx a) { cx r; r.re = a.re; r.im = -1.0 * a.im; return r; }
static inline cx c_mul(cx a, cx b) {
  cx r;
  r.re = a.re * b.re - a.im * b.im;
  r.im = a.re * b.im + a.im * b.re;
  return r;
}
static inline cx c_add(cx a, cx b) { cx r; r.re = a.re + b.re; r.im = a.im + b.im; return r; }
static inline cx c_sub(cx a, cx b) { cx r; r.re = a.re - b.re; r.im = a.im - b.im; return r; }

static void m_zero(m3 m) {
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) m[i][j] = c_mk(0.0, 0.0);
}
static void m_unit(m3 m) {
  m_zero(m);
  m[0][0].re = 1.0; m[1][1].re = 1.0; m[2][2].re = 1.0;
}
static void m_copy(m3 to, m3 from) { memcpy(to, from, sizeof(m3)); }

/* u = v * w  (dev_su3.cu:1418-1433) */
static void m_mul(m3 u, m3 v, m3 w) {
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) {
      cx h2 = c_mk(0.0, 0.0);
      for (int k = 0; k < 3; k++) h2 = c_add(c_mul(v[i][k], w[k][j]), h2);
      u[i][j] = h2;
    }
}
/* u += v * w  (dev_su3.cu:1440-1456) */
static void m_addmul(m3 u, m3 v, m3 w) {
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) {
      cx h2 = c_mk(0.0, 0.0);
      for (int k = 0; k < 3; k++) h2 = c_add(c_mul(v[i][k], w[k][j]), h2);
      u[i][j].re += h2.re;
      u[i][j].im += h2.im;
    }
}
/* u = v * w^+  (dev_su3.cu:1461-1475) */
static void m_mul_d(m3 u, m3 v, m3 w) {
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) {
      cx h2 = c_mk(0.0, 0.0);
      for (int k = 0; k < 3; k++) h2 = c_add(c_mul(v[i][k], c_conj(w[j][k])), h2);
      u[i][j] = h2;
    }
}
static void m_dagger(m3 r, m3 m) {
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) r[i][j] = c_conj(m[j][i]);
}
static void m_sub_inplace(m3 a, m3 b) {
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) a[i][j] = c_sub(a[i][j], b[i][j]);
}
static void m_add_inplace(m3 a, m3 b) {
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) a[i][j] = c_add(a[i][j], b[i][j]);
}
static cx m_trace(m3 m) {
  cx e = c_mk(0.0, 0.0);
  for (int i = 0; i < 3; i++) e = c_add(e, m[i][i]);
  return e;
}
static double m_retrace(m3 m) {
  double e = 0.0;
  for (int i = 0; i < 3; i++) e = e + m[i][i].re;
  return e;
}

/* row 2 = conj(row0 x row1), the order of dev_su3.cu:289-305 */
static void m_row2(m3 g) {
  cx h1, h2;
  h1 = c_mul(g[0][1], g[1][2]); h2 = c_mul(g[0][2], g[1][1]); g[2][0] = c_conj(c_sub(h1, h2));
  h1 = c_mul(g[0][2], g[1][0]); h2 = c_mul(g[0][0], g[1][2]); g[2][1] = c_conj(c_sub(h1, h2));
  h1 = c_mul(g[0][0], g[1][1]); h2 = c_mul(g[0][1], g[1][0]); g[2][2] = c_conj(c_sub(h1, h2));
}

/* 12-real reconstruct (dev_su3.cu:225-308) */
static void load12(const double *f, long idx, m3 g) {
  const double *p = f + 12 * idx;
  for (int r = 0; r < 2; r++)
    for (int c = 0; c < 3; c++) g[r][c] = c_mk(p[(r * 3 + c) * 2], p[(r * 3 + c) * 2 + 1]);
  m_row2(g);
}
/* 12-real dagger reconstruct (dev_su3.cu:314-416) */
static void load12_dagger(const double *f, long idx, m3 g) {
  const double *p = f + 12 * idx;
  g[0][0] = c_mk(p[0], -p[1]);
  g[1][0] = c_mk(p[2], -p[3]);
  g[2][0] = c_mk(p[4], -p[5]);
  g[0][1] = c_mk(p[6], -p[7]);
  g[1][1] = c_mk(p[8], -p[9]);
  g[2][1] = c_mk(p[10], -p[11]);
  cx h1, h2;
  h1 = c_conj(c_mul(g[1][0], g[2][1])); h2 = c_conj(c_mul(g[2][0], g[1][1]));
  g[0][2] = c_sub(h1, h2);
  h1 = c_conj(c_mul(g[2][0], g[0][1])); h2 = c_conj(c_mul(g[0][0], g[2][1]));
  g[1][2] = c_sub(h1, h2);
  h1 = c_conj(c_mul(g[0][0], g[1][1])); h2 = c_conj(c_mul(g[1][0], g[0][1]));
  g[2][2] = c_sub(h1, h2);
}
static void store12(double *f, long idx, m3 g) {
  double *p = f + 12 * idx;
  for (int r = 0; r < 2; r++)
    for (int c = 0; c < 3; c++) {
      p[(r * 3 + c) * 2] = g[r][c].re;
      p[(r * 3 + c) * 2 + 1] = g[r][c].im;
    }
}

/* Gram-Schmidt reunitarization (dev_su3.cu:1569-1634); rsqrt -> 1/sqrt */
static void m_normalize(m3 u) {
  double len = (u[0][0].re * u[0][0].re + u[0][0].im * u[0][0].im) +
               (u[0][1].re * u[0][1].re + u[0][1].im * u[0][1].im) +
               (u[0][2].re * u[0][2].re + u[0][2].im * u[0][2].im);
  len = 1.0 / sqrt(len);
  for (int i = 0; i < 3; i++) { u[0][i].re = u[0][i].re * len; u[0][i].im = u[0][i].im * len; }
  cx proj = c_mk(0.0, 0.0);
  for (int i = 0; i < 3; i++) proj = c_add(proj, c_mul(u[1][i], c_conj(u[0][i])));
  for (int i = 0; i < 3; i++) u[1][i] = c_sub(u[1][i], c_mul(proj, u[0][i]));
  len = (u[1][0].re * u[1][0].re + u[1][0].im * u[1][0].im) +
        (u[1][1].re * u[1][1].re + u[1][1].im * u[1][1].im) +
        (u[1][2].re * u[1][2].re + u[1][2].im * u[1][2].im);
  len = 1.0 / sqrt(len);
  for (int i = 0; i < 3; i++) { u[1][i].re = u[1][i].re * len; u[1][i].im = u[1][i].im * len; }
  m_row2(u);
}

/* ------------------------------------------------------------------ */
/* geometry                                                            */
/* ------------------------------------------------------------------ */
void orc_initnn(int LX, int LY, int LZ, int T, int *nn) {
  for (int t = 0; t < T; t++)
    for (int z = 0; z < LZ; z++)
      for (int y = 0; y < LY; y++)
        for (int x = 0; x < LX; x++) {
          long pos = x + (long)LX * (y + (long)LY * (z + (long)LZ * t));
          nn[8 * pos + 0] = (x + 1) % LX + LX * (y + LY * (z + LZ * t));
          nn[8 * pos + 1] = x + LX * ((y + 1) % LY + LY * (z + LZ * t));
          nn[8 * pos + 2] = x + LX * (y + LY * ((z + 1) % LZ + LZ * t));
          nn[8 * pos + 3] = x + LX * (y + LY * (z + LZ * ((t + 1) % T)));
          nn[8 * pos + 4] = (x + LX - 1) % LX + LX * (y + LY * (z + LZ * t));
          nn[8 * pos + 5] = x + LX * ((y + LY - 1) % LY + LY * (z + LZ * t));
          nn[8 * pos + 6] = x + LX * (y + LY * ((z + LZ - 1) % LZ + LZ * t));
          nn[8 * pos + 7] = x + LX * (y + LY * (z + LZ * ((t + T - 1) % T)));
        }
}

void orc_initnn_eo(int LX, int LY, int LZ, int T, int *eo_even, int *eo_odd) {
  long ne = 0, no = 0;
  for (int t = 0; t < T; t++)
    for (int z = 0; z < LZ; z++)
      for (int y = 0; y < LY; y++)
        for (int x = 0; x < LX; x++) {
          int pos = x + LX * (y + LY * (z + LZ * t));
          if (((x + y + z + t) % 2) == 0) eo_even[ne++] = pos;
          else eo_odd[no++] = pos;
        }
}

void orc_su3_to_2v(const double *su3, double *v12, long n) {
  for (long i = 0; i < n; i++) memcpy(v12 + 12 * i, su3 + 18 * i, 12 * sizeof(double));
}

/* from2vtosu3_trafo (su3manip.c:303-359) */
void orc_2v_to_su3(const double *v12, double *su3, long n) {
  for (long i = 0; i < n; i++) {
    m3 g;
    for (int r = 0; r < 2; r++)
      for (int c = 0; c < 3; c++)
        g[r][c] = c_mk(v12[12 * i + (r * 3 + c) * 2], v12[12 * i + (r * 3 + c) * 2 + 1]);
    m_row2(g);
    memcpy(su3 + 18 * i, g, sizeof(m3));
  }
}

/* ------------------------------------------------------------------ */
/* star and SU(2)-subgroup updates                                     */
/* ------------------------------------------------------------------ */
/* star w(x) = sum_mu U_mu(x) g^+(x+mu) + U_mu^+(x-mu) g^+(x-mu)  (overrelax.cu:350-394) */
static void gauge_star(const orc_lattice *L, const double *gf12, const double *g12, long pos,
                       int ndir, m3 star) {
  m3 a, b;
  m_zero(star);
  for (int mu = 0; mu < ndir; mu++) {
    long hop = L->nn[8 * pos + mu];
    load12(gf12, 4 * pos + mu, a);
    load12_dagger(g12, hop, b);
    m_addmul(star, a, b);
    hop = L->nn[8 * pos + 4 + mu];
    load12_dagger(gf12, 4 * hop + mu, a);
    load12_dagger(g12, hop, b);
    m_addmul(star, a, b);
  }
}

/* the 4-vector of SU(2) subgroup (a,b) of X = g * star (overrelax.cu:217-223);
 * w = {a.x, a.y, b.x, b.y} */
static void su2_extract(m3 g, m3 star, int a, int b, double w[4]) {
  m3 X;
  m_mul(X, g, star);
  w[0] = X[a][a].re + X[b][b].re;
  w[3] = -X[a][a].im + X[b][b].im;
  w[1] = -X[a][b].im - X[b][a].im;
  w[2] = -X[a][b].re + X[b][a].re;
}

/* left-multiply rows a,b of g by the SU(2) element alpha (overrelax.cu:244-265) */
static void su2_rotate(m3 g, int a, int b, const double al[4]) {
  for (int c = 0; c < 3; c++) {
    cx d = c_mul(c_mk(al[0], al[3]), g[a][c]);
    cx d2 = c_mul(c_mk(al[2], al[1]), g[b][c]);
    d = c_add(d, d2);
    d2 = c_mul(c_mk(-al[2], al[1]), g[a][c]);
    cx d3 = c_mul(c_mk(al[0], -al[3]), g[b][c]);
    g[b][c] = c_add(d2, d3);
    g[a][c] = d;
  }
}

static const int SUB_A[3] = {0, 0, 1};
static const int SUB_B[3] = {1, 2, 2};

/* cabibbo_marinari_relax (overrelax.cu:188-269) */
static void cm_relax(m3 g, m3 star) {
  for (int s = 0; s < 3; s++) {
    double w[4], al[4];
    su2_extract(g, star, SUB_A[s], SUB_B[s], w);
    double det = w[0] * w[0] + w[1] * w[1] + w[2] * w[2] + w[3] * w[3];
    det = 1.0 / sqrt(det);
    for (int k = 0; k < 4; k++) al[k] = w[k] * det;
    su2_rotate(g, SUB_A[s], SUB_B[s], al);
  }
}

/* g = R^w g with R = gn g^+ - 1, truncated binomial series (overrelax.cu:149-177) */
static void overrelax_series(m3 g, m3 gn, double w, int N) {
  m3 one, R, a, Rw, help;
  m_unit(one);
  m_mul_d(R, gn, g);
  m_sub_inplace(R, one);
  m_copy(Rw, one);
  m_copy(a, one);
  for (int i = 1; i < N; i++) {
    m_mul(help, a, R);
    m_copy(a, help);
    double f = (1.0 + w - i) / i;
    for (int r = 0; r < 3; r++)
      for (int c = 0; c < 3; c++) { a[r][c].re *= f; a[r][c].im *= f; }
    m_add_inplace(Rw, a);
  }
  m_normalize(Rw);
  m_mul(help, Rw, g);
  m_copy(g, help);
}

static const int *eo_table(const orc_lattice *L, int parity) {
  return parity == 0 ? L->eo_even : L->eo_odd;
}

void orc_overrelax_halfsweep(const orc_lattice *L, const double *gf12, double *g12, int parity,
                             double omega, int ndir) {
  const int *tab = eo_table(L, parity);
  long nh = L->vol / 2;
#pragma omp parallel for schedule(static)
  for (long e = 0; e < nh; e++) {
    long pos = tab[e];
    m3 star, g, help;
    gauge_star(L, gf12, g12, pos, ndir, star);
    load12(g12, pos, g);
    m_copy(help, g);
    cm_relax(help, star);
    m_normalize(help);
    overrelax_series(g, help, omega, 3);
    m_normalize(g);
    store12(g12, pos, g);
  }
}

/* ------------------------------------------------------------------ */
/* functional (overrelax.cu:451-605)                                    */
/* ------------------------------------------------------------------ */
/* U -> -i/2 (U - U^+), traceless (overrelax.cu:451-473) */
static void vectorpotential_inplace(m3 U) {
  m3 temp;
  m_dagger(temp, U);
  m_sub_inplace(temp, U);
  cx ih = c_mk(0.0, 0.5);
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) U[i][j] = c_mul(ih, temp[i][j]);
  cx tr = m_trace(U);
  tr.re = tr.re / 3.0;
  tr.im = tr.im / 3.0;
  for (int i = 0; i < 3; i++) U[i][i] = c_sub(U[i][i], tr);
}

/* per-site F and tr[Delta Delta^+] exactly as dev_functional computes them */
static void site_functional(const orc_lattice *L, const double *gf12, const double *g12,
                            long pos, int ndir, double *F, double *dada) {
  m3 gather, help, fw, bw, a, b;
  m_zero(gather);
  double f = 0.0;
  for (int mu = 0; mu < ndir; mu++) {
    long hop = L->nn[8 * pos + mu];
    load12(gf12, 4 * pos + mu, a);
    load12(g12, pos, b);
    m_mul(help, b, a);
    load12_dagger(g12, hop, b);
    m_mul(fw, help, b);
    f += m_retrace(fw);
    hop = L->nn[8 * pos + 4 + mu];
    load12(gf12, 4 * hop + mu, a);
    load12(g12, hop, b);
    m_mul(help, b, a);
    load12_dagger(g12, pos, b);
    m_mul(bw, help, b);
    vectorpotential_inplace(fw);
    vectorpotential_inplace(bw);
    m_sub_inplace(bw, fw);
    m_add_inplace(gather, bw);
  }
  m_mul_d(help, gather, gather);
  *F = f;
  *dada = m_retrace(help);
}

void orc_functional(const orc_lattice *L, const double *gf12, const double *g12, int ndir,
                    double *out) {
  /* per-block partial sums over 128 consecutive sites, then the host sum
   * (overrelax.cu:590-603, 644-661) */
  long V = L->vol;
  long nblk = (V + 127) / 128;
  double *pf = (double *)calloc(nblk, sizeof(double));
  double *pd = (double *)calloc(nblk, sizeof(double));
  double *pm = (double *)calloc(nblk, sizeof(double));
#pragma omp parallel for schedule(static)
  for (long bk = 0; bk < nblk; bk++) {
    double sf = 0.0, sd = 0.0, mx = 0.0;
    for (long pos = bk * 128; pos < (bk + 1) * 128 && pos < V; pos++) {
      double f, d;
      site_functional(L, gf12, g12, pos, ndir, &f, &d);
      sf += f;
      sd += d;
      if (d > mx) mx = d;
    }
    pf[bk] = sf;
    pd[bk] = sd;
    pm[bk] = mx;
  }
  double F = 0.0, D = 0.0, M = 0.0;
  for (long bk = 0; bk < nblk; bk++) {
    F += pf[bk];
    D += pd[bk];
    if (pm[bk] > M) M = pm[bk];
  }
  out[0] = F / ((double)ndir * (double)V);
  out[1] = D / (double)V;
  out[2] = M;
  free(pf);
  free(pd);
  free(pm);
}

void orc_theta_slices(const orc_lattice *L, const double *gf12, const double *g12, int ndir,
                      double *theta_t) {
  long V3 = (long)L->lx * L->ly * L->lz;
#pragma omp parallel for schedule(static)
  for (int t = 0; t < L->lt; t++) {
    double s = 0.0;
    for (long k = 0; k < V3; k++) {
      double f, d;
      site_functional(L, gf12, g12, k + V3 * t, ndir, &f, &d);
      s += d;
    }
    theta_t[t] = s / (3.0 * (double)V3);
  }
}

/* mean plaquette (overrelax.cu:34-111) */
double orc_plaquette(const orc_lattice *L, const double *gf12) {
  long V = L->vol;
  double total = 0.0;
  long nt = L->lt;
  double *pt = (double *)calloc(nt, sizeof(double));
  long V3 = V / nt;
#pragma omp parallel for schedule(static)
  for (long t = 0; t < nt; t++) {
    double acc = 0.0;
    for (long k = 0; k < V3; k++) {
      long x0 = k + V3 * t;
      for (int nu = 0; nu < 3; nu++)
        for (int mu = nu + 1; mu < 4; mu++) {
          long x1 = L->nn[8 * x0 + mu], x2 = L->nn[8 * x0 + nu];
          m3 M1, M2, M3, M4, s1, s2;
          load12(gf12, 4 * x0 + mu, M1);
          load12(gf12, 4 * x1 + nu, M2);
          load12_dagger(gf12, 4 * x2 + mu, M3);
          load12_dagger(gf12, 4 * x0 + nu, M4);
          m_mul(s1, M3, M4);
          m_mul(s2, M2, s1);
          m_mul(s1, M1, s2);
          acc += m_trace(s1).re / 3.0;
        }
    }
    pt[t] = acc;
  }
  for (long t = 0; t < nt; t++) total += pt[t];
  free(pt);
  return total * (1.0 / (6.0 * (double)V));
}

/* Polyakov loop: P = (1/V3) sum_xvec (1/3) tr prod_t U_t(xvec, t) */
void orc_polyakov(const orc_lattice *L, const double *gf12, double *re_im) {
  long V3 = (long)L->lx * L->ly * L->lz;
  double sr = 0.0, si = 0.0;
  for (long k = 0; k < V3; k++) {
    m3 P, U, tmp;
    m_unit(P);
    for (int t = 0; t < L->lt; t++) {
      load12(gf12, 4 * (k + V3 * t) + 3, U);
      m_mul(tmp, P, U);
      m_copy(P, tmp);
    }
    cx tr = m_trace(P);
    sr += tr.re / 3.0;
    si += tr.im / 3.0;
  }
  re_im[0] = sr / (double)V3;
  re_im[1] = si / (double)V3;
}

/* ------------------------------------------------------------------ */
/* heatbath (simulated_annealing.cu:5-142)                             */
/* ------------------------------------------------------------------ */
/* dev_get_a0 (simulated_annealing.cu:5-27): single-precision trial */
static int get_a0(double *a0, double kb, const float *gauss, const float *unif, long ind) {
  float a, b, y, help;
  a = fabsf(gauss[ind]);
  b = -logf(1.0f - unif[4 * ind]);
  y = a * a + b;
  y = (float)((double)y / kb);
  help = unif[4 * ind + 1];
  if ((2.0f * (help * help)) <= (2.0f - y)) {
    *a0 = (double)(1.0f - y);
    return 1;
  }
  *a0 = 0.0;
  return 0;
}

/* dev_heatbath_su2 (simulated_annealing.cu:33-73) */
static void heatbath_su2(double al[4], const double w[4], double beta, const float *gauss,
                         const float *unif, long ind) {
  double v[4], a[4];
  double k = w[0] * w[0] + w[1] * w[1] + w[2] * w[2] + w[3] * w[3];
  double rdet = 1.0 / sqrt(k);
  for (int i = 0; i < 4; i++) v[i] = w[i] * rdet;
  int ret = get_a0(&a[0], k * beta, gauss, unif, ind);
  double norm = sqrt(1.0 - a[0] * a[0]);
  double cos_theta = 2.0 * (double)unif[4 * ind + 2] - 1.0;
  double sin_theta = sqrt(1.0 - cos_theta * cos_theta);
  double phi = 6.2831853071795862 * (double)unif[4 * ind + 3];
  double sphi = sin(phi), cphi = cos(phi);
  a[2] = sphi;
  a[1] = cphi;
  a[1] = norm * sin_theta * a[1];
  a[2] = norm * sin_theta * a[2];
  a[3] = norm * cos_theta;
  if (ret == 1) {
    /* dev_su2_ti_su2 (dev_su3.cu:1385-1399) with (a.x,a.y,b.x,b.y) = (0,1,2,3) */
    al[0] = a[0] * v[0] - a[1] * v[1] - a[2] * v[2] - a[3] * v[3];
    al[1] = a[0] * v[1] + a[1] * v[0] - a[2] * v[3] + a[3] * v[2];
    al[2] = a[0] * v[2] + a[2] * v[0] - a[3] * v[1] + a[1] * v[3];
    al[3] = a[0] * v[3] + a[3] * v[0] - a[1] * v[2] + a[2] * v[1];
  } else {
    for (int i = 0; i < 4; i++) al[i] = w[i];
  }
}

/* cabibbo_marinari_heatbath (simulated_annealing.cu:81-142) */
static void cm_heatbath(m3 g, m3 star, double beta, const float *gauss, const float *unif,
                        long ind) {
  for (int s = 0; s < 3; s++) {
    double w[4], al[4];
    su2_extract(g, star, SUB_A[s], SUB_B[s], w);
    heatbath_su2(al, w, beta, gauss, unif, ind);
    su2_rotate(g, SUB_A[s], SUB_B[s], al);
  }
}

void orc_heatbath_halfsweep(const orc_lattice *L, const double *gf12, double *g12, int parity,
                            const float *gauss, const float *unif, double beta) {
  const int *tab = eo_table(L, parity);
  long nh = L->vol / 2;
#pragma omp parallel for schedule(static)
  for (long e = 0; e < nh; e++) {
    long pos = tab[e];
    m3 star, help;
    gauge_star(L, gf12, g12, pos, 4, star);
    load12(g12, pos, help);
    cm_heatbath(help, star, beta, gauss, unif, e);
    m_normalize(help);
    store12(g12, pos, help);
  }
}

/* dev_microorx_su2 (heatbath_thermalization.cu:318-338) */
static void microorx_su2(double out[4], const double in[4]) {
  double tr = in[0] * in[0] + in[1] * in[1] + in[2] * in[2] + in[3] * in[3];
  if (fabs(tr) < 1.0e-9) {
    out[0] = 1.0; out[1] = 0.0; out[2] = 0.0; out[3] = 0.0;
  } else {
    double fac = 2.0 * in[0] / tr;
    for (int i = 0; i < 4; i++) out[i] = fac * in[i];
    out[0] = out[0] - 1.0;
  }
}

static void cm_micro(m3 g, m3 star) {
  for (int s = 0; s < 3; s++) {
    double w[4], al[4];
    su2_extract(g, star, SUB_A[s], SUB_B[s], w);
    microorx_su2(al, w);
    su2_rotate(g, SUB_A[s], SUB_B[s], al);
  }
}

void orc_micro_halfsweep(const orc_lattice *L, const double *gf12, double *g12, int parity,
                         int ndir) {
  const int *tab = eo_table(L, parity);
  long nh = L->vol / 2;
#pragma omp parallel for schedule(static)
  for (long e = 0; e < nh; e++) {
    long pos = tab[e];
    m3 star, help;
    gauge_star(L, gf12, g12, pos, ndir, star);
    load12(g12, pos, help);
    cm_micro(help, star);
    m_normalize(help);
    store12(g12, pos, help);
  }
}

/* staple of U_nu(x) (heatbath_thermalization.cu:235-308) */
static void link_staple(const orc_lattice *L, const double *gf12, long pos, int nu, m3 staple) {
  m3 h1, h2, h3;
  m_zero(staple);
  for (int mu = 0; mu < 4; mu++) {
    if (mu == nu) continue;
    long hop = L->nn[8 * pos + nu];
    load12(gf12, 4 * hop + mu, h1);
    hop = L->nn[8 * pos + mu];
    load12_dagger(gf12, 4 * hop + nu, h2);
    m_mul(h3, h1, h2);
    load12_dagger(gf12, 4 * pos + mu, h1);
    m_addmul(staple, h3, h1);
    hop = L->nn[8 * pos + nu];
    hop = L->nn[8 * hop + 4 + mu];
    load12_dagger(gf12, 4 * hop + mu, h1);
    hop = L->nn[8 * pos + 4 + mu];
    load12_dagger(gf12, 4 * hop + nu, h2);
    m_mul(h3, h1, h2);
    load12(gf12, 4 * hop + mu, h1);
    m_addmul(staple, h3, h1);
  }
}

void orc_link_heatbath_halfsweep(const orc_lattice *L, double *gf12, int parity, int nu,
                                 const float *gauss, const float *unif, double beta3) {
  const int *tab = eo_table(L, parity);
  long nh = L->vol / 2;
#pragma omp parallel for schedule(static)
  for (long e = 0; e < nh; e++) {
    long pos = tab[e];
    m3 st, help;
    load12(gf12, 4 * pos + nu, help);
    link_staple(L, gf12, pos, nu, st);
    cm_heatbath(help, st, beta3, gauss, unif, 4 * e + nu);
    m_normalize(help);
    store12(gf12, 4 * pos + nu, help);
  }
}

/* Kennedy-Pendleton SU(2) heatbath for the Wilson action (A. D. Kennedy and
 * B. J. Pendleton, Phys. Lett. B 156 (1985) 393).  The subgroup weight is
 * exp(beta3 alpha.w), so with k = |w| the component a0 along w/k has density
 * sqrt(1 - a0^2) exp(beta3 k a0).  One trial: 2 lambda^2 = (E + g^2 / 2) / (beta3 k)
 * with E = -ln(1 - u0) exponential and g standard normal, a0 = 1 - 2 lambda^2,
 * accepted when u1^2 <= 1 - lambda^2; the direction of (a1, a2, a3) is uniform on the
 * sphere (cos theta = 2 u2 - 1, phi = 2 pi u3).  A rejected trial leaves the
 * subgroup unchanged (alpha = 1).  alpha = a v with v = w / k (quaternion product). */
static void heatbath_su2_kp(double al[4], const double w[4], double beta3, const float *gauss,
                            const float *unif, long ind) {
  double k = sqrt(w[0] * w[0] + w[1] * w[1] + w[2] * w[2] + w[3] * w[3]);
  al[0] = 1.0;
  al[1] = al[2] = al[3] = 0.0;
  if (!(k > 0.0)) return;
  double g = (double)gauss[ind];
  double E = -log(1.0 - (double)unif[4 * ind]);
  double y = (E + 0.5 * g * g) / (beta3 * k); /* 2 lambda^2 */
  double u1 = (double)unif[4 * ind + 1];
  if (!(u1 * u1 <= 1.0 - 0.5 * y)) return;
  double a[4], v[4];
  for (int i = 0; i < 4; i++) v[i] = w[i] / k;
  a[0] = 1.0 - y;
  double norm = sqrt(fmax(0.0, 1.0 - a[0] * a[0]));
  double cos_theta = 2.0 * (double)unif[4 * ind + 2] - 1.0;
  double sin_theta = sqrt(fmax(0.0, 1.0 - cos_theta * cos_theta));
  double phi = 6.2831853071795862 * (double)unif[4 * ind + 3];
  a[1] = norm * sin_theta * cos(phi);
  a[2] = norm * sin_theta * sin(phi);
  a[3] = norm * cos_theta;
  al[0] = a[0] * v[0] - a[1] * v[1] - a[2] * v[2] - a[3] * v[3];
  al[1] = a[0] * v[1] + a[1] * v[0] - a[2] * v[3] + a[3] * v[2];
  al[2] = a[0] * v[2] + a[2] * v[0] - a[3] * v[1] + a[1] * v[3];
  al[3] = a[0] * v[3] + a[3] * v[0] - a[1] * v[2] + a[2] * v[1];
}

/* Cabibbo-Marinari link heatbath with the Kennedy-Pendleton SU(2) step (the Wilson
 * action heatbath; the reference's variant above is not, see orc_link_heatbath_halfsweep).
 * Subgroup s of link (e, nu) takes random slot 4 e + ((nu + s) & 3), so the three
 * subgroups use independent numbers from the same fields. */
void orc_link_heatbath_halfsweep_kp(const orc_lattice *L, double *gf12, int parity, int nu,
                                    const float *gauss, const float *unif, double beta3) {
  const int *tab = eo_table(L, parity);
  long nh = L->vol / 2;
#pragma omp parallel for schedule(static)
  for (long e = 0; e < nh; e++) {
    long pos = tab[e];
    m3 st, help;
    load12(gf12, 4 * pos + nu, help);
    link_staple(L, gf12, pos, nu, st);
    for (int sg = 0; sg < 3; sg++) {
      double w[4], al[4];
      su2_extract(help, st, SUB_A[sg], SUB_B[sg], w);
      heatbath_su2_kp(al, w, beta3, gauss, unif, 4 * e + ((nu + sg) & 3));
      su2_rotate(help, SUB_A[sg], SUB_B[sg], al);
    }
    m_normalize(help);
    store12(gf12, 4 * pos + nu, help);
  }
}

/* ------------------------------------------------------------------ */
/* Mersenne Twister MT607 bank                                          */
/* ------------------------------------------------------------------ */
#define MT_MM 9
#define MT_UMASK 0xFFFFFFFEu
#define MT_LMASK 0x1u

int orc_mt_nper(int n) {
  int q = (n % ORC_MT_COUNT) ? n / ORC_MT_COUNT + 1 : n / ORC_MT_COUNT;
  return (q % 2) ? q + 1 : q;
}

/* RandomGPU (MersenneTwister.cu:142-199): each call restarts at ring slot 0 */
void orc_mt_generate(orc_mt *M, float *out, int nper, int initialized) {
  for (int r = 0; r < ORC_MT_COUNT; r++) {
    uint32_t mt[ORC_MT_NN];
    uint32_t *st = M->status + (long)r * ORC_MT_NN;
    if (!initialized) {
      mt[0] = M->seed[r];
      for (int s = 1; s < ORC_MT_NN; s++)
        mt[s] = 1812433253u * (mt[s - 1] ^ (mt[s - 1] >> 30)) + (uint32_t)s;
    } else {
      for (int s = 0; s < ORC_MT_NN; s++) mt[s] = st[s];
    }
    int is = 0;
    uint32_t mti1 = mt[0];
    for (int o = 0; o < nper; o++) {
      int is1 = is + 1, isM = is + MT_MM;
      if (is1 >= ORC_MT_NN) is1 -= ORC_MT_NN;
      if (isM >= ORC_MT_NN) isM -= ORC_MT_NN;
      uint32_t mti = mti1;
      mti1 = mt[is1];
      uint32_t mtiM = mt[isM];
      uint32_t x = (mti & MT_UMASK) | (mti1 & MT_LMASK);
      x = mtiM ^ (x >> 1) ^ ((x & 1) ? M->matrix_a[r] : 0u);
      mt[is] = x;
      is = is1;
      x ^= (x >> 12);
      x ^= (x << 7) & M->mask_b[r];
      x ^= (x << 15) & M->mask_c[r];
      x ^= (x >> 18);
      out[r + (long)o * ORC_MT_COUNT] = ((float)x + 1.0f) / 4294967296.0f;
    }
    M->seed[r] = mt[0];
    for (int s = 0; s < ORC_MT_NN; s++) st[s] = mt[s];
  }
}

/* BoxMullerGPU (MersenneTwister.cu:210-229) with libm functions */
void orc_boxmuller(float *d, int nper) {
  const float PIf = 3.14159265358979f;
  for (int r = 0; r < ORC_MT_COUNT; r++)
    for (int o = 0; o < nper; o += 2) {
      float *u1 = d + r + (long)o * ORC_MT_COUNT;
      float *u2 = d + r + (long)(o + 1) * ORC_MT_COUNT;
      float rr = sqrtf(-2.0f * logf(*u1));
      float phi = 2 * PIf * *u2;
      *u1 = rr * cosf(phi);
      *u2 = rr * sinf(phi);
    }
}

/* init_MT (MersenneTwister.cu:236-289): both fields seeded with initialized=0 */
void orc_mt_init_fields(orc_mt *M, float *gauss, int nper_g, float *unif, int nper_u) {
  orc_mt_generate(M, gauss, nper_g, 0);
  orc_boxmuller(gauss, nper_g);
  orc_mt_generate(M, unif, nper_u, 0);
}

/* update_MT (MersenneTwister.cu:295-323) */
void orc_mt_update_fields(orc_mt *M, float *gauss, int nper_g, float *unif, int nper_u) {
  orc_mt_generate(M, gauss, nper_g, 1);
  orc_boxmuller(gauss, nper_g);
  orc_mt_generate(M, unif, nper_u, 1);
}

/* textbook Mersenne Twister with general parameters (Matsumoto & Nishimura 1998),
 * state[n] already initialized, generating nout outputs from slot 0 */
void orc_mt_generic(uint32_t *state, int n, int m, uint32_t umask, uint32_t lmask, uint32_t a,
                    int u, int s, uint32_t b, int t, uint32_t c, int l, uint32_t *out, int nout) {
  int i = 0;
  for (int o = 0; o < nout; o++) {
    int i1 = (i + 1) % n, im = (i + m) % n;
    uint32_t y = (state[i] & umask) | (state[i1] & lmask);
    state[i] = state[im] ^ (y >> 1) ^ ((y & 1u) ? a : 0u);
    uint32_t x = state[i];
    x ^= (x >> u);
    x ^= (x << s) & b;
    x ^= (x << t) & c;
    x ^= (x >> l);
    out[o] = x;
    i = i1;
  }
}

/* glibc srandom()/random() for the default TYPE_3 state (degree 31, separation 3):
 * r[0] = seed, r[i] = 16807 r[i-1] mod (2^31-1) for i < 31 (Schrage's method),
 * then r[i] = r[i-31] + r[i-3] (mod 2^32) with the first 310 outputs discarded;
 * each output is the new word >> 1. */
void orc_glibc_rand(unsigned int seed, int n, int32_t *out) {
  int32_t st[31];
  if (seed == 0) seed = 1;
  st[0] = (int32_t)seed;
  int32_t word = (int32_t)seed;
  for (int i = 1; i < 31; i++) {
    long hi = word / 127773;
    long lo = word % 127773;
    word = (int32_t)(16807 * lo - 2836 * hi);
    if (word < 0) word += 2147483647;
    st[i] = word;
  }
  int f = 3, r = 0;
  for (int k = -310; k < n; k++) {
    uint32_t val = (uint32_t)st[f] + (uint32_t)st[r];
    st[f] = (int32_t)val;
    if (k >= 0) out[k] = (int32_t)(val >> 1);
    f = (f + 1) % 31;
    r = (r + 1) % 31;
  }
}

/* ------------------------------------------------------------------ */
/* Park-Miller (rngs.c:51-126)                                          */
/* ------------------------------------------------------------------ */
#define PM_MOD 2147483647L
#define PM_MUL 48271L
#define PM_A256 22925L

double orc_pm_random(orc_pm *pm) {
  const long Q = PM_MOD / PM_MUL, R = PM_MOD % PM_MUL;
  long s = pm->seed[pm->stream];
  long t = PM_MUL * (s % Q) - R * (s / Q);
  pm->seed[pm->stream] = (t > 0) ? t : t + PM_MOD;
  return (double)pm->seed[pm->stream] / PM_MOD;
}

void orc_pm_plant(orc_pm *pm, long x) {
  const long Q = PM_MOD / PM_A256, R = PM_MOD % PM_A256;
  if (x > 0) x = x % PM_MOD;
  pm->seed[0] = x;
  for (int j = 1; j < 256; j++) {
    long y = PM_A256 * (pm->seed[j - 1] % Q) - R * (pm->seed[j - 1] / Q);
    pm->seed[j] = (y > 0) ? y : y + PM_MOD;
  }
  pm->stream = 0;
}

/* random_init_trafo (su3manip.c:539-641): rows by sequential fractions, then
 * Gram-Schmidt of row 1 and row 2 = conj(row0 x row1) */
void orc_random_init_su3_field(orc_pm *pm, double *su3, long n) {
  for (long i = 0; i < n; i++) {
    m3 g;
    for (int r = 0; r < 2; r++) {
      double norm = 0.0, help;
      double v[6];
      help = orc_pm_random(pm); v[0] = help; norm = help * help;
      for (int k = 1; k < 5; k++) {
        help = (1.0 - norm) * orc_pm_random(pm);
        v[k] = help;
        norm += help * help;
      }
      v[5] = sqrt(1.0 - norm);
      for (int c = 0; c < 3; c++) g[r][c] = c_mk(v[2 * c], v[2 * c + 1]);
    }
    cx proj = c_mk(0.0, 0.0);
    for (int j = 0; j < 3; j++) proj = c_add(proj, c_mul(g[1][j], c_conj(g[0][j])));
    for (int j = 0; j < 3; j++) g[1][j] = c_sub(g[1][j], c_mul(proj, g[0][j]));
    double len = g[1][0].re * g[1][0].re + g[1][0].im * g[1][0].im + g[1][1].re * g[1][1].re +
                 g[1][1].im * g[1][1].im + g[1][2].re * g[1][2].re + g[1][2].im * g[1][2].im;
    len = 1.0 / sqrt(len);
    for (int j = 0; j < 3; j++) { g[1][j].re *= len; g[1][j].im *= len; }
    cx h1, h2;
    h1 = c_sub(c_mul(g[0][1], g[1][2]), c_mul(g[0][2], g[1][1])); h1.im = -h1.im; g[2][0] = h1;
    h1 = c_sub(c_mul(g[0][2], g[1][0]), c_mul(g[0][0], g[1][2])); h1.im = -h1.im; g[2][1] = h1;
    h2 = c_sub(c_mul(g[0][0], g[1][1]), c_mul(g[0][1], g[1][0])); h2.im = -h2.im; g[2][2] = h2;
    memcpy(su3 + 18 * i, g, sizeof(m3));
  }
}

/* ------------------------------------------------------------------ */
/* host observables on 18-real fields (observables.c:17-242)           */
/* ------------------------------------------------------------------ */
static void ld18(const double *f, long idx, m3 m) { memcpy(m, f + 18 * idx, sizeof(m3)); }

void orc_g_trafo18(const orc_lattice *L, double *u18, const double *g18) {
  long V = L->vol;
#pragma omp parallel for schedule(static)
  for (long pos = 0; pos < V; pos++) {
    m3 g, u, gd, h1, h2, r;
    ld18(g18, pos, g);
    for (int mu = 0; mu < 4; mu++) {
      ld18(u18, 4 * pos + mu, u);
      m_mul(h1, g, u);
      ld18(g18, L->nn[8 * pos + mu], gd);
      m_dagger(h2, gd);
      m_mul(r, h1, h2);
      memcpy(u18 + 18 * (4 * pos + mu), r, sizeof(m3));
    }
  }
}

double orc_gauge_functional18(const orc_lattice *L, const double *u18) {
  double h = 0.0;
  for (long k = 0; k < 4 * L->vol; k++) {
    m3 m;
    ld18(u18, k, m);
    h += m_trace(m).re;
  }
  return h / (4.0 * (double)L->vol);
}

/* vectorpotential (observables.c:144-165): A = 1/(2i) (U - U^+), traceless */
static void vecpot18(m3 A, m3 U) {
  m3 h1, h2;
  m_dagger(h1, U);
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) h2[i][j] = c_sub(U[i][j], h1[i][j]);
  cx oti = c_mk(0.0, -0.5);
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) A[i][j] = c_mul(oti, h2[i][j]);
  cx tr = m_trace(A);
  tr.re = tr.re / 3.0;
  tr.im = tr.im / 3.0;
  for (int k = 0; k < 3; k++) A[k][k] = c_sub(A[k][k], tr);
}

double orc_dAdA18(const orc_lattice *L, const double *u18, double *max_dAdA) {
  long V = L->vol;
  double sum = 0.0, mx = 0.0;
  for (long pos = 0; pos < V; pos++) {
    m3 dA, h1, h2, M1, M2, h3, h4;
    m_zero(dA);
    for (int mu = 0; mu < 4; mu++) {
      ld18(u18, 4 * L->nn[8 * pos + 4 + mu] + mu, h1);
      ld18(u18, 4 * pos + mu, h2);
      vecpot18(M1, h1);
      vecpot18(M2, h2);
      for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) h3[i][j] = c_sub(M1[i][j], M2[i][j]);
      for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) dA[i][j] = c_add(h3[i][j], dA[i][j]);
    }
    m_dagger(h1, dA);
    m_mul(h4, dA, h1);
    double c = m_trace(h4).re;
    sum += c;
    if (c > mx) mx = c;
  }
  if (max_dAdA) *max_dAdA = mx;
  return sum / (double)V;
}

double orc_mean_plaq18(const orc_lattice *L, const double *u18) {
  long V = L->vol;
  double mplaq = 0.0;
  for (long x0 = 0; x0 < V; x0++)
    for (int nu = 0; nu < 3; nu++)
      for (int mu = nu + 1; mu < 4; mu++) {
        long x1 = L->nn[8 * x0 + mu], x2 = L->nn[8 * x0 + nu];
        m3 M1, M2, M3, M4, s1, s2, t;
        ld18(u18, 4 * x0 + mu, M1);
        ld18(u18, 4 * x1 + nu, M2);
        ld18(u18, 4 * x2 + mu, t);
        m_dagger(M3, t);
        ld18(u18, 4 * x0 + nu, t);
        m_dagger(M4, t);
        m_mul(s1, M3, M4);
        m_mul(s2, M2, s1);
        m_mul(s1, M1, s2);
        mplaq += m_trace(s1).re / 3.0;
      }
  return mplaq * (1.0 / (6.0 * (double)V));
}
