/*
 * gfx_oracle.h -- CPU oracle for the cudagfx gauge-fixing hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker that the CUDA
 * implementation in cudagfx_gb300/ is compared against.  Only tests/,
 * __graft_entry__.smoke() and bench.py's CPU-baseline leg may load it.  The
 * product never links or calls it.
 *
 * Data formats follow the reference's host/device formats exactly:
 *   - sites are lexicographic, pos = x + LX*(y + LY*(z + LZ*t))
 *     (cudagaugefix.cu:79), directions mu = 0,1,2,3 = x,y,z,t;
 *   - neighbour table nn[8*pos + mu] (+mu) and nn[8*pos + 4 + mu] (-mu)
 *     (cudagaugefix.cu:72-118);
 *   - "2v" (12-real) matrices: rows 0 and 1, each 3 complex (re, im), i.e.
 *     12 doubles per matrix, link (pos,mu) at matrix index 4*pos+mu, gauge
 *     transformation g(pos) at matrix index pos (su3manip.c:212-299);
 *   - "su3" (18-real) matrices: complex[3][3] row-major (global.h:26-33).
 */
#ifndef GFX_ORACLE_H
#define GFX_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
  int lx, ly, lz, lt;
  long vol;        /* LX*LY*LZ*LT */
  int *nn;         /* 8*vol */
  int *eo_even;    /* vol/2: eo index -> lexicographic site (cudagaugefix.cu:176) */
  int *eo_odd;     /* vol/2 */
} orc_lattice;

/* geometry (cudagaugefix.cu:72-196) */
void orc_initnn(int lx, int ly, int lz, int lt, int *nn);
void orc_initnn_eo(int lx, int ly, int lz, int lt, int *eo_even, int *eo_odd);

/* layout conversions (su3manip.c:212-230, 281-359) */
void orc_su3_to_2v(const double *su3, double *v12, long n);
void orc_2v_to_su3(const double *v12, double *su3, long n);

/* checkerboard overrelaxation half-sweep (overrelax.cu:149-269, 335-446).
 * ndir = 4: Landau (reference); ndir = 3: Coulomb (spatial directions only). */
void orc_overrelax_halfsweep(const orc_lattice *L, const double *gf12, double *g12,
                             int parity, double omega, int ndir);

/* gauge functional (overrelax.cu:451-671): out[0] = F, out[1] = dAdA, out[2] = max dAdA.
 * For ndir = 3 the sums run over spatial directions and F is divided by 3V. */
void orc_functional(const orc_lattice *L, const double *gf12, const double *g12, int ndir,
                    double *out);
/* theta per time slice for Coulomb gauge: theta_t = (1/(3*V3)) sum_{x in slice} tr[DD^+] */
void orc_theta_slices(const orc_lattice *L, const double *gf12, const double *g12, int ndir,
                      double *theta_t);

/* mean plaquette (overrelax.cu:34-138) and Polyakov loop (new: (1/V3) sum tr P / 3) */
double orc_plaquette(const orc_lattice *L, const double *gf12);
void orc_polyakov(const orc_lattice *L, const double *gf12, double *re_im);

/* simulated-annealing gauge-transformation heatbath half-sweep
 * (simulated_annealing.cu:5-257); beta = 1/T */
void orc_heatbath_halfsweep(const orc_lattice *L, const double *gf12, double *g12, int parity,
                            const float *gauss, const float *unif, double beta);
/* microcanonical half-sweep of g: SU(2)-subgroup reflection (the micro-OR update of
 * heatbath_thermalization.cu:318-401 applied to the gauge-transformation star) */
void orc_micro_halfsweep(const orc_lattice *L, const double *gf12, double *g12, int parity,
                         int ndir);

/* Cabibbo-Marinari link heatbath of U_nu on one parity
 * (heatbath_thermalization.cu:235-308, 493-550), with the result stored at link
 * 4*pos+nu (the reference stores it at index pos, heatbath_thermalization.cu:527).
 * beta3 = beta/3 (heatbath_thermalization.cu:557-562). */
void orc_link_heatbath_halfsweep(const orc_lattice *L, double *gf12, int parity, int nu,
                                 const float *gauss, const float *unif, double beta3);

/* the same half-sweep with the Kennedy-Pendleton SU(2) step (the Wilson-action
 * heatbath); subgroup s of link (e, nu) uses random slot 4 e + ((nu + s) & 3) */
void orc_link_heatbath_halfsweep_kp(const orc_lattice *L, double *gf12, int parity, int nu,
                                    const float *gauss, const float *unif, double beta3);

/* Mersenne Twister MT607 bank (MersenneTwister.cu:142-229, 236-323) */
#define ORC_MT_COUNT 4096
#define ORC_MT_NN 19
typedef struct {
  uint32_t matrix_a[ORC_MT_COUNT];
  uint32_t mask_b[ORC_MT_COUNT];
  uint32_t mask_c[ORC_MT_COUNT];
  uint32_t seed[ORC_MT_COUNT];
  uint32_t status[ORC_MT_COUNT * ORC_MT_NN]; /* [twister][19] */
} orc_mt;

/* one RandomGPU call: nper outputs per twister, element i + 4096*j */
void orc_mt_generate(orc_mt *mt, float *out, int nper, int initialized);
/* BoxMullerGPU on pairs (2k, 2k+1) of each twister's lane */
void orc_boxmuller(float *d, int nper);
/* nper = alignUp(ceil(n / 4096), 2) (MersenneTwister.cu:245-253) */
int orc_mt_nper(int n);
/* init_MT (both RandomGPU calls with initialized=0) and update_MT */
void orc_mt_init_fields(orc_mt *mt, float *gauss, int nper_g, float *unif, int nper_u);
void orc_mt_update_fields(orc_mt *mt, float *gauss, int nper_g, float *unif, int nper_u);
/* generic MT core used for the known-answer test against std::mt19937 */
void orc_mt_generic(uint32_t *state, int n, int m, uint32_t umask, uint32_t lmask,
                    uint32_t a, int u, int s, uint32_t b, int t, uint32_t c, int l,
                    uint32_t *out, int nout);

/* glibc srand()/rand() stream (TYPE_3 additive feedback generator) */
void orc_glibc_rand(unsigned int seed, int n, int32_t *out);

/* Park-Miller multi-stream Lehmer generator (rngs.c:51-126) */
typedef struct {
  long seed[256];
  int stream;
} orc_pm;
void orc_pm_plant(orc_pm *pm, long x);
double orc_pm_random(orc_pm *pm);
/* random_init_trafo / random_init_gauge (su3manip.c:539-767), n matrices, su3 format */
void orc_random_init_su3_field(orc_pm *pm, double *su3, long n);

/* host observables on su3 (18-real) fields (observables.c:17-242) */
void orc_g_trafo18(const orc_lattice *L, double *u18, const double *g18);
double orc_gauge_functional18(const orc_lattice *L, const double *u18);
double orc_dAdA18(const orc_lattice *L, const double *u18, double *max_dAdA);
double orc_mean_plaq18(const orc_lattice *L, const double *u18);

#ifdef __cplusplus
}
#endif
#endif
