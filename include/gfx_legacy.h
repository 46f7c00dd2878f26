/*
 * gfx_legacy.h -- the reference's own C entry points and globals, exported by libgfx.
 *
 * The reference's host program (cudagaugefix.cu:599-828 main) calls these by name;
 * libgfx implements them on one process-wide context so that the reference's C
 * host files (read_input.c, gauge_io.c, observables.c, su3manip.c) and a main
 * written against them link unchanged.  Globals are defined here with default
 * visibility; a program that defines the same globals (the reference's main
 * defines them through global.h with MAIN_PROGRAM, read_input.c defines the
 * input parameters) overrides these definitions and libgfx then reads and writes
 * the program's copies.
 *
 * Types: gfx_su3 has the layout of the reference's su3 (complex[3][3] of doubles,
 * global.h:26-33); gfx_saparam_list and gfx_thermparam_list have the layouts of
 * SAPARAM_LIST and THERMPARAM_LIST (global.h:51-67).  A translation unit that
 * includes the reference's global.h declares the functions with su3* itself; the
 * symbols are the same.
 */
#ifndef GFX_LEGACY_H
#define GFX_LEGACY_H

#include "gfx.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
  double re, im;
} gfx_complex;
typedef gfx_complex gfx_su3[3][3];

typedef struct {
  double Tmin, Tmax, expo;
  int N, checkint;
} gfx_saparam_list;

typedef struct {
  int Nsweep, Nsave;
  double beta;
  int checkint, startcond;
} gfx_thermparam_list;

/* lattice and results (global.h:77-94) */
extern int T, L, LX, LY, LZ, VOLUME;
extern double PLAQ, FUNC, DADA, maxDADA;
/* input parameters (read_input.h:6-14) */
extern int randseed, orxmaxit, orxcheckinterval, saflag, orxflag, thermflag;
extern double orxeps;
extern gfx_saparam_list saparam;
extern gfx_thermparam_list thermparam;
/* opaque handles of the context's device fields; pass them where the reference
 * passes dev_gf / dev_trafo1 (global.h:128, 140) */
extern void *dev_gf, *dev_trafo1;
/* host geometry tables (global.h:104-119), allocated and filled by init_gaugefixing
 * and init_thermalization as the reference's initnn/initnn_eo do
 * (cudagaugefix.cu:72-196, 285-323), freed by finalize_*: nn[8V] (+mu at 8 pos + mu,
 * -mu at 8 pos + 4 + mu), ind[V], lexic2eo[V], nn_eo[4V], nn_oe[4V], eoidx_even[V/2],
 * eoidx_odd[V/2].  The reference's host observables (observables.c) read nn. */
extern int *nn, *ind, *lexic2eo, *nn_eo, *nn_oe, *eoidx_even, *eoidx_odd;

/* cudagaugefix.cu:204 -- upload gf[4V] and trafo[V]; exit(100) on a bad volume,
 * exit(200) on allocation failure, as the reference */
void init_gaugefixing(gfx_su3 *gf, gfx_su3 *trafo);
/* cudagaugefix.cu:381 */
void finalize_gaugefixing(void);
/* cudagaugefix.cu:420 */
void init_thermalization(gfx_su3 *gf);
/* cudagaugefix.cu:556 */
void finalize_thermalization(void);
/* overrelax.cu:677 -- iteration of convergence or -1; prints the reference's lines */
int overrelax_gauge(int maxit, double eps, int checkinterval);
/* overrelax.cu:610 -- returns maxdAdA, sets FUNC, DADA, maxDADA; the arguments name
 * the context's fields (dev_gf, dev_trafo1) */
double calc_functional(void *gf, void *trafo);
/* overrelax.cu:115 */
double calc_plaquette(void *U, int outputyn);
/* simulated_annealing.cu:309 (uses saparam) */
void simannealing_gauge(void);
/* heatbath_thermalization.cu:568 (uses thermparam; writes plaq.txt) */
void thermalize_gauge(void);
/* MersenneTwister.h:47-49 -- parameters from ./MersenneTwister.dat (or $GFX_MT_DAT) */
void init_MT(int n_gaussnumbers, int n_unifnumbers);
void update_MT(void);
void finalize_MT(void);
/* overrelax.cu:830 */
void benchmark(void);

/* No counterpart by name in the reference: the D2H copies its main does inline
 * (cudagaugefix.cu:785-793) and options the reference fixes at compile time. */
int gfx_legacy_get_trafo(gfx_su3 *trafo);      /* g(x), V matrices */
/* the geometry tables above for the current LX, LY, LZ, T (what init_* call); 0 or -1 */
int gfx_legacy_init_tables(void);
int gfx_legacy_get_gauge(gfx_su3 *gf);         /* current links, 4V matrices */
void gfx_legacy_set_precision(int precision);  /* gfx_precision; default GFX_PREC_DOUBLE */
void gfx_legacy_set_omega(double omega);       /* default 1.68 (overrelax.cu:416) */
void gfx_legacy_set_mtseed(unsigned int seed); /* srand(seed) instead of srand(time(NULL)) */
void gfx_legacy_set_nmicro(int nmicro);        /* microcanonical sweeps per SA step, default 0 */
gfx_ctx *gfx_legacy_context(void);

#ifdef __cplusplus
}
#endif
#endif
