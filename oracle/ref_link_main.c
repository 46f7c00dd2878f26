/*
 * ref_link_main.c -- the reference's host-side program flow (cudagaugefix.cu:599-828)
 * over the reference's own host C files (read_input.c, gauge_io.c, spinor_io.c,
 * cksum.c, su3manip.c, observables.c, rngs.c, complex.c), compiled unchanged and
 * linked against libgfx.so, which supplies the CUDA side: init_gaugefixing,
 * init_MT, simannealing_gauge, overrelax_gauge, calc_plaquette,
 * finalize_gaugefixing, the device globals and the LIME records gauge_io.c needs.
 * It shows the drop-in boundary at link level; the recipe (oracle/build.py)
 * builds it into oracle/_ref/.  Test infrastructure only.
 */
#define MAIN_PROGRAM
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <sys/stat.h>

#include "cudaglobal.h"
#include "global.h"
#include "read_input.h"
#include "gauge_io.h"
#include "observables.h"
#include "su3manip.h"
#include "rngs.h"

/* the CUDA side, as the reference declares it (cudagaugefix.cu:204-560, overrelax.cu,
 * simulated_annealing.cu, MersenneTwister.h); dev_gf and dev_trafo1 come from global.h */
void init_gaugefixing(su3 *gf, su3 *trafo);
void finalize_gaugefixing(void);
int overrelax_gauge(int maxit, double eps, int checkinterval);
double calc_plaquette(dev_su3_2v *U, int print);
void simannealing_gauge(void);
void init_MT(int n_gauss, int n_unif);
/* the D2H of g that the reference's main does with a raw cudaMemcpy (:785-793) */
int gfx_legacy_get_trafo(su3 *trafo);

int main(int argc, char *argv[]) {
  if (argc != 3) {
    printf("usage: ref_gaugefix input.in config.ildg\n");
    return 2;
  }
  char fixedname[600];
  snprintf(fixedname, sizeof(fixedname), "landau_%s", argv[2]);
  read_input(argv[1]);
  su3 *gf = (su3 *)malloc(4 * VOLUME * sizeof(su3));
  su3 *trafo = (su3 *)malloc(VOLUME * sizeof(su3));
  if (read_gf_ildg(gf, argv[2]) != 0) return 1;
  struct stat st;
  if (stat(fixedname, &st) == 0) return 255;
  PlantSeeds(randseed);
  random_init_trafo(trafo);
  init_gaugefixing(gf, trafo);
  init_MT(VOLUME / 2, 4 * VOLUME / 2);
  calc_plaquette(dev_gf, 1);
  if (saflag == 1) simannealing_gauge();
  if (orxflag == 1 && overrelax_gauge(orxmaxit, orxeps, orxcheckinterval) < 0) return 300;
  gfx_legacy_get_trafo(trafo);
  g_trafo(gf, trafo);
  PLAQ = mean_plaq(gf);
  DADA = dAdA(gf);
  FUNC = gauge_functional(gf);
  printf("Final HOST values:\nPLAQ = %.16f\nF = %.16e \t dAdA = %.16e\n", PLAQ, FUNC, DADA);
  if (write_gf_ildg(gf, fixedname, 64) != 0) return 400;
  finalize_gaugefixing();
  free(trafo);
  free(gf);
  return 0;
}
