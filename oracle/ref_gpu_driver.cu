// ref_gpu_driver.cu -- ctypes entry points into the reference's own CUDA code.
//
// Test infrastructure only.  This file includes the reference's translation unit
// (cudagaugefix.cu, shimmed by oracle/ref_gpu.py) and calls its functions and kernels
// unchanged, so fixtures produced with it are the reference's results.  Two hooks:
//   * srand() inside the reference (seedMTGPU, MersenneTwister.cu:104) uses a seed set
//     here instead of time(NULL), so twister seeds are reproducible;
//   * the reference's main and its ILDG/input-file I/O are not used; stubs satisfy
//     the linker.
#include <assert.h>
#include <cuda_runtime.h>
#include <getopt.h>
#include <math.h>
#include <sys/stat.h>
#include <sys/types.h>
#include <time.h>
#include <unistd.h>

#include <cstdio>
#include <cstdlib>
#include <cstring>

static unsigned int g_mtseed = 1;
static void ref_srand_hook(unsigned int) { srand(g_mtseed); }

// the overrelaxation parameter of dev_overrelax_step (a literal 1.68 in the reference,
// overrelax.cu:416; the shim reads it from here, with the same default)
__constant__ double ref_omega = 1.68;

#define srand(x) ref_srand_hook(x)
#define main cudagaugefix_reference_main
#include "cudagaugefix.cu"
#undef main
#undef srand

extern "C" {
// stubs for the reference's file I/O and input parser (not linked here)
int read_gf_ildg(su3* gf, char* filename) { return -1; }
int write_gf_ildg(su3* gf, char* filename, const int prec) { return -1; }
int read_input(char* conf_file) { return 2; }
// the input-parameter globals that read_input.c defines in the reference
int orxmaxit, orxcheckinterval, orxflag, saflag, thermflag, randseed;
double orxeps;
SAPARAM_LIST saparam;
THERMPARAM_LIST thermparam;

int ref_setup(int lx, int ly, int lz, int lt, double* gf_su3, double* trafo_su3) {
  LX = lx;
  LY = ly;
  LZ = lz;
  T = lt;
  L = lx;
  VOLUME = lx * ly * lz * lt;
  init_gaugefixing((su3*)gf_su3, (su3*)trafo_su3);
  return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

void ref_finalize(void) { finalize_gaugefixing(); }

int ref_overrelax(int maxit, double eps, int checkinterval) {
  return overrelax_gauge(maxit, eps, checkinterval);
}

int ref_set_omega(double w) {
  return cudaMemcpyToSymbol(ref_omega, &w, sizeof(double)) == cudaSuccess ? 0 : -1;
}

double ref_calc_functional(double* out3) {
  double m = calc_functional(dev_gf, dev_trafo1);
  out3[0] = FUNC;
  out3[1] = DADA;
  out3[2] = maxDADA;
  return m;
}

double ref_calc_plaquette(void) { return calc_plaquette(dev_gf, 0); }

// one overrelaxation half-sweep of one parity, as overrelax_gauge launches it
// (overrelax.cu:727-731)
int ref_or_halfsweep(int parity) {
  dim3 block(BLOCK, 1, 1), grid((VOLUME / 2) / BLOCK, 1, 1);
  if (parity == 0)
    dev_overrelax_step<<<grid, block>>>(dev_trafo1, dev_gf, dev_trafo1, dev_eoidx_even,
                                        dev_eoidx_odd, dev_nn);
  else
    dev_overrelax_step<<<grid, block>>>(dev_trafo1, dev_gf, dev_trafo1, dev_eoidx_odd,
                                        dev_eoidx_even, dev_nn);
  return cudaDeviceSynchronize() == cudaSuccess ? 0 : -1;
}

// the gauge transformation as the reference's main copies it back (cudagaugefix.cu:790-792)
void ref_get_trafo(double* trafo_su3) {
  size_t bytes = 6 * VOLUME * sizeof(dev_su3_2v);
  cudaMemcpy(h2d_trafo, dev_trafo1, bytes, cudaMemcpyDeviceToHost);
  from2vtosu3_trafo((su3*)trafo_su3, h2d_trafo);
}

// init_MT with MersenneTwister.dat read from directory `dir`
int ref_init_mt(const char* dir, unsigned int mtseed, int n_gauss, int n_unif) {
  char cwd[4096];
  if (!getcwd(cwd, sizeof(cwd))) return -1;
  if (chdir(dir) != 0) return -1;
  g_mtseed = mtseed;
  init_MT(n_gauss, n_unif);
  int rc = chdir(cwd);
  (void)rc;
  return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

void ref_update_mt(void) { update_MT(); }

void ref_mt_sizes(int* nper_gauss, int* nper_unif) {
  *nper_gauss = N_PER_RNG_GAUSS;
  *nper_unif = N_PER_RNG_UNIF;
}

void ref_read_rng(float* gauss, float* unif) {
  cudaMemcpy(gauss, dev_rndgauss_field, sizeof(float) * RAND_N_GAUSS, cudaMemcpyDeviceToHost);
  cudaMemcpy(unif, dev_rndunif_field, sizeof(float) * RAND_N_UNIF, cudaMemcpyDeviceToHost);
}

// one SA heatbath half-sweep at inverse temperature beta with the current random
// fields, as simannealing_gauge launches it (simulated_annealing.cu:343, 402-426)
int ref_sa_halfsweep(int parity, double beta) {
  cudaMemcpyToSymbol(sa_beta, &beta, sizeof(double));
  dim3 block(BLOCK, 1, 1), grid((VOLUME / 2) / BLOCK, 1, 1);
  if (parity == 0)
    dev_heatbath_sweep<<<grid, block>>>(dev_trafo1, dev_gf, dev_trafo1, dev_eoidx_even,
                                        dev_eoidx_odd, dev_nn, dev_rndgauss_field,
                                        dev_rndunif_field);
  else
    dev_heatbath_sweep<<<grid, block>>>(dev_trafo1, dev_gf, dev_trafo1, dev_eoidx_odd,
                                        dev_eoidx_even, dev_nn, dev_rndgauss_field,
                                        dev_rndunif_field);
  return cudaDeviceSynchronize() == cudaSuccess ? 0 : -1;
}

// simannealing_gauge with the given schedule (simulated_annealing.cu:309-476)
void ref_simanneal(double Tmin, double Tmax, double expo, int N, int checkint) {
  saparam.Tmin = Tmin;
  saparam.Tmax = Tmax;
  saparam.expo = expo;
  saparam.N = N;
  saparam.checkint = checkint;
  simannealing_gauge();
}

// PlantSeeds + random_init_trafo, the reference main's random start
// (cudagaugefix.cu:684, 708)
void ref_random_init_trafo(long seed, int volume, double* trafo_su3) {
  VOLUME = volume;
  PlantSeeds(seed);
  random_init_trafo((su3*)trafo_su3);
}
}
