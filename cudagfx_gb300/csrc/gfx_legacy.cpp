// gfx_legacy.cpp -- the reference's entry points (init_gaugefixing, overrelax_gauge,
// calc_functional, simannealing_gauge, thermalize_gauge, init_MT, ...) on one
// process-wide context, with the reference's globals, printed lines and exit codes.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <ctime>
#include <string>
#include <vector>

#include "../../include/gfx_legacy.h"

extern "C" {
int T, L, LX, LY, LZ, VOLUME;
double PLAQ, FUNC, DADA, maxDADA;
int randseed, orxmaxit, orxcheckinterval, saflag, orxflag, thermflag;
double orxeps;
gfx_saparam_list saparam;
gfx_thermparam_list thermparam;
void *dev_gf, *dev_trafo1;
// host geometry tables of the reference (global.h:104-119), filled by init_gaugefixing
// and init_thermalization as the reference's do (cudagaugefix.cu:285-323, 72-196);
// the reference's host observables (observables.c) walk the lattice through nn
int *nn, *ind, *lexic2eo, *nn_eo, *nn_oe, *eoidx_even, *eoidx_odd;
}

namespace {
gfx_ctx* g_ctx = nullptr;
int g_precision = -1;
double g_omega = 1.68;
int g_nmicro = 0;
bool g_have_mtseed = false;
unsigned int g_mtseed = 0;
int g_n_gauss = 0, g_n_unif = 0;

int legacy_precision() {
  if (g_precision >= 0) return g_precision;
  const char* e = std::getenv("GFX_PRECISION");
  if (e && !std::strcmp(e, "mixed")) return GFX_PREC_MIXED;
  if (e && !std::strcmp(e, "single")) return GFX_PREC_SINGLE;
  return GFX_PREC_DOUBLE;
}

void die(int code, const char* what) {
  std::printf("%s\n", what);
  std::fflush(stdout);
  std::exit(code);
}

void create_context() {
  if (g_ctx) {
    gfx_destroy(g_ctx);
    g_ctx = nullptr;
  }
  // the reference rejects volumes that its fixed block size does not divide
  // (cudagaugefix.cu:344-348, overrelax.cu:687-690)
  if (VOLUME % 128 != 0) die(100, "Error: VOLUME is not a multiple of BLOCK. Aborting...");
  gfx_status s = gfx_create(&g_ctx, LX, LY, LZ, T, legacy_precision(), 12, nullptr);
  if (s == GFX_ERR_BAD_VOLUME) die(100, gfx_last_error(nullptr));
  if (s != GFX_OK) {
    std::printf("Error in init_gaugefixing(): %s. Aborting...\n", gfx_last_error(nullptr));
    std::exit(200);
  }
  dev_gf = (void*)g_ctx;
  dev_trafo1 = (void*)g_ctx;
}

void free_tables() {
  int** t[] = {&nn, &ind, &lexic2eo, &nn_eo, &nn_oe, &eoidx_even, &eoidx_odd};
  for (int** p : t) {
    std::free(*p);
    *p = nullptr;
  }
}

void require_ctx(const char* who) {
  if (!g_ctx) {
    std::fprintf(stderr, "%s called before init_gaugefixing/init_thermalization\n", who);
    std::exit(100);
  }
}
}  // namespace

extern "C" {

// Lexicographic site pos = x + LX (y + LY (z + LZ t)).  nn[8 pos + mu] is the site
// x + mu and nn[8 pos + 4 + mu] the site x - mu (mu = x, y, z, t; periodic); ind[pos] =
// pos; lexic2eo[pos] numbers the sites of each parity (x + y + z + t even / odd) in
// lexicographic order; eoidx_even / eoidx_odd map those numbers back to pos; nn_eo /
// nn_oe hold the eo numbers of the neighbours of even / odd sites, in nn's order.
int gfx_legacy_init_tables(void) {
  free_tables();
  const long v = (long)LX * LY * LZ * T;
  if (LX < 1 || LY < 1 || LZ < 1 || T < 1 || v % 2) return -1;
  nn = (int*)std::malloc(sizeof(int) * 8 * v);
  ind = (int*)std::malloc(sizeof(int) * v);
  lexic2eo = (int*)std::malloc(sizeof(int) * v);
  nn_eo = (int*)std::malloc(sizeof(int) * 4 * v);
  nn_oe = (int*)std::malloc(sizeof(int) * 4 * v);
  eoidx_even = (int*)std::malloc(sizeof(int) * v / 2);
  eoidx_odd = (int*)std::malloc(sizeof(int) * v / 2);
  if (!nn || !ind || !lexic2eo || !nn_eo || !nn_oe || !eoidx_even || !eoidx_odd) {
    free_tables();
    return -1;
  }
  const int ext[4] = {LX, LY, LZ, T};
  const long stride[4] = {1, LX, (long)LX * LY, (long)LX * LY * LZ};
  long ne = 0, no = 0;
  for (long pos = 0; pos < v; pos++) {
    long c[4], r = pos;
    for (int mu = 0; mu < 4; mu++) {
      c[mu] = r % ext[mu];
      r /= ext[mu];
    }
    for (int mu = 0; mu < 4; mu++) {
      const long up = c[mu] + 1 == ext[mu] ? -(ext[mu] - 1) : 1;
      const long dn = c[mu] == 0 ? ext[mu] - 1 : -1;
      nn[8 * pos + mu] = (int)(pos + up * stride[mu]);
      nn[8 * pos + 4 + mu] = (int)(pos + dn * stride[mu]);
    }
    ind[pos] = (int)pos;
    if ((c[0] + c[1] + c[2] + c[3]) % 2 == 0) {
      eoidx_even[ne] = (int)pos;
      lexic2eo[pos] = (int)ne++;
    } else {
      eoidx_odd[no] = (int)pos;
      lexic2eo[pos] = (int)no++;
    }
  }
  for (long pos = 0; pos < v; pos++) {
    int* out = ((pos % LX + (pos / LX) % LY + (pos / stride[2]) % LZ + pos / stride[3]) % 2 == 0
                    ? nn_eo : nn_oe) + 8 * (long)lexic2eo[pos];
    for (int j = 0; j < 8; j++) out[j] = lexic2eo[nn[8 * pos + j]];
  }
  return 0;
}

void init_gaugefixing(gfx_su3* gf, gfx_su3* trafo) {
  create_context();
  if (gfx_legacy_init_tables() != 0) die(200, "Error in init_gaugefixing(): host tables");
  if (gfx_set_links(g_ctx, (const double*)gf) != GFX_OK ||
      gfx_set_trafo(g_ctx, (const double*)trafo) != GFX_OK) {
    std::printf("Error in init_gaugefixing(): %s. Aborting...\n", gfx_last_error(g_ctx));
    std::exit(200);
  }
  std::printf("Allocated gauge field on device\n");
  std::printf("Allocated trafo field 1 on device\n");
  std::printf("VOLUME/BLOCK = %d\n", VOLUME / 128);
}

void finalize_gaugefixing(void) {
  if (g_ctx) gfx_destroy(g_ctx);
  g_ctx = nullptr;
  dev_gf = dev_trafo1 = nullptr;
  free_tables();
}

void init_thermalization(gfx_su3* gf) {
  create_context();
  if (gfx_legacy_init_tables() != 0) die(200, "Error in init_thermalization(): host tables");
  if (gfx_set_links(g_ctx, (const double*)gf) != GFX_OK) {
    std::printf("Error in init_thermalization(): %s. Aborting...\n", gfx_last_error(g_ctx));
    std::exit(200);
  }
  std::printf("Allocated gauge field on device\n");
}

void finalize_thermalization(void) { finalize_gaugefixing(); }

double calc_functional(void* gf, void* trafo) {
  (void)gf;
  (void)trafo;
  require_ctx("calc_functional");
  gfx_functional_t r;
  const int prec = legacy_precision() == GFX_PREC_SINGLE ? 0 : 1;
  if (gfx_functional(g_ctx, GFX_GAUGE_LANDAU, prec, &r) != GFX_OK) {
    std::printf("%s\n", gfx_last_error(g_ctx));
    return 0.0;
  }
  FUNC = r.F;
  DADA = r.dAdA;
  maxDADA = r.maxdAdA;
  return r.maxdAdA;
}

double calc_plaquette(void* U, int outputyn) {
  (void)U;
  require_ctx("calc_plaquette");
  double p = 0.0;
  if (gfx_plaquette(g_ctx, &p) != GFX_OK) std::printf("%s\n", gfx_last_error(g_ctx));
  if (outputyn == 1) std::printf("PLAQ = %.16f\n", p);
  return p;
}

int overrelax_gauge(int maxit, double eps, int checkinterval) {
  require_ctx("overrelax_gauge");
  if ((VOLUME / 2) % 128 != 0) die(100, "Error: VOLUME/2 is not a multiple of BLOCK. Aborting...");
  gfx_or_params p;
  gfx_or_params_default(&p);
  p.maxit = maxit;
  p.eps = eps;
  p.checkinterval = checkinterval;
  p.omega = g_omega;
  p.criterion = GFX_CRIT_MAXDADA;
  const clock_t start = clock();
  gfx_or_result r;
  gfx_status s = gfx_overrelax(g_ctx, &p, &r);
  if (s != GFX_OK && s != GFX_ERR_NOT_CONVERGED) {
    std::printf("%s\n", gfx_last_error(g_ctx));
    return -1;
  }
  const int n = gfx_or_history(g_ctx, nullptr, 0);
  std::vector<gfx_check_record> h(n);
  gfx_or_history(g_ctx, h.data(), n);
  for (const auto& c : h)
    std::printf("iter %6d:\t FUNC = %.16e \t dAdA = %.16e\t max(dAdA) = %.16e\n", c.iter, c.F,
                c.dAdA, c.maxdAdA);
  FUNC = r.final_values.F;
  DADA = r.final_values.dAdA;
  maxDADA = r.final_values.maxdAdA;
  const double el = (double)(clock() - start) / CLOCKS_PER_SEC;
  if (r.converged) {
    std::printf("CONVERGENCE!\nFinal values: F = %.16e dAdA = %.16e, maxdAdA = %.16e\n", FUNC,
                DADA, maxDADA);
    std::printf("Overrelaxation finished after %f sec\n", el);
    return r.iterations;
  }
  std::printf("Overrelaxation finished after %f sec\n", el);
  if (r.iterations < 0)
    std::printf("FAIL! Gauge condition not reached!\nFinal values: F = %.16e dAdA = %.16e, "
                "maxdAdA = %.16e\n",
                FUNC, DADA, maxDADA);
  return r.iterations;
}

void init_MT(int n_gaussnumbers, int n_unifnumbers) {
  require_ctx("init_MT");
  std::printf("Initializing MT random number generator...\n");
  const char* path = std::getenv("GFX_MT_DAT");
  if (!path) path = "MersenneTwister.dat";
  std::printf("Loading GPU twisters configurations from file %s...\n", path);
  if (gfx_mt_load_file(g_ctx, path) != GFX_OK) {
    // loadMTGPU (MersenneTwister.cu:79-92)
    std::printf("initMTGPU(): failed to open %s\n", path);
    std::printf("FAILED\n");
    std::exit(0);
  }
  unsigned int seed = g_mtseed;
  if (!g_have_mtseed) {
    const char* e = std::getenv("GFX_MT_SEED");
    seed = e ? (unsigned int)std::strtoul(e, nullptr, 10) : (unsigned int)time(nullptr);
  }
  gfx_mt_seed(g_ctx, seed);
  g_n_gauss = n_gaussnumbers;
  g_n_unif = n_unifnumbers;
  if (gfx_mt_init(g_ctx, n_gaussnumbers, n_unifnumbers) != GFX_OK)
    std::printf("%s\n", gfx_last_error(g_ctx));
  int ng = 0, nu = 0;
  gfx_mt_sizes(g_ctx, &ng, &nu);
  std::printf("No. of gauss random numbers: %d\n", 4096 * ng);
  std::printf("No. of unif. dist. random numbers: %d\n", 4096 * nu);
}

void update_MT(void) {
  require_ctx("update_MT");
  if (gfx_mt_update(g_ctx) != GFX_OK) std::printf("%s\n", gfx_last_error(g_ctx));
}

void finalize_MT(void) {}

void simannealing_gauge(void) {
  require_ctx("simannealing_gauge");
  if ((VOLUME / 2) % 128 != 0) die(100, "Error: VOLUME/2 is not a multiple of BLOCK. Aborting...");
  gfx_sa_params p;
  p.Tmin = saparam.Tmin;
  p.Tmax = saparam.Tmax;
  p.expo = saparam.expo;
  p.N = saparam.N;
  p.checkint = saparam.checkint > 0 ? saparam.checkint : 1;
  p.nmicro = g_nmicro;
  const clock_t start = clock();
  // step i, then the functional when i % checkint == 0 (simulated_annealing.cu:341-466)
  int i = 0;
  while (i < p.N) {
    int next = (i % p.checkint == 0) ? i + 1 : ((i / p.checkint) + 1) * p.checkint + 1;
    if (next > p.N) next = p.N;
    // run steps i .. next-1; the last one of the range is a check step or N-1
    int last = next - 1;
    if (gfx_simanneal_range(g_ctx, &p, i, next - i) != GFX_OK) {
      std::printf("%s\n", gfx_last_error(g_ctx));
      return;
    }
    if (last % p.checkint == 0) {
      const double m = calc_functional(dev_gf, dev_trafo1);
      std::printf("iter %6d:\t FUNC = %.16e \t dAdA = %.16e\t max(dAdA) = %.16e\n", last, FUNC,
                  DADA, m);
    }
    i = next;
  }
  std::printf("SA finished after %f sec\n", (double)(clock() - start) / CLOCKS_PER_SEC);
}

void thermalize_gauge(void) {
  require_ctx("thermalize_gauge");
  if ((VOLUME / 2) % 128 != 0) die(100, "Error: VOLUME/2 is not a multiple of BLOCK. Aborting...");
  FILE* pf = std::fopen("plaq.txt", "w");
  if (!pf) std::fprintf(stderr, "Could not open file 'plaq.txt'\n");
  const clock_t start = clock();
  std::printf("Setting beta to %f\n", thermparam.beta);
  gfx_therm_params tp;
  tp.Nsweep = 1;
  tp.checkint = 0;
  tp.beta = thermparam.beta;
  tp.variant = GFX_HB_REFERENCE;
  tp.precision = 0;
  const int ck = thermparam.checkint > 0 ? thermparam.checkint : 1;
  for (int i = 0; i < thermparam.Nsweep; i++) {
    if (gfx_thermalize(g_ctx, &tp, nullptr, 0) != GFX_OK) {
      std::printf("%s\n", gfx_last_error(g_ctx));
      break;
    }
    if (i % ck == 0) {
      const double plaq = calc_plaquette(dev_gf, 0);
      if (pf) std::fprintf(pf, "%d %.16e\n", i, plaq);
      std::printf("therm %6d:\t PLAQ = %.16e\n", i, plaq);
    }
  }
  if (pf) std::fclose(pf);
  std::printf("Thermalization finished after %f sec\n", (double)(clock() - start) / CLOCKS_PER_SEC);
}

void benchmark(void) {
  require_ctx("benchmark");
  std::printf("Doing small benchmark...");
  gfx_synchronize(g_ctx);
  const clock_t start = clock();
  const int prec = legacy_precision() == GFX_PREC_DOUBLE ? 1 : 0;
  gfx_or_sweeps(g_ctx, 100, g_omega, GFX_GAUGE_LANDAU, prec);
  const double el = (double)(clock() - start) / CLOCKS_PER_SEC;
  std::printf("Done\n");
  // 4766 flop per site update (overrelax.cu:897)
  std::printf("Benchmark: %f Gflops\n", 4766.0 * VOLUME * 100 / el / 1.0e9);
}

int gfx_legacy_get_trafo(gfx_su3* trafo) {
  if (!g_ctx) return GFX_ERR_STATE;
  return gfx_get_trafo(g_ctx, (double*)trafo);
}
int gfx_legacy_get_gauge(gfx_su3* gf) {
  if (!g_ctx) return GFX_ERR_STATE;
  return gfx_get_links(g_ctx, (double*)gf);
}
void gfx_legacy_set_precision(int precision) { g_precision = precision; }
void gfx_legacy_set_omega(double omega) { g_omega = omega; }
void gfx_legacy_set_mtseed(unsigned int seed) {
  g_have_mtseed = true;
  g_mtseed = seed;
}
void gfx_legacy_set_nmicro(int nmicro) { g_nmicro = nmicro; }
gfx_ctx* gfx_legacy_context(void) { return g_ctx; }

}  // extern "C"
