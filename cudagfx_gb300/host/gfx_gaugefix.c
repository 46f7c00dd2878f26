/*
 * gfx_gaugefix -- the cudagfx gauge-fixing program on libgfx: the steps of the
 * reference's main (cudagaugefix.cu:599-828) through the reference-named entry
 * points of gfx_legacy.h and the file functions of gfx_io.h.
 *
 *   gfx_gaugefix -i input.in -f config.ildg [-d device] [-p double|single|mixed]
 *                [-w omega] [-m mtseed] [-o output.ildg]
 *
 * input.in uses the reference's grammar (read_input.l): T = .., L = ..,
 * RandSeed = .., and the blocks BeginORXInit .. EndORXInit (eps, ckinterval,
 * maxit), BeginSAInit .. EndSAInit (Tmin, Tmax, ckinterval, Nstep, expo) and
 * BeginTHERMInit .. EndTHERMInit (Nsweep, Nsave, ckinterval, beta, start =
 * hot|cold); '#' starts a comment.  Real values are read as float, as the
 * reference's lexer does (sscanf "%f" into a float).
 *
 * Without a THERM block: g starts from the reference's random transformation
 * (Park-Miller, seed RandSeed), simulated annealing runs when the SA block is
 * present, overrelaxation when the ORX block is, and the gauge-fixed field
 * g U g^+ is written (64-bit ILDG) to landau_<config> or the -o path.  With a
 * THERM block the links are thermalized from a cold or hot start and the
 * thermalized field is written (the reference writes nothing,
 * cudagaugefix.cu:702-705).
 * Exit codes as the reference: 1 configuration unreadable, 255 (-1) output file
 * present, 300 gauge condition not reached, 400 output not written (a process
 * status keeps the low 8 bits: 44 and 144); 2 bad input file or option.
 */
#include <getopt.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <sys/stat.h>

#include "gfx_io.h"
#include "gfx_legacy.h"

static int line_no = 0;

static void input_error(const char *line) {
  printf("Parsing error in line %d\nAborting...!\n%s\n", line_no, line);
  exit(2);
}

/* "key = value" with optional blanks; returns 1 and the value text */
static int key_value(const char *s, const char *key, const char **val) {
  size_t n = strlen(key);
  while (*s == ' ' || *s == '\t') s++;
  if (strncmp(s, key, n) != 0) return 0;
  s += n;
  while (*s == ' ' || *s == '\t') s++;
  if (*s != '=') return 0;
  s++;
  while (*s == ' ' || *s == '\t') s++;
  *val = s;
  return 1;
}

static float as_float(const char *v, const char *line) {
  char *end;
  float f = strtof(v, &end);
  if (end == v) input_error(line);
  return f;
}
static int as_int(const char *v, const char *line) {
  char *end;
  long k = strtol(v, &end, 10);
  if (end == v) input_error(line);
  return (int)k;
}

/* the grammar of read_input.l, restated as a line parser */
static int read_input_file(const char *path) {
  FILE *f = fopen(path, "r");
  char buf[512];
  enum { TOP, ORX, SA, THERM } block = TOP;
  if (!f) return 2;
  while (fgets(buf, sizeof(buf), f)) {
    const char *v;
    char *hash = strchr(buf, '#');
    line_no++;
    if (hash) *hash = '\0';
    buf[strcspn(buf, "\r\n")] = '\0';
    {
      const char *p = buf;
      while (*p == ' ' || *p == '\t') p++;
      if (!*p) continue;
    }
    if (block == TOP) {
      if (key_value(buf, "T", &v)) T = as_int(v, buf);
      else if (key_value(buf, "L", &v)) L = as_int(v, buf);
      else if (key_value(buf, "RandSeed", &v)) randseed = as_int(v, buf);
      else if (strstr(buf, "BeginORXInit")) block = ORX;
      else if (strstr(buf, "BeginSAInit")) block = SA;
      else if (strstr(buf, "BeginTHERMInit")) block = THERM;
      else input_error(buf);
    } else if (block == ORX) {
      if (key_value(buf, "eps", &v)) orxeps = as_float(v, buf);
      else if (key_value(buf, "maxit", &v)) orxmaxit = as_int(v, buf);
      else if (key_value(buf, "ckinterval", &v)) orxcheckinterval = as_int(v, buf);
      else if (strstr(buf, "EndORXInit")) {
        orxflag = 1;
        block = TOP;
      } else input_error(buf);
    } else if (block == SA) {
      if (key_value(buf, "Tmin", &v)) saparam.Tmin = as_float(v, buf);
      else if (key_value(buf, "Tmax", &v)) saparam.Tmax = as_float(v, buf);
      else if (key_value(buf, "Nstep", &v)) saparam.N = as_int(v, buf);
      else if (key_value(buf, "ckinterval", &v)) saparam.checkint = as_int(v, buf);
      else if (key_value(buf, "expo", &v)) saparam.expo = as_float(v, buf);
      else if (strstr(buf, "EndSAInit")) {
        saflag = 1;
        block = TOP;
      } else input_error(buf);
    } else {
      if (key_value(buf, "Nsweep", &v)) thermparam.Nsweep = as_int(v, buf);
      else if (key_value(buf, "Nsave", &v)) thermparam.Nsave = as_int(v, buf);
      else if (key_value(buf, "ckinterval", &v)) thermparam.checkint = as_int(v, buf);
      else if (key_value(buf, "beta", &v)) thermparam.beta = as_float(v, buf);
      else if (key_value(buf, "start", &v)) thermparam.startcond = strncmp(v, "hot", 3) == 0;
      else if (strstr(buf, "EndTHERMInit")) {
        thermflag = 1;
        block = TOP;
      } else input_error(buf);
    }
  }
  fclose(f);
  if (block != TOP) {
    printf("Input file ends inside a block\n");
    return 2;
  }
  LX = LY = LZ = L;
  VOLUME = LX * LY * LZ * T;
  return 0;
}

static void usage(void) {
  printf("usage: gfx_gaugefix -i input -f config.ildg [-d device] [-p double|single|mixed]\n"
         "                    [-w omega] [-m mtseed] [-o output.ildg]\n");
  exit(2);
}

int main(int argc, char *argv[]) {
  char input[512] = "", config[512] = "", output[600] = "";
  int device = 0, c;
  while ((c = getopt(argc, argv, "h?i:d:f:p:w:m:o:")) != -1) {
    switch (c) {
      case 'i': snprintf(input, sizeof(input), "%s", optarg); break;
      case 'd': device = atoi(optarg); break;
      case 'f': snprintf(config, sizeof(config), "%s", optarg); break;
      case 'p':
        if (!strcmp(optarg, "double")) gfx_legacy_set_precision(GFX_PREC_DOUBLE);
        else if (!strcmp(optarg, "single")) gfx_legacy_set_precision(GFX_PREC_SINGLE);
        else if (!strcmp(optarg, "mixed")) gfx_legacy_set_precision(GFX_PREC_MIXED);
        else usage();
        break;
      case 'w': gfx_legacy_set_omega(atof(optarg)); break;
      case 'm': gfx_legacy_set_mtseed((unsigned)strtoul(optarg, NULL, 10)); break;
      case 'o': snprintf(output, sizeof(output), "%s", optarg); break;
      default: usage();
    }
  }
  if (!input[0] || !config[0]) usage();
  printf("setting device to %d\n", device);
  if (gfx_set_device(device) != GFX_OK) {
    printf("%s\n", gfx_last_error(NULL));
    return 2;
  }
  if (read_input_file(input) != 0) {
    printf("Cannot read input file %s\n", input);
    return 2;
  }
  printf("LX = %d, LY = %d, LZ = %d, T = %d\n", LX, LY, LZ, T);
  if (!output[0]) {
    /* landau_<config> beside the config, as the reference names it */
    const char *slash = strrchr(config, '/');
    size_t dir = slash ? (size_t)(slash - config + 1) : 0;
    snprintf(output, sizeof(output), "%.*s%s%s", (int)dir, config,
             thermflag ? "thermalized_" : "landau_", config + dir);
  }

  gfx_su3 *gf = (gfx_su3 *)malloc(sizeof(gfx_su3) * 4 * (size_t)VOLUME);
  gfx_su3 *trafo = (gfx_su3 *)malloc(sizeof(gfx_su3) * (size_t)VOLUME);
  const int dims[4] = {LX, LY, LZ, T};
  gfx_ildg_info info;
  if (!gf || !trafo) return 2;
  if (gfx_ildg_read(config, dims, (double *)gf, &info) != GFX_OK) {
    printf("Error reading configuration from %s\n%s\n", config, gfx_last_error(NULL));
    return 1;
  }
  struct stat st;
  if (stat(output, &st) == 0) {
    printf(" output file %s is present, exiting...\n", output);
    return 255;
  }
  printf("Setting random seed to %d\n", randseed);

  if (thermflag) {
    if (thermparam.startcond == 0) gfx_unit_init((double *)gf, 4 * (long)VOLUME);
    else gfx_random_init_reference(randseed, (double *)gf, 4 * (long)VOLUME);
    init_thermalization(gf);
    init_MT(4 * VOLUME / 2, 4 * 4 * VOLUME / 2);
    calc_plaquette(dev_gf, 1);
    thermalize_gauge();
    if (gfx_write_links_ildg(gfx_legacy_context(), output, 64, thermparam.beta) != GFX_OK) {
      fprintf(stderr, "Error writing gauge field. Aborting...\n");
      return 400;
    }
    printf("Thermalized field written to %s\n", output);
    finalize_thermalization();
  } else {
    gfx_random_init_reference(randseed, (double *)trafo, VOLUME);
    init_gaugefixing(gf, trafo);
    init_MT(VOLUME / 2, 4 * VOLUME / 2);
    calc_plaquette(dev_gf, 1);
    if (saflag) {
      printf("Starting simulated annealing...\n");
      printf("Tmin = %f, Tmax = %f, N = %d, expo = %f\n", saparam.Tmin, saparam.Tmax, saparam.N,
             saparam.expo);
      simannealing_gauge();
    }
    if (orxflag) {
      printf("Starting overrelaxation...\n");
      if (overrelax_gauge(orxmaxit, orxeps, orxcheckinterval) < 0) {
        printf("Gauge condition not reached. Aborting...\n");
        finalize_gaugefixing();
        return 300;
      }
    }
    calc_functional(dev_gf, dev_trafo1);
    PLAQ = calc_plaquette(dev_gf, 0);
    printf("Final values:\n");
    printf("PLAQ = %.16f\n", PLAQ);
    printf("F = %.16e \t dAdA = %.16e\t max(dAdA) = %.16e\n", FUNC, DADA, maxDADA);
    printf("Writing out the gauge fixed field ...");
    if (gfx_write_fixed_ildg(gfx_legacy_context(), output, 64, info.beta) != GFX_OK) {
      fprintf(stderr, "Error writing gauge field. Aborting...\n%s\n", gfx_last_error(NULL));
      return 400;
    }
    printf("done.\n");
    finalize_gaugefixing();
  }
  free(trafo);
  free(gf);
  return 0;
}
