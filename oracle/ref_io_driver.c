/*
 * ref_io_driver.c -- entry points into the reference's own file code (gauge_io.c,
 * spinor_io.c, cksum.c), compiled unchanged into oracle/_ref/libref_io.so together
 * with libgfx's LIME implementation (cudagfx_gb300/csrc/gfx_lime.cpp) in place of
 * the absent c-lime.  Each function sets the reference's lattice globals and calls
 * one reference routine.  Test infrastructure only: it generates the golden file
 * hashes the I/O tests compare against.
 */
#include <stdlib.h>
#include <string.h>

#include "cudaglobal.h"
#include "global.h"
#include "gauge_io.h"

extern int LX, LY, LZ, T, VOLUME;
extern double PLAQ, BETA;
extern void CKSUM_INIT(void);
extern void CKSUM_ADD(void *memptr, INT8 *nbytes);
extern void CKSUM_GET(INT8 *total_crc, INT8 *total_bytes);

static void set_dims(const int *d) {
  LX = d[0];
  LY = d[1];
  LZ = d[2];
  T = d[3];
  VOLUME = LX * LY * LZ * T;
}

/* write_gf_ildg (gauge_io.c:452-595) */
int ref_io_write_ildg(const char *path, const int *dims, double *links, int prec, double plaq,
                      double beta) {
  set_dims(dims);
  PLAQ = plaq;
  BETA = beta;
  return write_gf_ildg((su3 *)links, (char *)path, prec);
}

/* read_gf_ildg (gauge_io.c:245-448); 64-bit files only (the 32-bit branch reads
 * past the data block, gauge_io.c:384-405) */
int ref_io_read_ildg(const char *path, const int *dims, double *links, double *plaq,
                     double *beta) {
  set_dims(dims);
  int r = read_gf_ildg((su3 *)links, (char *)path);
  *plaq = PLAQ;
  *beta = BETA;
  return r;
}

/* write_gf_bqcd (gauge_io.c:710-792) */
int ref_io_write_bqcd(const char *base, const int *dims, double *links, double plaq,
                      double beta) {
  set_dims(dims);
  PLAQ = plaq;
  BETA = beta;
  return write_gf_bqcd((su3 *)links, (char *)base);
}

/* read_gf_bqcd (gauge_io.c:837-884): links and the per-slice checksums */
int ref_io_read_bqcd(const char *base, const int *dims, double *links, unsigned long *sums) {
  set_dims(dims);
  type_cksum *cks = (type_cksum *)calloc(T, sizeof(type_cksum));
  type_conf_info ci;
  memset(&ci, 0, sizeof(ci));
  int r = read_gf_bqcd((su3 *)links, (char *)base, ci, cks);
  for (int t = 0; t < T; t++) sums[t] = (unsigned long)cks[t].sum;
  free(cks);
  return r;
}

/* cksum.c over one buffer */
void ref_io_cksum(const void *data, long n, unsigned long *crc, unsigned long *bytes) {
  INT8 nb = (INT8)n, c = 0, b = 0;
  CKSUM_INIT();
  if (n > 0) CKSUM_ADD((void *)data, &nb);
  CKSUM_GET(&c, &b);
  *crc = (unsigned long)c;
  *bytes = (unsigned long)b;
}
