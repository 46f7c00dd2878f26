/*
 * gfx_io.h -- gauge-field files of the cudagfx host code, implemented in libgfx:
 * ILDG (LIME records "ildg-format", "xlf-info", "ildg-binary-data"; gauge_io.c:139-595)
 * and BQCD (one big-endian file per time slice, an info file with POSIX cksum
 * checksums; gauge_io.c:602-1108, cksum.c), plus the device-side steps around them
 * (load links into a context; write the gauge-fixed field, the g and the twister
 * state as a checkpoint).
 *
 * A field is the reference's host layout (gfx.h): 4*V su3 of 18 doubles, link
 * (pos, mu) at 4*pos+mu, pos = x + LX*(y + LY*(z + LZ*t)) -- the ILDG site order.
 * dims = {LX, LY, LZ, T}.  Errors are GFX_ERR_IO (file missing, truncated,
 * malformed or of another lattice) with the reason in gfx_last_error(NULL);
 * the reference prints and exits instead (exit(120) wrong extent, exit(500)
 * corrupt, gauge_io.c:312-338, 431-440).
 */
#ifndef GFX_IO_H
#define GFX_IO_H

#include <stddef.h>
#include <stdint.h>

#include "gfx.h"

#ifdef __cplusplus
extern "C" {
#endif

/* What an ILDG file's metadata records say (read_gf_header_ildg, gauge_io.c:139-242). */
typedef struct {
  int dims[4];       /* lx, ly, lz, lt of <ildgFormat> */
  int precision;     /* 32 or 64 (0 when the record gives none) */
  double plaquette;  /* xlf-info "plaquette = ..." (0 when absent) */
  double beta;       /* xlf-info "beta = ..." (0 when absent) */
  uint64_t data_bytes; /* length of the ildg-binary-data record */
} gfx_ildg_info;

gfx_status gfx_ildg_read_info(const char *path, gfx_ildg_info *info);

/* Read the links (read_gf_ildg, gauge_io.c:245-448).  dims must match the file;
 * 32-bit data is widened to double.  info may be NULL.  The reference's 32-bit
 * branch stores record 4i+3 into link i and reads past the data block
 * (gauge_io.c:384-405); this reader stores record i into link i. */
gfx_status gfx_ildg_read(const char *path, const int dims[4], double *links, gfx_ildg_info *info);

/* Write the links (write_gf_ildg, gauge_io.c:452-595): the same three records,
 * byte for byte, with precision 64 or 32 (values rounded to float). */
gfx_status gfx_ildg_write(const char *path, const int dims[4], const double *links, int precision,
                          double plaquette, double beta);

/* POSIX cksum (the CRC of cksum.c): CRC-32, polynomial 0x04C11DB7, bits most
 * significant first, followed by the byte count, complemented. */
typedef struct {
  uint32_t crc;
  uint64_t bytes;
} gfx_cksum_state;
void gfx_cksum_init(gfx_cksum_state *s);
void gfx_cksum_add(gfx_cksum_state *s, const void *data, size_t n);
/* the checksum as cksum(1) prints it (the state is left unchanged) */
uint32_t gfx_cksum_get(const gfx_cksum_state *s);

typedef struct {
  char file[80];     /* <basename>.<ttt>.u or .g */
  uint64_t sum;      /* POSIX cksum of the slice's big-endian bytes */
  uint64_t bytes;
} gfx_slice_cksum;

/* BQCD: <basename>.<ttt>.u = time slice t, 4*LX*LY*LZ big-endian su3; the info
 * file <basename>.info with the dimensions, beta, plaquette and a checksum per
 * slice (write_gf_bqcd, write_conf_info, gauge_io.c:710-833).  cks (lt entries)
 * may be NULL. */
gfx_status gfx_bqcd_write(const char *basename, const int dims[4], const double *links,
                          double plaquette, double beta, int ensemble, gfx_slice_cksum *cks);
/* read_gf_bqcd (gauge_io.c:837-884): the slices and their checksums */
gfx_status gfx_bqcd_read(const char *basename, const int dims[4], double *links,
                         gfx_slice_cksum *cks);
/* read_trafo_bqcd (gauge_io.c:956-1002): a gauge transformation, V su3 in
 * <basename>.<ttt>.g files, with its checksums */
gfx_status gfx_bqcd_read_trafo(const char *basename, const int dims[4], double *trafo,
                               gfx_slice_cksum *cks);
gfx_status gfx_bqcd_write_trafo(const char *basename, const int dims[4], const double *trafo,
                                gfx_slice_cksum *cks);

/* An info file (read_conf_info, gauge_io.c:889-947). */
typedef struct {
  int run;
  int dims[4]; /* lx, ly, lz, lt */
  double beta, plaquette;
} gfx_bqcd_info;
/* cks: up to cap slice checksums, in file order; *ncks = the number found */
gfx_status gfx_bqcd_read_info(const char *path, gfx_bqcd_info *info, gfx_slice_cksum *cks,
                              int cap, int *ncks);

/* ---- device-side steps ---- */
/* the links of an ILDG file into a context (read + gfx_set_links) */
gfx_status gfx_load_links_ildg(gfx_ctx *ctx, const char *path, gfx_ildg_info *info);
/* The gauge-fixed field g U g^+ (the reference main's host g_trafo and
 * write_gf_ildg, cudagaugefix.cu:785-810), formed on the device: the context's
 * links are left as they were.  The plaquette written is the fixed field's. */
gfx_status gfx_write_fixed_ildg(gfx_ctx *ctx, const char *path, int precision, double beta);
/* The context's links as an ILDG file (e.g. a thermalized configuration, which
 * the reference never writes, cudagaugefix.cu:702-705). */
gfx_status gfx_write_links_ildg(gfx_ctx *ctx, const char *path, int precision, double beta);

/* Checkpoint: links, g and (when initialised) the twister bank with its
 * generated fields, as one LIME file with records "gfx-checkpoint-info",
 * "gfx-links", "gfx-trafo" and "gfx-mt-state".  Restoring it into a context of
 * the same lattice continues bit for bit where the saved one stood. */
gfx_status gfx_checkpoint_save(gfx_ctx *ctx, const char *path);
gfx_status gfx_checkpoint_load(gfx_ctx *ctx, const char *path);

#ifdef __cplusplus
}
#endif
#endif
