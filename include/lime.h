/*
 * lime.h -- LIME (Lattice QCD Interchange Message Encapsulation) records, the
 * container of ILDG gauge-field files, with the function names and types of the
 * USQCD c-lime library (1.3.2, the version the reference build links:
 * cudagf.tar:Makefile:5).  libgfx implements this subset itself (gfx_lime.cpp), so
 * the reference's gauge_io.c, which includes "lime.h" and calls exactly these
 * functions (gauge_io.c:18-22, 172-190, 282-437, 484-590), links against libgfx
 * unchanged.
 *
 * Record format (LIME specification): a 144-byte header of big-endian fields,
 *   bytes 0-3   magic number 0x456789ab
 *   bytes 4-5   format version (1)
 *   bytes 6-7   flags: 0x8000 message begin (MB), 0x4000 message end (ME)
 *   bytes 8-15  data length in bytes
 *   bytes 16-143 record type, ASCII, NUL padded
 * followed by the data, zero-padded to a multiple of 8 bytes.
 */
#ifndef GFX_LIME_H
#define GFX_LIME_H

#include <stdint.h>
#include <stdio.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef uint64_t n_uint64_t;

#define LIME_MAGIC_NO 0x456789ab
#define LIME_VERSION 1
#define LIME_HDR_TYPE_BYTES 128
#define LIME_HDR_BYTES 144

/* status codes */
#define LIME_SUCCESS 0
#define LIME_ERR_LAST_NOT_WRITTEN -1
#define LIME_ERR_PARAM -2
#define LIME_ERR_HEADER_NEXT -3
#define LIME_LAST_REC_WRITTEN -4
#define LIME_ERR_WRITE -5
#define LIME_EOR -6
#define LIME_EOF -7
#define LIME_ERR_READ -8
#define LIME_ERR_SEEK -9
#define LIME_ERR_MBME -10
#define LIME_ERR_CLOSE -11

typedef struct LimeRecordHeader {
  int MB_flag, ME_flag;
  char type[LIME_HDR_TYPE_BYTES + 1];
  n_uint64_t data_length;
} LimeRecordHeader;

typedef struct LimeWriter LimeWriter;
typedef struct LimeReader LimeReader;

/* ---- writing ---- */
LimeWriter *limeCreateWriter(FILE *fp);
int limeDestroyWriter(LimeWriter *w);
LimeRecordHeader *limeCreateHeader(int MB_flag, int ME_flag, char *type, n_uint64_t reclen);
void limeDestroyHeader(LimeRecordHeader *h);
/* starts a record; the previous one must be complete */
int limeWriteRecordHeader(LimeRecordHeader *props, LimeWriter *w);
/* appends *nbytes of data to the current record (never past its length); the
 * padding is written when the record is complete.  *nbytes = bytes written. */
int limeWriteRecordData(void *source, n_uint64_t *nbytes, LimeWriter *w);

/* ---- reading ---- */
LimeReader *limeCreateReader(FILE *fp);
void limeDestroyReader(LimeReader *r);
/* advances to the next record header: LIME_SUCCESS, LIME_EOF or an error */
int limeReaderNextRecord(LimeReader *r);
char *limeReaderType(LimeReader *r);
n_uint64_t limeReaderBytes(LimeReader *r);
int limeReaderMBFlag(LimeReader *r);
int limeReaderMEFlag(LimeReader *r);
/* reads up to *nbytes from the current record; *nbytes = bytes read; LIME_EOR
 * when the record had fewer bytes left than asked for */
int limeReaderReadData(void *dest, n_uint64_t *nbytes, LimeReader *r);

#ifdef __cplusplus
}
#endif
#endif
