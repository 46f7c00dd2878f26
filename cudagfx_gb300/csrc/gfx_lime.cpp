// gfx_lime.cpp -- LIME record reader and writer (format in include/lime.h), written
// from the LIME record specification.  Plain stdio, no seeking required for
// writing; the reader skips unread data and padding with fseek or, on a pipe,
// by reading it.
#include <cstdlib>
#include <cstring>
#include <new>

#include "../../include/lime.h"

namespace {

void put_be(unsigned char* p, uint64_t v, int n) {
  for (int k = n - 1; k >= 0; k--) {
    p[k] = (unsigned char)(v & 0xff);
    v >>= 8;
  }
}
uint64_t get_be(const unsigned char* p, int n) {
  uint64_t v = 0;
  for (int k = 0; k < n; k++) v = (v << 8) | p[k];
  return v;
}
uint64_t padding(uint64_t n) { return (8 - (n & 7)) & 7; }

// skip n bytes of the input
bool skip(FILE* fp, uint64_t n) {
  if (n == 0) return true;
  if (fseeko(fp, (off_t)n, SEEK_CUR) == 0) return true;
  unsigned char buf[4096];
  while (n > 0) {
    const size_t k = n < sizeof(buf) ? (size_t)n : sizeof(buf);
    if (fread(buf, 1, k, fp) != k) return false;
    n -= k;
  }
  return true;
}

}  // namespace

struct LimeWriter {
  FILE* fp;
  bool in_record;       // a header was written and its data is not complete
  uint64_t remaining;   // data bytes still owed to the current record
  uint64_t pad;         // padding after the current record
};

struct LimeReader {
  FILE* fp;
  bool have_header;
  LimeRecordHeader hdr;
  uint64_t remaining;  // unread data bytes of the current record
  uint64_t pad;
};

extern "C" {

LimeWriter* limeCreateWriter(FILE* fp) {
  if (!fp) return nullptr;
  LimeWriter* w = new (std::nothrow) LimeWriter();
  if (!w) return nullptr;
  w->fp = fp;
  return w;
}

int limeDestroyWriter(LimeWriter* w) {
  if (!w) return LIME_ERR_PARAM;
  const int incomplete = w->in_record && w->remaining > 0;
  delete w;
  return incomplete ? LIME_ERR_LAST_NOT_WRITTEN : LIME_SUCCESS;
}

LimeRecordHeader* limeCreateHeader(int MB_flag, int ME_flag, char* type, n_uint64_t reclen) {
  LimeRecordHeader* h = new (std::nothrow) LimeRecordHeader();
  if (!h) return nullptr;
  h->MB_flag = MB_flag ? 1 : 0;
  h->ME_flag = ME_flag ? 1 : 0;
  std::strncpy(h->type, type ? type : "", LIME_HDR_TYPE_BYTES);
  h->type[LIME_HDR_TYPE_BYTES] = '\0';
  h->data_length = reclen;
  return h;
}

void limeDestroyHeader(LimeRecordHeader* h) { delete h; }

int limeWriteRecordHeader(LimeRecordHeader* props, LimeWriter* w) {
  if (!props || !w) return LIME_ERR_PARAM;
  if (w->in_record && w->remaining > 0) return LIME_ERR_LAST_NOT_WRITTEN;
  unsigned char h[LIME_HDR_BYTES];
  std::memset(h, 0, sizeof(h));
  put_be(h, LIME_MAGIC_NO, 4);
  put_be(h + 4, LIME_VERSION, 2);
  put_be(h + 6, (props->MB_flag ? 0x8000u : 0u) | (props->ME_flag ? 0x4000u : 0u), 2);
  put_be(h + 8, props->data_length, 8);
  std::memcpy(h + 16, props->type, std::strlen(props->type));
  if (fwrite(h, 1, sizeof(h), w->fp) != sizeof(h)) return LIME_ERR_WRITE;
  w->in_record = true;
  w->remaining = props->data_length;
  w->pad = padding(props->data_length);
  if (w->remaining == 0 && w->pad == 0) w->in_record = false;
  return LIME_SUCCESS;
}

int limeWriteRecordData(void* source, n_uint64_t* nbytes, LimeWriter* w) {
  if (!source || !nbytes || !w) return LIME_ERR_PARAM;
  if (!w->in_record) {
    *nbytes = 0;
    return LIME_ERR_HEADER_NEXT;
  }
  uint64_t n = *nbytes;
  if (n > w->remaining) n = w->remaining;
  const size_t done = fwrite(source, 1, (size_t)n, w->fp);
  *nbytes = done;
  w->remaining -= done;
  if (done != n) return LIME_ERR_WRITE;
  if (w->remaining == 0) {
    static const unsigned char zeros[8] = {0};
    if (w->pad && fwrite(zeros, 1, (size_t)w->pad, w->fp) != w->pad) return LIME_ERR_WRITE;
    w->in_record = false;
  }
  return LIME_SUCCESS;
}

LimeReader* limeCreateReader(FILE* fp) {
  if (!fp) return nullptr;
  LimeReader* r = new (std::nothrow) LimeReader();
  if (!r) return nullptr;
  r->fp = fp;
  return r;
}

void limeDestroyReader(LimeReader* r) { delete r; }

int limeReaderNextRecord(LimeReader* r) {
  if (!r) return LIME_ERR_PARAM;
  if (r->have_header && !skip(r->fp, r->remaining + r->pad)) return LIME_ERR_SEEK;
  r->have_header = false;
  unsigned char h[LIME_HDR_BYTES];
  const size_t got = fread(h, 1, sizeof(h), r->fp);
  if (got == 0 && feof(r->fp)) return LIME_EOF;
  if (got != sizeof(h)) return LIME_ERR_READ;
  if (get_be(h, 4) != LIME_MAGIC_NO) return LIME_ERR_READ;
  const unsigned flags = (unsigned)get_be(h + 6, 2);
  r->hdr.MB_flag = (flags & 0x8000u) ? 1 : 0;
  r->hdr.ME_flag = (flags & 0x4000u) ? 1 : 0;
  r->hdr.data_length = get_be(h + 8, 8);
  std::memcpy(r->hdr.type, h + 16, LIME_HDR_TYPE_BYTES);
  r->hdr.type[LIME_HDR_TYPE_BYTES] = '\0';
  r->remaining = r->hdr.data_length;
  r->pad = padding(r->hdr.data_length);
  r->have_header = true;
  return LIME_SUCCESS;
}

char* limeReaderType(LimeReader* r) { return r && r->have_header ? r->hdr.type : nullptr; }
n_uint64_t limeReaderBytes(LimeReader* r) { return r && r->have_header ? r->hdr.data_length : 0; }
int limeReaderMBFlag(LimeReader* r) { return r && r->have_header ? r->hdr.MB_flag : -1; }
int limeReaderMEFlag(LimeReader* r) { return r && r->have_header ? r->hdr.ME_flag : -1; }

int limeReaderReadData(void* dest, n_uint64_t* nbytes, LimeReader* r) {
  if (!dest || !nbytes || !r || !r->have_header) return LIME_ERR_PARAM;
  const uint64_t want = *nbytes;
  const uint64_t n = want < r->remaining ? want : r->remaining;
  const size_t got = fread(dest, 1, (size_t)n, r->fp);
  *nbytes = got;
  r->remaining -= got;
  if (got != n) return LIME_ERR_READ;
  return n < want ? LIME_EOR : LIME_SUCCESS;
}

}  // extern "C"
