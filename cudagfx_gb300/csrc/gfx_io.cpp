// gfx_io.cpp -- ILDG and BQCD gauge-field files and the POSIX cksum (include/gfx_io.h).
// Host code only.  Files are written and read in large big-endian blocks; the
// record layout and the text of the metadata follow the reference's gauge_io.c so
// that either program reads the other's files, byte for byte the same on writing.
#include <algorithm>
#include <cerrno>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/gfx_io.h"
#include "../../include/lime.h"

#include "gfx_io_internal.h"

namespace {

gfx_status io_fail(const std::string& msg) {
  gfx::set_global_error(msg);
  return GFX_ERR_IO;
}

bool valid_dims(const int* d) {
  return d && d[0] > 0 && d[1] > 0 && d[2] > 0 && d[3] > 0;
}
uint64_t volume(const int* d) { return (uint64_t)d[0] * d[1] * d[2] * d[3]; }

// byte order: host (little-endian on every supported machine) <-> big-endian
inline uint64_t bswap64(uint64_t v) { return __builtin_bswap64(v); }
inline uint32_t bswap32(uint32_t v) { return __builtin_bswap32(v); }
bool host_is_big_endian() {
  const uint16_t one = 1;
  unsigned char b;
  std::memcpy(&b, &one, 1);
  return b == 0;
}

void doubles_to_be(const double* in, size_t n, unsigned char* out) {
  const bool be = host_is_big_endian();
  for (size_t k = 0; k < n; k++) {
    uint64_t u;
    std::memcpy(&u, in + k, 8);
    if (!be) u = bswap64(u);
    std::memcpy(out + 8 * k, &u, 8);
  }
}
void be_to_doubles(const unsigned char* in, size_t n, double* out) {
  const bool be = host_is_big_endian();
  for (size_t k = 0; k < n; k++) {
    uint64_t u;
    std::memcpy(&u, in + 8 * k, 8);
    if (!be) u = bswap64(u);
    std::memcpy(out + k, &u, 8);
  }
}
void doubles_to_be_floats(const double* in, size_t n, unsigned char* out) {
  const bool be = host_is_big_endian();
  for (size_t k = 0; k < n; k++) {
    const float f = (float)in[k];
    uint32_t u;
    std::memcpy(&u, &f, 4);
    if (!be) u = bswap32(u);
    std::memcpy(out + 4 * k, &u, 4);
  }
}
void be_floats_to_doubles(const unsigned char* in, size_t n, double* out) {
  const bool be = host_is_big_endian();
  for (size_t k = 0; k < n; k++) {
    uint32_t u;
    std::memcpy(&u, in + 4 * k, 4);
    if (!be) u = bswap32(u);
    float f;
    std::memcpy(&f, &u, 4);
    out[k] = f;
  }
}

// text of <tag> ... </tag> (getXmlEntry, spinor_io.c:310-341)
bool xml_entry(const std::string& s, const char* tag, std::string& out) {
  const std::string b = std::string("<") + tag + ">", e = std::string("</") + tag + ">";
  const size_t p = s.find(b);
  if (p == std::string::npos) return false;
  const size_t q = s.find(e, p + b.size());
  if (q == std::string::npos) return false;
  out = s.substr(p + b.size(), q - p - b.size());
  return true;
}

// value after "<tag> =" in whitespace-separated text (get_unformatted_entry,
// gauge_io.c:119-135)
bool unformatted_entry(const std::string& s, const char* tag, std::string& out) {
  std::vector<std::string> tok;
  size_t i = 0;
  while (i < s.size()) {
    while (i < s.size() && (s[i] == ' ' || s[i] == '\n' || s[i] == '\t')) i++;
    size_t j = i;
    while (j < s.size() && !(s[j] == ' ' || s[j] == '\n' || s[j] == '\t')) j++;
    if (j > i) tok.push_back(s.substr(i, j - i));
    i = j;
  }
  for (size_t k = 0; k + 2 < tok.size(); k++)
    if (tok[k] == tag) {
      out = tok[k + 2];
      return true;
    }
  return false;
}

std::string ildg_format_xml(const int* d, int prec) {
  char m[1024];
  std::snprintf(m, sizeof(m),
                "<?xml version=\"1.0\" encoding=\"UTF-8\"?>\n"
                "<ildgFormat xmlns=\"http://www.lqcd.org/ildg\"\n"
                "            xmlns:xsi=\"http://www.w3.org/2001/XMLSchema-instance\"\n"
                "            xsi:schemaLocation=\"http://www.lqcd.org/ildg filefmt.xsd\">\n"
                "  <version> 1.0 </version>\n"
                "  <field> su3gauge </field>\n"
                "  <precision> %d </precision>\n"
                "  <lx> %d </lx>\n  <ly> %d </ly>\n  <lz> %d </lz>\n  <lt> %d </lt>\n"
                "</ildgFormat>",
                prec, d[0], d[1], d[2], d[3]);
  return m;
}

// the xlf-info text of write_gf_ildg (gauge_io.c:519), fixed fields included
std::string xlf_info(double plaq, double beta) {
  char m[1024];
  std::snprintf(m, sizeof(m),
                " plaquette = %.6f\ntrajectory nr = \nbeta = %.6f, kappa = , mu = , c2_rec = \n"
                "time = 1216028646\nhmcversion = 4.0.1\nmubar = \nepsilonbar = \ndate = ",
                plaq, beta);
  return m;
}

struct File {
  FILE* f = nullptr;
  ~File() {
    if (f) std::fclose(f);
  }
};

int write_record(LimeWriter* w, const char* type, const void* data, uint64_t n) {
  LimeRecordHeader* h = limeCreateHeader(1, 1, (char*)type, n);
  if (!h) return LIME_ERR_PARAM;
  int s = limeWriteRecordHeader(h, w);
  limeDestroyHeader(h);
  if (s != LIME_SUCCESS) return s;
  if (n == 0) return LIME_SUCCESS;
  n_uint64_t k = n;
  return limeWriteRecordData((void*)data, &k, w);
}

// the slices of a BQCD field: file name <base>.<ttt>.<ext>
std::string slice_name(const char* base, int t, const char* ext) {
  char s[16];
  std::snprintf(s, sizeof(s), ".%.3d.", t);
  return std::string(base) + s + ext;
}

gfx_status bqcd_write_field(const char* base, const int* dims, const double* field, int per_site,
                            const char* ext, gfx_slice_cksum* cks) {
  const size_t slice_su3 = (size_t)per_site * dims[0] * dims[1] * dims[2];
  std::vector<unsigned char> buf(slice_su3 * 144);
  for (int t = 0; t < dims[3]; t++) {
    doubles_to_be(field + (size_t)t * slice_su3 * 18, slice_su3 * 18, buf.data());
    const std::string name = slice_name(base, t, ext);
    File f;
    if (!(f.f = std::fopen(name.c_str(), "wb"))) return io_fail("cannot create " + name);
    if (std::fwrite(buf.data(), 1, buf.size(), f.f) != buf.size())
      return io_fail("write failed: " + name);
    if (cks) {
      gfx_cksum_state c;
      gfx_cksum_init(&c);
      gfx_cksum_add(&c, buf.data(), buf.size());
      std::snprintf(cks[t].file, sizeof(cks[t].file), "%s", name.c_str());
      cks[t].sum = gfx_cksum_get(&c);
      cks[t].bytes = c.bytes;
    }
  }
  return GFX_OK;
}

gfx_status bqcd_read_field(const char* base, const int* dims, double* field, int per_site,
                           const char* ext, gfx_slice_cksum* cks) {
  const size_t slice_su3 = (size_t)per_site * dims[0] * dims[1] * dims[2];
  std::vector<unsigned char> buf(slice_su3 * 144);
  for (int t = 0; t < dims[3]; t++) {
    const std::string name = slice_name(base, t, ext);
    File f;
    if (!(f.f = std::fopen(name.c_str(), "rb"))) return io_fail("cannot open " + name);
    if (std::fread(buf.data(), 1, buf.size(), f.f) != buf.size())
      return io_fail("file shorter than a time slice of the lattice: " + name);
    be_to_doubles(buf.data(), slice_su3 * 18, field + (size_t)t * slice_su3 * 18);
    if (cks) {
      gfx_cksum_state c;
      gfx_cksum_init(&c);
      gfx_cksum_add(&c, buf.data(), buf.size());
      std::snprintf(cks[t].file, sizeof(cks[t].file), "%s", name.c_str());
      cks[t].sum = gfx_cksum_get(&c);
      cks[t].bytes = c.bytes;
    }
  }
  return GFX_OK;
}

}  // namespace

namespace gfx {
void to_be64(const void* in, size_t n, void* out) {
  doubles_to_be((const double*)in, n, (unsigned char*)out);
}
void from_be64(const void* in, size_t n, void* out) {
  be_to_doubles((const unsigned char*)in, n, (double*)out);
}
void to_be32(const void* in, size_t n, void* out) {
  const bool be = host_is_big_endian();
  for (size_t k = 0; k < n; k++) {
    uint32_t u;
    std::memcpy(&u, (const char*)in + 4 * k, 4);
    if (!be) u = bswap32(u);
    std::memcpy((char*)out + 4 * k, &u, 4);
  }
}
void from_be32(const void* in, size_t n, void* out) { to_be32(in, n, out); }
}  // namespace gfx

extern "C" {

// ---------------------------------------------------------------------------
// POSIX cksum.  The table is built from the polynomial (CRC-32, MSB first).
// ---------------------------------------------------------------------------
static const uint32_t* crc_table() {
  static uint32_t tab[256];
  static bool ready = false;
  if (!ready) {
    for (uint32_t i = 0; i < 256; i++) {
      uint32_t c = i << 24;
      for (int k = 0; k < 8; k++) c = (c & 0x80000000u) ? (c << 1) ^ 0x04C11DB7u : (c << 1);
      tab[i] = c;
    }
    ready = true;
  }
  return tab;
}

void gfx_cksum_init(gfx_cksum_state* s) {
  crc_table();
  s->crc = 0;
  s->bytes = 0;
}

void gfx_cksum_add(gfx_cksum_state* s, const void* data, size_t n) {
  const uint32_t* tab = crc_table();
  const unsigned char* p = (const unsigned char*)data;
  uint32_t c = s->crc;
  for (size_t i = 0; i < n; i++) c = (c << 8) ^ tab[((c >> 24) ^ p[i]) & 0xff];
  s->crc = c;
  s->bytes += n;
}

uint32_t gfx_cksum_get(const gfx_cksum_state* s) {
  const uint32_t* tab = crc_table();
  uint32_t c = s->crc;
  for (uint64_t n = s->bytes; n > 0; n >>= 8) c = (c << 8) ^ tab[((c >> 24) ^ (uint32_t)n) & 0xff];
  return ~c;
}

// ---------------------------------------------------------------------------
// ILDG
// ---------------------------------------------------------------------------
static gfx_status ildg_scan(FILE* f, LimeReader* r, gfx_ildg_info* info, bool* at_data) {
  std::memset(info, 0, sizeof(*info));
  *at_data = false;
  bool have_format = false;
  int st;
  while ((st = limeReaderNextRecord(r)) == LIME_SUCCESS) {
    const std::string type = limeReaderType(r);
    const uint64_t n = limeReaderBytes(r);
    if (type == "ildg-binary-data") {
      info->data_bytes = n;
      *at_data = true;
      break;
    }
    if (type != "ildg-format" && type != "xlf-info") continue;
    if (n > (1u << 20)) return io_fail("metadata record too long: " + type);
    std::string text(n, '\0');
    n_uint64_t k = n;
    if (limeReaderReadData(&text[0], &k, r) != LIME_SUCCESS || k != n)
      return io_fail("truncated record " + type);
    std::string v;
    if (type == "ildg-format") {
      have_format = true;
      static const char* tags[4] = {"lx", "ly", "lz", "lt"};
      for (int d = 0; d < 4; d++)
        if (xml_entry(text, tags[d], v)) info->dims[d] = std::atoi(v.c_str());
      if (xml_entry(text, "precision", v)) info->precision = std::atoi(v.c_str());
    } else {
      if (unformatted_entry(text, "plaquette", v)) info->plaquette = std::atof(v.c_str());
      if (unformatted_entry(text, "beta", v)) info->beta = std::atof(v.c_str());
    }
  }
  (void)f;
  if (st != LIME_SUCCESS && st != LIME_EOF) return io_fail("LIME read error");
  if (!have_format) return io_fail("no ildg-format record");
  return GFX_OK;
}

gfx_status gfx_ildg_read_info(const char* path, gfx_ildg_info* info) {
  if (!path || !info) return io_fail("gfx_ildg_read_info: NULL argument");
  File f;
  if (!(f.f = std::fopen(path, "rb"))) return io_fail(std::string("cannot open ") + path);
  LimeReader* r = limeCreateReader(f.f);
  bool at_data;
  gfx_status s = ildg_scan(f.f, r, info, &at_data);
  limeDestroyReader(r);
  return s;
}

gfx_status gfx_ildg_read(const char* path, const int dims[4], double* links, gfx_ildg_info* out) {
  if (!path || !valid_dims(dims) || !links) return io_fail("gfx_ildg_read: bad argument");
  File f;
  if (!(f.f = std::fopen(path, "rb"))) return io_fail(std::string("cannot open ") + path);
  LimeReader* r = limeCreateReader(f.f);
  gfx_ildg_info info;
  bool at_data;
  gfx_status s = ildg_scan(f.f, r, &info, &at_data);
  if (s == GFX_OK && !at_data) s = io_fail(std::string("no ildg-binary-data record in ") + path);
  for (int d = 0; s == GFX_OK && d < 4; d++)
    if (info.dims[d] != dims[d]) s = io_fail(std::string("lattice extents differ from ") + path);
  const uint64_t nlink = 4 * volume(dims);
  int bytes_per = 0;
  if (s == GFX_OK) {
    if (info.data_bytes == nlink * 144 && (info.precision == 64 || info.precision == 0))
      bytes_per = 8;
    else if (info.data_bytes == nlink * 72 && (info.precision == 32 || info.precision == 0))
      bytes_per = 4;
    else
      s = io_fail(std::string("precision entry does not match the data size in ") + path);
  }
  if (s == GFX_OK) {
    // in blocks of up to 2^20 matrices
    const uint64_t block = 1u << 20;
    std::vector<unsigned char> buf((size_t)std::min<uint64_t>(block, nlink) * 18 * bytes_per);
    for (uint64_t k0 = 0; k0 < nlink && s == GFX_OK; k0 += block) {
      const uint64_t nk = std::min<uint64_t>(block, nlink - k0);
      n_uint64_t want = nk * 18 * bytes_per;
      if (limeReaderReadData(buf.data(), &want, r) != LIME_SUCCESS || want != nk * 18 * bytes_per) {
        s = io_fail(std::string("truncated binary data in ") + path);
        break;
      }
      if (bytes_per == 8)
        be_to_doubles(buf.data(), nk * 18, links + k0 * 18);
      else
        be_floats_to_doubles(buf.data(), nk * 18, links + k0 * 18);
    }
  }
  limeDestroyReader(r);
  if (s == GFX_OK && out) *out = info;
  return s;
}

gfx_status gfx_ildg_write(const char* path, const int dims[4], const double* links, int prec,
                          double plaq, double beta) {
  if (!path || !valid_dims(dims) || !links) return io_fail("gfx_ildg_write: bad argument");
  if (prec != 32 && prec != 64) return io_fail("gfx_ildg_write: precision must be 32 or 64");
  File f;
  if (!(f.f = std::fopen(path, "wb"))) return io_fail(std::string("cannot create ") + path);
  LimeWriter* w = limeCreateWriter(f.f);
  const std::string fmt = ildg_format_xml(dims, prec), xlf = xlf_info(plaq, beta);
  const uint64_t nlink = 4 * volume(dims);
  const int bytes_per = prec / 8;
  int st = write_record(w, "ildg-format", fmt.data(), fmt.size());
  if (st == LIME_SUCCESS) st = write_record(w, "xlf-info", xlf.data(), xlf.size());
  if (st == LIME_SUCCESS) {
    LimeRecordHeader* h = limeCreateHeader(1, 1, (char*)"ildg-binary-data", nlink * 18 * bytes_per);
    st = limeWriteRecordHeader(h, w);
    limeDestroyHeader(h);
  }
  const uint64_t block = 1u << 20;
  std::vector<unsigned char> buf((size_t)std::min<uint64_t>(block, nlink) * 18 * bytes_per);
  for (uint64_t k0 = 0; k0 < nlink && st == LIME_SUCCESS; k0 += block) {
    const uint64_t nk = std::min<uint64_t>(block, nlink - k0);
    if (bytes_per == 8)
      doubles_to_be(links + k0 * 18, nk * 18, buf.data());
    else
      doubles_to_be_floats(links + k0 * 18, nk * 18, buf.data());
    n_uint64_t k = nk * 18 * bytes_per;
    st = limeWriteRecordData(buf.data(), &k, w);
  }
  const int st2 = limeDestroyWriter(w);
  if (st != LIME_SUCCESS || st2 != LIME_SUCCESS || std::fflush(f.f) != 0)
    return io_fail(std::string("write failed: ") + path);
  return GFX_OK;
}

// ---------------------------------------------------------------------------
// BQCD
// ---------------------------------------------------------------------------
gfx_status gfx_bqcd_write(const char* base, const int dims[4], const double* links, double plaq,
                          double beta, int ensemble, gfx_slice_cksum* cks_out) {
  if (!base || !valid_dims(dims) || !links) return io_fail("gfx_bqcd_write: bad argument");
  std::vector<gfx_slice_cksum> cks(dims[3]);
  gfx_status s = bqcd_write_field(base, dims, links, 4, "u", cks.data());
  if (s) return s;
  // the info file of write_conf_info (gauge_io.c:798-833), fixed header lines included
  const std::string name = std::string(base) + ".info";
  File f;
  if (!(f.f = std::fopen(name.c_str(), "w"))) return io_fail("cannot create " + name);
  (void)ensemble;  // not part of the info file
  std::fprintf(f.f, " >BeginConfInfoHeader\n");
  std::fprintf(f.f, " Format           2\n");
  std::fprintf(f.f, " Program bqcd YM-JSCC-1.2 [$Rev: 21 $ $Date: 2009-08-21 09:03:38 $]\n");
  std::fprintf(f.f, " Run         999\n");
  std::fprintf(f.f, " Host pha41\n");
  std::fprintf(f.f, " Date 2008-07-01 17:41:16.263\n");
  std::fprintf(f.f, " L  %3d %3d %3d %3d\n", dims[0], dims[1], dims[2], dims[3]);
  std::fprintf(f.f, " REAL_kind           8\n");
  std::fprintf(f.f, " beta  %.3f\n", beta);
  std::fprintf(f.f, " PlaqEnergy %25.14E\n", plaq);
  std::fprintf(f.f, " >EndConfInfoHeader\n");
  std::fprintf(f.f, " >BeginCheckSum\n");
  for (int t = 0; t < dims[3]; t++)
    std::fprintf(f.f, " %s            %10u            %10u\n", cks[t].file, (unsigned)cks[t].sum,
                 (unsigned)cks[t].bytes);
  std::fprintf(f.f, " >EndCheckSum\n");
  if (std::ferror(f.f)) return io_fail("write failed: " + name);
  if (cks_out) std::memcpy(cks_out, cks.data(), sizeof(gfx_slice_cksum) * dims[3]);
  return GFX_OK;
}

gfx_status gfx_bqcd_read(const char* base, const int dims[4], double* links, gfx_slice_cksum* cks) {
  if (!base || !valid_dims(dims) || !links) return io_fail("gfx_bqcd_read: bad argument");
  return bqcd_read_field(base, dims, links, 4, "u", cks);
}

gfx_status gfx_bqcd_read_trafo(const char* base, const int dims[4], double* trafo,
                               gfx_slice_cksum* cks) {
  if (!base || !valid_dims(dims) || !trafo) return io_fail("gfx_bqcd_read_trafo: bad argument");
  return bqcd_read_field(base, dims, trafo, 1, "g", cks);
}

gfx_status gfx_bqcd_write_trafo(const char* base, const int dims[4], const double* trafo,
                                gfx_slice_cksum* cks) {
  if (!base || !valid_dims(dims) || !trafo) return io_fail("gfx_bqcd_write_trafo: bad argument");
  return bqcd_write_field(base, dims, trafo, 1, "g", cks);
}

gfx_status gfx_bqcd_read_info(const char* path, gfx_bqcd_info* info, gfx_slice_cksum* cks,
                              int cap, int* ncks) {
  if (!path || !info) return io_fail("gfx_bqcd_read_info: NULL argument");
  File f;
  if (!(f.f = std::fopen(path, "r"))) return io_fail(std::string("cannot open ") + path);
  std::memset(info, 0, sizeof(*info));
  if (ncks) *ncks = 0;
  char line[512];
  bool in_ck = false, header = false;
  int n = 0;
  while (std::fgets(line, sizeof(line), f.f)) {
    char key[256] = {0};
    if (std::sscanf(line, "%255s", key) != 1) continue;
    const std::string k = key;
    if (k == ">BeginConfInfoHeader") header = true;
    else if (k == ">BeginCheckSum") in_ck = true;
    else if (k == ">EndCheckSum") in_ck = false;
    else if (in_ck) {
      char file[256];
      unsigned long long sum, bytes;
      if (std::sscanf(line, "%255s %llu %llu", file, &sum, &bytes) == 3) {
        if (cks && n < cap) {
          std::snprintf(cks[n].file, sizeof(cks[n].file), "%.79s", file);  // the field's width
          cks[n].sum = sum;
          cks[n].bytes = bytes;
        }
        n++;
      }
    } else if (k == "Run") std::sscanf(line, " Run %d", &info->run);
    else if (k == "L")
      std::sscanf(line, " L %d %d %d %d", &info->dims[0], &info->dims[1], &info->dims[2],
                  &info->dims[3]);
    else if (k == "beta") std::sscanf(line, " beta %lf", &info->beta);
    else if (k == "PlaqEnergy") std::sscanf(line, " PlaqEnergy %lf", &info->plaquette);
  }
  if (!header || !valid_dims(info->dims)) return io_fail(std::string("not a BQCD info file: ") + path);
  if (ncks) *ncks = n < cap ? n : cap;
  return GFX_OK;
}

}  // extern "C"
