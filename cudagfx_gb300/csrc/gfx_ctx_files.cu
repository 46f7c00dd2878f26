// gfx_ctx_files.cu -- the file steps around a context (include/gfx_io.h): links from
// ILDG, the context's links and its gauge-fixed field to ILDG, and checkpoints of
// links, g and the twister state as LIME records.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <string>
#include <vector>

#include "../../include/gfx.h"
#include "../../include/gfx_io.h"
#include "../../include/lime.h"
#include "gfx_context.h"
#include "gfx_io_internal.h"

using namespace gfx;

extern "C" {

// ---------------------------------------------------------------------------
// files around a context (include/gfx_io.h)
// ---------------------------------------------------------------------------



gfx_status gfx_load_links_ildg(gfx_ctx* ctx, const char* path, gfx_ildg_info* info) {
  if (!ctx || !path) return fail(ctx, GFX_ERR_ARG, "gfx_load_links_ildg: NULL argument");
  int d[4];
  ctx_dims(ctx, d);
  std::vector<double> links(18 * 4 * (size_t)ctx->vol);
  gfx_status s = gfx_ildg_read(path, d, links.data(), info);
  if (s) return fail(ctx, s, global_error());
  return gfx_set_links(ctx, links.data());
}

gfx_status gfx_write_links_ildg(gfx_ctx* ctx, const char* path, int precision, double beta) {
  if (!ctx || !path) return fail(ctx, GFX_ERR_ARG, "gfx_write_links_ildg: NULL argument");
  double plaq = 0.0;
  gfx_status s = gfx_plaquette(ctx, &plaq);
  if (s) return s;
  std::vector<double> links;
  if ((s = links_to_host(ctx, ctx->U64, links))) return s;
  int d[4];
  ctx_dims(ctx, d);
  s = gfx_ildg_write(path, d, links.data(), precision, plaq, beta);
  return s ? fail(ctx, s, global_error()) : GFX_OK;
}

gfx_status gfx_write_fixed_ildg(gfx_ctx* ctx, const char* path, int precision, double beta) {
  if (!ctx || !path) return fail(ctx, GFX_ERR_ARG, "gfx_write_fixed_ildg: NULL argument");
  gfx_status s = sync_g64(ctx);
  if (s) return s;
  // U' = g U g^+ in place, then the saved links back: the context is unchanged
  void* saved = nullptr;
  if ((s = dalloc(ctx, &saved, link_bytes64(ctx)))) return s;
  CK(cudaMemcpyAsync(saved, ctx->U64, link_bytes64(ctx), cudaMemcpyDeviceToDevice, ctx->stream));
  launch_apply_trafo(ctx->link_nr, ctx->L, ctx->U64, ctx->G64, ctx->stream);
  double plaq = 0.0;
  std::vector<double> links;
  s = gfx_plaquette(ctx, &plaq);
  if (s == GFX_OK) s = links_to_host(ctx, ctx->U64, links);
  cudaMemcpyAsync(ctx->U64, saved, link_bytes64(ctx), cudaMemcpyDeviceToDevice, ctx->stream);
  cudaError_t e = cudaStreamSynchronize(ctx->stream);
  cudaFree(saved);
  ctx->dev_bytes -= link_bytes64(ctx);
  if (s) return s;
  if (e != cudaSuccess) return fail(ctx, GFX_ERR_CUDA, cudaGetErrorString(e));
  int d[4];
  ctx_dims(ctx, d);
  s = gfx_ildg_write(path, d, links.data(), precision, plaq, beta);
  return s ? fail(ctx, s, global_error()) : GFX_OK;
}

// ---- checkpoints: LIME records of big-endian words ----
namespace {
struct CkptFile {
  FILE* f = nullptr;
  ~CkptFile() {
    if (f) std::fclose(f);
  }
};
int ckpt_record(LimeWriter* w, const char* type, const void* data, uint64_t n) {
  LimeRecordHeader* h = limeCreateHeader(1, 1, (char*)type, n);
  int st = limeWriteRecordHeader(h, w);
  limeDestroyHeader(h);
  if (st != LIME_SUCCESS || n == 0) return st;
  n_uint64_t k = n;
  return limeWriteRecordData((void*)data, &k, w);
}
}  // namespace

gfx_status gfx_checkpoint_save(gfx_ctx* ctx, const char* path) {
  if (!ctx || !path) return fail(ctx, GFX_ERR_ARG, "gfx_checkpoint_save: NULL argument");
  gfx_status s;
  std::vector<double> links;
  if ((s = links_to_host(ctx, ctx->U64, links))) return s;
  // g: the FP64 field as host su3, plus the FP32 field as stored when it is the
  // current one (the widening to FP64 reunitarizes, so both are kept)
  const int active = ctx->g_active;
  std::vector<float> g32;
  if (active == 0) {
    g32.resize(g_bytes32(ctx) / 4);
    CK(cudaMemcpyAsync(g32.data(), ctx->G32, g_bytes32(ctx), cudaMemcpyDeviceToHost, ctx->stream));
  }
  std::vector<double> g(18 * (size_t)ctx->vol);
  if ((s = gfx_get_trafo(ctx, g.data()))) return s;
  if (active == 0) ctx->g_active = 0;  // gfx_get_trafo widened a current FP32 g; it stays current
  char info[512];
  std::snprintf(info, sizeof(info),
                "gfx-checkpoint 1\ndims %d %d %d %d\nprecision %d\nlink_reals %d\ng_fp32 %d\n"
                "mt_params %d\nmt_seeded %d\nmt_init %d\nn_gauss %d\nn_unif %d\n",
                ctx->lx, ctx->ly, ctx->lz, ctx->lt, ctx->precision, ctx->link_nr, active == 0,
                (int)ctx->mt_params, (int)ctx->mt_seeded, (int)ctx->mt_init, ctx->n_gauss,
                ctx->n_unif);
  CkptFile f;
  if (!(f.f = std::fopen(path, "wb"))) return fail(ctx, GFX_ERR_IO, std::string("cannot create ") + path);
  LimeWriter* w = limeCreateWriter(f.f);
  int st = ckpt_record(w, "gfx-checkpoint-info", info, std::strlen(info));
  to_be64(links.data(), links.size(), links.data());
  if (st == LIME_SUCCESS) st = ckpt_record(w, "gfx-links", links.data(), 8 * links.size());
  to_be64(g.data(), g.size(), g.data());
  if (st == LIME_SUCCESS) st = ckpt_record(w, "gfx-trafo", g.data(), 8 * g.size());
  if (st == LIME_SUCCESS && active == 0) {
    to_be32(g32.data(), g32.size(), g32.data());
    st = ckpt_record(w, "gfx-trafo-fp32", g32.data(), 4 * g32.size());
  }
  if (st == LIME_SUCCESS && ctx->mt_params) {
    std::vector<uint32_t> p(ctx->h_params, ctx->h_params + 4 * kMTCount);
    to_be32(p.data(), p.size(), p.data());
    st = ckpt_record(w, "gfx-mt-params", p.data(), 4 * p.size());
  }
  if (st == LIME_SUCCESS && ctx->mt_init) {
    std::vector<uint32_t> state((size_t)kMTN * kMTCount);
    std::vector<float> ga((size_t)kMTCount * ctx->nper_g), un((size_t)kMTCount * ctx->nper_u);
    if ((s = gfx_mt_read(ctx, ga.data(), un.data(), state.data(), nullptr))) {
      limeDestroyWriter(w);
      return s;
    }
    to_be32(state.data(), state.size(), state.data());
    to_be32(ga.data(), ga.size(), ga.data());
    to_be32(un.data(), un.size(), un.data());
    st = ckpt_record(w, "gfx-mt-state", state.data(), 4 * state.size());
    if (st == LIME_SUCCESS) st = ckpt_record(w, "gfx-mt-gauss", ga.data(), 4 * ga.size());
    if (st == LIME_SUCCESS) st = ckpt_record(w, "gfx-mt-unif", un.data(), 4 * un.size());
  }
  const int st2 = limeDestroyWriter(w);
  if (st != LIME_SUCCESS || st2 != LIME_SUCCESS || std::fflush(f.f) != 0)
    return fail(ctx, GFX_ERR_IO, std::string("checkpoint write failed: ") + path);
  return GFX_OK;
}

gfx_status gfx_checkpoint_load(gfx_ctx* ctx, const char* path) {
  if (!ctx || !path) return fail(ctx, GFX_ERR_ARG, "gfx_checkpoint_load: NULL argument");
  CkptFile f;
  if (!(f.f = std::fopen(path, "rb"))) return fail(ctx, GFX_ERR_IO, std::string("cannot open ") + path);
  LimeReader* r = limeCreateReader(f.f);
  std::string info;
  std::vector<unsigned char> links, g, g32, params, state, ga, un;
  int st;
  auto bad = [&](const std::string& why) {
    limeDestroyReader(r);
    return fail(ctx, GFX_ERR_IO, "checkpoint " + std::string(path) + ": " + why);
  };
  while ((st = limeReaderNextRecord(r)) == LIME_SUCCESS) {
    const std::string type = limeReaderType(r);
    std::vector<unsigned char>* dst = type == "gfx-links" ? &links
                                      : type == "gfx-trafo" ? &g
                                      : type == "gfx-trafo-fp32" ? &g32
                                      : type == "gfx-mt-params" ? &params
                                      : type == "gfx-mt-state" ? &state
                                      : type == "gfx-mt-gauss" ? &ga
                                      : type == "gfx-mt-unif" ? &un : nullptr;
    const uint64_t n = limeReaderBytes(r);
    if (type == "gfx-checkpoint-info") {
      if (n > 4096) return bad("info record too long");
      info.assign(n, '\0');
      n_uint64_t k = n;
      if (limeReaderReadData(&info[0], &k, r) != LIME_SUCCESS || k != n) return bad("truncated");
    } else if (dst) {
      dst->resize(n);
      n_uint64_t k = n;
      if (n && (limeReaderReadData(dst->data(), &k, r) != LIME_SUCCESS || k != n))
        return bad("truncated " + type);
    }
  }
  limeDestroyReader(r);
  if (st != LIME_EOF) return fail(ctx, GFX_ERR_IO, std::string("checkpoint read error: ") + path);
  int ver = 0, d[4] = {0, 0, 0, 0}, prec = -1, nr = 0, fp32 = 0, mp = 0, ms = 0, mi = 0, ng = 0,
      nu = 0;
  if (std::sscanf(info.c_str(),
                  "gfx-checkpoint %d\ndims %d %d %d %d\nprecision %d\nlink_reals %d\ng_fp32 %d\n"
                  "mt_params %d\nmt_seeded %d\nmt_init %d\nn_gauss %d\nn_unif %d",
                  &ver, &d[0], &d[1], &d[2], &d[3], &prec, &nr, &fp32, &mp, &ms, &mi, &ng,
                  &nu) != 13 ||
      ver != 1)
    return fail(ctx, GFX_ERR_IO, std::string("not a checkpoint: ") + path);
  if (d[0] != ctx->lx || d[1] != ctx->ly || d[2] != ctx->lz || d[3] != ctx->lt)
    return fail(ctx, GFX_ERR_IO, std::string("checkpoint of another lattice: ") + path);
  const size_t nl = 18 * 4 * (size_t)ctx->vol, ng64 = 18 * (size_t)ctx->vol;
  if (links.size() != 8 * nl || g.size() != 8 * ng64)
    return fail(ctx, GFX_ERR_IO, std::string("checkpoint fields of the wrong size: ") + path);
  if (fp32 && (!ctx->G32 || g32.size() != g_bytes32(ctx)))
    return fail(ctx, GFX_ERR_IO, "checkpoint holds an FP32 g this context cannot take");
  gfx_status s;
  if (nr != ctx->link_nr && (s = relayout_links(ctx, nr))) return s;
  from_be64(links.data(), nl, links.data());
  if ((s = gfx_set_links(ctx, (const double*)links.data()))) return s;
  from_be64(g.data(), ng64, g.data());
  if ((s = gfx_set_trafo(ctx, (const double*)g.data()))) return s;
  if (fp32) {
    from_be32(g32.data(), g32.size() / 4, g32.data());
    CK(cudaMemcpy(ctx->G32, g32.data(), g32.size(), cudaMemcpyHostToDevice));
    ctx->g_active = 0;
  }
  if (mp) {
    if (params.size() != 16 * (size_t)kMTCount) return fail(ctx, GFX_ERR_IO, "checkpoint: twister parameters");
    from_be32(params.data(), 4 * kMTCount, params.data());
    if ((s = gfx_mt_load_params(ctx, (const uint32_t*)params.data()))) return s;
    ctx->mt_seeded = ms != 0;
  }
  if (mi) {
    if ((s = gfx_mt_init(ctx, ng, nu))) return s;
    if (state.size() != 4 * (size_t)kMTN * kMTCount || ga.size() != 4 * (size_t)kMTCount * ctx->nper_g ||
        un.size() != 4 * (size_t)kMTCount * ctx->nper_u)
      return fail(ctx, GFX_ERR_IO, "checkpoint: twister state of the wrong size");
    from_be32(state.data(), state.size() / 4, state.data());
    from_be32(ga.data(), ga.size() / 4, ga.data());
    from_be32(un.data(), un.size() / 4, un.data());
    CK(cudaMemcpy(ctx->bank.status, state.data(), state.size(), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(ctx->gauss, ga.data(), ga.size(), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(ctx->unif, un.data(), un.size(), cudaMemcpyHostToDevice));
  }
  return GFX_OK;
}

}  // extern "C"
