// gfx_api.cu -- contexts behind the gfx_* C ABI: lifecycle and buffers, fields,
// sweeps and measurements, the convergence loop (a CUDA-graph while loop), the
// twister bank, annealing and thermalization.  The context itself and the helpers
// shared with gfx_tune.cu and gfx_ctx_files.cu are in gfx_context.h.
// Everything runs on the context's stream; host synchronisation happens only where
// a result is returned to the caller.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <ctime>
#include <functional>
#include <string>
#include <vector>

#include "../../include/gfx.h"
#include "gfx_context.h"
#include "gfx_internal.h"
#include "gfx_io_internal.h"

using namespace gfx;

static std::string g_global_err;

// page-locked host allocations made by gfx_host_alloc: start -> size
static std::mutex g_pinned_mu;
static std::map<uintptr_t, size_t> g_pinned;

namespace gfx {
// The device address of [p, p + bytes) when that range lies in one gfx_host_alloc
// allocation and p is 16-byte aligned (the tiled layout kernels move 16-byte words);
// else nullptr and the caller stages through device memory.
void* host_direct_ptr(const void* p, size_t bytes) {
  const uintptr_t a = (uintptr_t)p;
  if (a % 16) return nullptr;
  uintptr_t base = 0;
  {
    std::lock_guard<std::mutex> lk(g_pinned_mu);
    auto it = g_pinned.upper_bound(a);
    if (it == g_pinned.begin()) return nullptr;
    --it;
    if (a < it->first || a + bytes > it->first + it->second) return nullptr;
    base = it->first;
  }
  void* d = nullptr;
  if (cudaHostGetDevicePointer(&d, (void*)base, 0) != cudaSuccess || !d) {
    cudaGetLastError();
    return nullptr;
  }
  return (char*)d + (a - base);
}
}  // namespace gfx






static gfx_status ensure_hist(gfx_ctx* ctx, int cap) {
  if (ctx->hist_cap >= cap) return GFX_OK;
  if (ctx->hist) {
    cudaFree(ctx->hist);
    ctx->dev_bytes -= sizeof(CheckRecord) * ctx->hist_cap;
  }
  ctx->hist = nullptr;
  ctx->hist_cap = 0;
  gfx_status s = dalloc(ctx, (void**)&ctx->hist, sizeof(CheckRecord) * (size_t)cap);
  if (s == GFX_OK) ctx->hist_cap = cap;
  return s;
}

namespace gfx {

gfx_status fail(gfx_ctx* ctx, gfx_status s, const std::string& msg) {
  if (ctx) ctx->err = msg;
  g_global_err = msg;
  return s;
}
void set_global_error(const std::string& msg) { g_global_err = msg; }
const std::string& global_error() { return g_global_err; }

gfx_status dalloc(gfx_ctx* ctx, void** p, size_t bytes) {
  cudaError_t e = cudaMalloc(p, bytes);
  if (e != cudaSuccess) {
    cudaGetLastError();
    *p = nullptr;
    return fail(ctx, e == cudaErrorMemoryAllocation ? GFX_ERR_OOM : GFX_ERR_CUDA,
                std::string("cudaMalloc(") + std::to_string(bytes) + "): " + cudaGetErrorString(e));
  }
  ctx->dev_bytes += bytes;
  return GFX_OK;
}

gfx_status ensure_scratch(gfx_ctx* ctx, size_t bytes) {
  if (ctx->scratch_bytes >= bytes) return GFX_OK;
  if (ctx->scratch_aos) {
    cudaFree(ctx->scratch_aos);
    ctx->dev_bytes -= ctx->scratch_bytes;
    ctx->scratch_aos = nullptr;
    ctx->scratch_bytes = 0;
  }
  gfx_status s = dalloc(ctx, (void**)&ctx->scratch_aos, bytes);
  if (s == GFX_OK) ctx->scratch_bytes = bytes;
  return s;
}

void destroy_graphs(gfx_ctx* ctx) {
  for (auto& g : ctx->graphs) {
    cudaGraphExecDestroy(g.exec);
    cudaGraphDestroy(g.graph);
  }
  ctx->graphs.clear();
}

// the FP32 link copy from the FP64 links, in the current FP32 layout
gfx_status refresh_u32(gfx_ctx* ctx) {
  ctx->rb_valid = false;  // the rebased links follow the FP64 links too
  if (!ctx->U32) return GFX_OK;
  launch_convert_links_64_to_32(ctx->link_nr, ctx->link_nr32, ctx->L, ctx->U64, ctx->U32,
                                ctx->stream);
  CK(cudaGetLastError());
  return GFX_OK;
}

gfx_status sync_g64(gfx_ctx* ctx) {
  if (ctx->g_active == 0) {
    launch_convert_g(0, 1, ctx->L, ctx->G32, ctx->G64, ctx->stream);
    CK(cudaGetLastError());
    ctx->g_active = 1;
  } else if (ctx->g_active == 2) {
    launch_convert_g_df(0, ctx->L, ctx->G64, ctx->Gdf, ctx->stream);  // exact
    CK(cudaGetLastError());
    ctx->g_active = 1;
  } else if (ctx->g_active == 3) {
    launch_compose_g(ctx->L, ctx->G64, ctx->G32, ctx->stream);  // g = (1 + a) g_c
    CK(cudaGetLastError());
    ctx->g_active = 1;
  }
  return GFX_OK;
}

// A new base: g_c = the current g (FP64), the rebased links and the split star from
// it, a = 0.  The links' FP32 remainders pass through the scratch buffer.
gfx_status rebase(gfx_ctx* ctx, int ndir) {
  if (!ctx->G32) return fail(ctx, GFX_ERR_STATE, "rebased FP32 sweeps need a SINGLE or MIXED context");
  gfx_status s;
  if (!ctx->Ur && (s = dalloc(ctx, &ctx->Ur, link_bytes32(ctx)))) return s;
  if (!ctx->W0 && (s = dalloc(ctx, &ctx->W0, rebased_w0_bytes(ctx->L)))) return s;
  if ((s = ensure_scratch(ctx, link_bytes32(ctx)))) return s;
  if ((s = sync_g64(ctx))) return s;
  launch_rebase(ctx->link_nr, ndir, ctx->L, ctx->U64, ctx->G64, ctx->Ur, ctx->scratch_aos,
                ctx->W0, ctx->stream);
  CK(cudaMemsetAsync(ctx->G32, 0, g_bytes32(ctx), ctx->stream));
  CK(cudaGetLastError());
  ctx->g_active = 3;
  ctx->rb_valid = true;
  ctx->rb_ndir = ndir;
  return GFX_OK;
}

gfx_status prepare_rebased(gfx_ctx* ctx, int ndir) {
  if (ctx->g_active == 3 && ctx->rb_valid && ctx->rb_ndir == ndir) return GFX_OK;
  return rebase(ctx, ndir);
}

// the double-float fields of the polish sweeps, allocated on first use; the links
// are converted again after any change of the FP64 links
gfx_status ensure_df(gfx_ctx* ctx) {
  gfx_status s;
  if (!ctx->Udf && (s = dalloc(ctx, &ctx->Udf, (size_t)8 * 9 * 16 * (size_t)ctx->L.vh))) return s;
  if (!ctx->Gdf && (s = dalloc(ctx, &ctx->Gdf, (size_t)2 * 6 * 16 * (size_t)ctx->L.vh))) return s;
  if (!ctx->udf_valid) {
    launch_convert_links_64_to_df(ctx->link_nr, ctx->L, ctx->U64, ctx->Udf, ctx->stream);
    CK(cudaGetLastError());
    ctx->udf_valid = true;
  }
  return GFX_OK;
}

// ---------------------------------------------------------------------------
// sweeps and measurements
// ---------------------------------------------------------------------------
gfx_status prepare_g(gfx_ctx* ctx, int prec) {
  if (prec == 2) {
    gfx_status s = ensure_df(ctx);
    if (s) return s;
    if ((ctx->g_active == 0 || ctx->g_active == 3) && (s = sync_g64(ctx))) return s;
    if (ctx->g_active == 1) {
      launch_convert_g_df(1, ctx->L, ctx->G64, ctx->Gdf, ctx->stream);
      CK(cudaGetLastError());
      ctx->g_active = 2;
    }
    return GFX_OK;
  }
  if (prec == 0) {
    if (!ctx->G32) return fail(ctx, GFX_ERR_STATE, "FP32 sweeps need a SINGLE or MIXED context");
    if (ctx->g_active >= 2) {
      gfx_status s = sync_g64(ctx);
      if (s) return s;
    }
    if (ctx->g_active == 1) {
      launch_convert_g(1, 0, ctx->L, ctx->G64, ctx->G32, ctx->stream);
      CK(cudaGetLastError());
      ctx->g_active = 0;
    }
  } else {
    gfx_status s = sync_g64(ctx);
    if (s) return s;
  }
  return GFX_OK;
}

void enqueue_sweep(gfx_ctx* ctx, int prec, int ndir, double omega) {
  if (prec == 3) {  // rebased FP32 (after prepare_rebased)
    for (int p = 0; p < 2; p++)
      launch_or_rebased(ndir, ctx->L, ctx->Ur, ctx->W0, ctx->G32, p, omega, ctx->stream);
    ctx->launches += 2;
    return;
  }
  const void* U = prec == 0 ? ctx->U32 : prec == 2 ? ctx->Udf : ctx->U64;
  void* G = prec == 0 ? ctx->G32 : prec == 2 ? ctx->Gdf : ctx->G64;
  for (int p = 0; p < 2; p++)
    launch_or_halfsweep(prec, lnr(ctx, prec), ndir, ctx->L, U, G, p, omega, ctx->or_block[prec],
                        ctx->or_pf[prec], ctx->stream, ctx->or_wide);
  ctx->launches += 2;
}

void enqueue_sweeps(gfx_ctx* ctx, int prec, int ndir, double omega, int n) {
  for (int k = 0; k < n; k++) enqueue_sweep(ctx, prec, ndir, omega);
}

static int meas_block(const gfx_ctx* ctx) {
  // a measurement block covers part of one time slice of one parity; the batched
  // measurement uses the same 128-site grouping, so sums agree bit for bit
  (void)ctx;
  return 128;
}

void enqueue_measure(gfx_ctx* ctx, int cprec, int gprec, int ndir) {
  const int b = meas_block(ctx);
  if (cprec == 3) {  // rebased FP32 (after prepare_rebased)
    launch_measure_rebased(ndir, ctx->L, ctx->Ur, ctx->W0, ctx->G32, ctx->partials, b, ctx->stream);
    ctx->launches += 1;
    return;
  }
  const void* U = cprec == 0 ? ctx->U32 : cprec == 2 ? ctx->Udf : ctx->U64;
  const void* G = gprec == 0 ? ctx->G32 : gprec == 2 ? ctx->Gdf : ctx->G64;
  launch_measure(cprec, lnr(ctx, cprec), gprec, ndir, ctx->L, U, G, ctx->partials, b, ctx->stream);
  ctx->launches += 1;
}

bool odd_only_checks(const gfx_ctx* ctx, int prec) {
  return ctx->odd_checks && prec == 0 && ctx->precision == GFX_PREC_MIXED &&
         fused_check_ok(ctx->L, ctx->link_nr32);
}

// n sweeps, then the check's partials.  FP32 with fused_check_ok: the last odd
// half-sweep writes the odd sites' partials (fuse_check) or a measurement of the odd
// sites does; odd_only stops there, else the even sites are measured as well.
void enqueue_sweeps_measure(gfx_ctx* ctx, int prec, int ndir, double omega, int n,
                            bool odd_only) {
  const bool ok = prec == 0 && n >= 1 && fused_check_ok(ctx->L, ctx->link_nr32);
  if (!ok) {
    enqueue_sweeps(ctx, prec, ndir, omega, n);
    enqueue_measure(ctx, prec, prec, ndir);
    return;
  }
  if (ctx->fuse_check) {
    enqueue_sweeps(ctx, 0, ndir, omega, n - 1);
    launch_or_halfsweep(0, 12, ndir, ctx->L, ctx->U32, ctx->G32, 0, omega, ctx->or_block[0],
                        ctx->or_pf[0], ctx->stream, ctx->or_wide);
    launch_or_halfsweep_measure(ndir, ctx->L, ctx->U32, ctx->G32, omega, ctx->or_pf[0] >= 2,
                                ctx->partials, ctx->stream);
    ctx->launches += 2;
  } else {
    enqueue_sweeps(ctx, 0, ndir, omega, n);
    launch_measure_parity(ndir, ctx->L, ctx->U32, ctx->G32, ctx->partials, 1, ctx->stream);
    ctx->launches += 1;
  }
  if (!odd_only) {
    launch_measure_parity(ndir, ctx->L, ctx->U32, ctx->G32, ctx->partials, 0, ctx->stream);
    ctx->launches += 1;
  }
}

void enqueue_reduce(gfx_ctx* ctx, int ndir, bool with_loop, int advance,
                           unsigned long long handle, int use_handle, bool odd_only) {
  const int nbx = measure_blocks_x(ctx->L, meas_block(ctx));
  launch_reduce(ctx->L, ndir, ctx->partials, nbx, ctx->slice_sums, ctx->reduced,
                with_loop ? ctx->loop : nullptr, with_loop ? ctx->hist : nullptr, advance, handle,
                use_handle, ctx->stream, odd_only ? 1 : 0);
  ctx->launches += 2;
}

// Re-pack the FP64 links as nr reals per link (12 or 18).  The new buffer is
// allocated first, so a failed allocation leaves the context as it was.
gfx_status relayout_links(gfx_ctx* ctx, int nr) {
  if (nr == ctx->link_nr) return GFX_OK;
  const size_t bytes = sizeof(double) * 18 * 4 * (size_t)ctx->vol;
  gfx_status s = ensure_scratch(ctx, bytes);
  if (s) return s;
  const size_t new_bytes = (size_t)8 * (nr / 2) * 16 * (size_t)ctx->L.vh;
  void* nu = nullptr;
  s = dalloc(ctx, &nu, new_bytes);
  if (s) return s;
  launch_unpack_links(ctx->link_nr, ctx->L, ctx->U64, ctx->scratch_aos, ctx->stream);
  launch_pack_links(nr, ctx->L, ctx->scratch_aos, nu, ctx->stream);
  CK(cudaGetLastError());
  CK(cudaStreamSynchronize(ctx->stream));
  cudaFree(ctx->U64);
  ctx->dev_bytes -= link_bytes64(ctx);
  ctx->U64 = nu;
  ctx->link_nr = nr;
  destroy_graphs(ctx);
  return GFX_OK;
}

// FP32 link layout 12 or 8; the 8-real copy needs a larger buffer (allocated first)
gfx_status set_link_layout32(gfx_ctx* ctx, int nr32) {
  if (!ctx->U32 || nr32 == ctx->link_nr32) return GFX_OK;
  const size_t need = link_bytes32_for(ctx, nr32);
  if (need > ctx->u32_bytes) {
    void* nu = nullptr;
    gfx_status s = dalloc(ctx, &nu, need);
    if (s) return s;
    CK(cudaStreamSynchronize(ctx->stream));
    cudaFree(ctx->U32);
    ctx->dev_bytes -= ctx->u32_bytes;
    ctx->U32 = nu;
    ctx->u32_bytes = need;
  }
  ctx->link_nr32 = nr32;
  destroy_graphs(ctx);
  gfx_status s = refresh_u32(ctx);
  if (s) return s;
  CK(cudaStreamSynchronize(ctx->stream));
  return GFX_OK;
}

// the links of U64 (or of `src`, a device field of the same layout) as host AoS
gfx_status links_to_host(gfx_ctx* ctx, const void* src, std::vector<double>& out) {
  const size_t bytes = sizeof(double) * 18 * 4 * (size_t)ctx->vol;
  gfx_status s = ensure_scratch(ctx, bytes);
  if (s) return s;
  out.resize(18 * 4 * (size_t)ctx->vol);
  launch_unpack_links(ctx->link_nr, ctx->L, src, ctx->scratch_aos, ctx->stream);
  CK(cudaGetLastError());
  CK(cudaMemcpyAsync(out.data(), ctx->scratch_aos, bytes, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  return GFX_OK;
}


}  // namespace gfx

extern "C" {

const char* gfx_last_error(const gfx_ctx* ctx) {
  return ctx ? ctx->err.c_str() : g_global_err.c_str();
}



gfx_status gfx_destroy(gfx_ctx* ctx) {
  if (!ctx) return GFX_OK;
  cudaStreamSynchronize(ctx->stream);
  destroy_graphs(ctx);
  void* ptrs[] = {ctx->U64,     ctx->G64,  ctx->U32,  ctx->G32,  ctx->partials,
                  ctx->slice_sums, ctx->reduced, ctx->loop, ctx->hist, ctx->scratch_aos,
                  ctx->bank.a,  ctx->bank.b, ctx->bank.c, ctx->bank.seed, ctx->bank.status,
                  ctx->gauss,   ctx->unif, ctx->Udf, ctx->Gdf, ctx->Ur, ctx->W0};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  if (ctx->loop_host) cudaFreeHost(ctx->loop_host);
  if (ctx->reduced_host) cudaFreeHost(ctx->reduced_host);
  for (int k = 0; k < 3; k++)
    if (ctx->io_ev[k]) cudaEventDestroy(ctx->io_ev[k]);
  if (ctx->own_stream) cudaStreamDestroy(ctx->stream);
  delete ctx;
  return GFX_OK;
}

gfx_status gfx_create(gfx_ctx** out, int lx, int ly, int lz, int lt, int precision,
                      int link_reals64, void* stream) {
  gfx_ctx* ctx = nullptr;
  if (!out) return fail(nullptr, GFX_ERR_ARG, "gfx_create: out is NULL");
  *out = nullptr;
  if (lx < 2 || ly < 2 || lz < 2 || lt < 2 || (lx | ly | lz | lt) & 1)
    return fail(nullptr, GFX_ERR_BAD_VOLUME, "gfx_create: every extent must be even and >= 2");
  const long long vol = (long long)lx * ly * lz * lt;
  if (vol / 2 > (1ll << 30))
    return fail(nullptr, GFX_ERR_BAD_VOLUME, "gfx_create: volume/2 must be below 2^30 sites");
  if (precision < GFX_PREC_DOUBLE || precision > GFX_PREC_MIXED)
    return fail(nullptr, GFX_ERR_ARG, "gfx_create: unknown precision");
  if (link_reals64 == 0) link_reals64 = 12;
  if (link_reals64 != 12 && link_reals64 != 18)
    return fail(nullptr, GFX_ERR_ARG, "gfx_create: link_reals64 must be 12 or 18");
  ctx = new gfx_ctx();
  std::memset((void*)&ctx->bank, 0, sizeof(ctx->bank));
  ctx->lx = lx;
  ctx->ly = ly;
  ctx->lz = lz;
  ctx->lt = lt;
  ctx->vol = vol;
  ctx->L = make_lattice(lx, ly, lz, lt);
  ctx->precision = precision;
  ctx->link_nr = link_reals64;
  ctx->link_nr32 = 12;
  ctx->block = 128;
  ctx->or_block[0] = ctx->or_block[1] = ctx->or_block[2] = 128;
  ctx->or_pf[0] = ctx->or_pf[1] = ctx->or_pf[2] = 2;  // odd half-sweeps in reverse order
  {
    // when the FP32 links and g (240 B per site) stream through the L2 but g alone fits
    // in half of it, g is kept there (evict_last) while the links pass as evict_first:
    // 4% faster FP32 sweeps on 32^4 (48 MB of g, 126 MB of L2)
    int dev = 0, l2 = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&l2, cudaDevAttrL2CacheSize, dev) != cudaSuccess) {
      cudaGetLastError();  // this query's own failure; the default stays 2
      l2 = 0;
    }
    if (l2 > 0 && (double)vol * 48.0 <= 0.5 * (double)l2 && (double)vol * 240.0 > (double)l2)
      ctx->or_pf[0] = 4;
  }
  ctx->or_wide = 1;
  ctx->fuse_check = 1;
  ctx->odd_checks = 1;
  ctx->Udf = ctx->Gdf = nullptr;
  ctx->udf_valid = false;
  ctx->Ur = ctx->W0 = nullptr;
  ctx->rb_valid = false;
  ctx->rb_ndir = 0;
  ctx->tune_sweep_ms[0] = ctx->tune_sweep_ms[1] = 0.0;
  ctx->tune_measure_ms[0] = ctx->tune_measure_ms[1] = 0.0;
  ctx->tune_ck = 0;
  ctx->g_active = 1;
  ctx->U64 = ctx->G64 = ctx->U32 = ctx->G32 = nullptr;
  ctx->partials = ctx->slice_sums = nullptr;
  ctx->reduced = nullptr;
  ctx->loop = nullptr;
  ctx->hist = nullptr;
  ctx->hist_cap = 0;
  ctx->loop_host = nullptr;
  ctx->reduced_host = nullptr;
  ctx->scratch_aos = nullptr;
  ctx->scratch_bytes = 0;
  ctx->mt_params = ctx->mt_seeded = ctx->mt_init = false;
  ctx->gauss = ctx->unif = nullptr;
  ctx->dev_bytes = 0;
  ctx->launches = 0;
  for (int k = 0; k < 3; k++) {
    ctx->io_ev[k] = nullptr;
    ctx->io_ms[k][0] = ctx->io_ms[k][1] = 0.0;
    ctx->io_direct[k] = 0;
  }
  for (int k = 0; k < 3; k++)
    if (cudaEventCreate(&ctx->io_ev[k]) != cudaSuccess) {
      cudaGetLastError();
      for (int j = 0; j < k; j++) cudaEventDestroy(ctx->io_ev[j]);
      delete ctx;
      return fail(nullptr, GFX_ERR_CUDA, "cudaEventCreate failed");
    }
  gfx_status s;
  if (stream) {
    ctx->stream = (cudaStream_t)stream;
    ctx->own_stream = false;
  } else {
    cudaError_t e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
      delete ctx;
      return fail(nullptr, GFX_ERR_CUDA, std::string("cudaStreamCreate: ") + cudaGetErrorString(e));
    }
    ctx->own_stream = true;
  }
#define TRY(x)           \
  do {                   \
    s = (x);             \
    if (s != GFX_OK) {   \
      std::string m = ctx->err; \
      gfx_destroy(ctx);  \
      g_global_err = m;  \
      return s;          \
    }                    \
  } while (0)
  TRY(dalloc(ctx, &ctx->U64, link_bytes64(ctx)));
  TRY(dalloc(ctx, &ctx->G64, g_bytes64(ctx)));
  if (precision != GFX_PREC_DOUBLE) {
    TRY(dalloc(ctx, &ctx->U32, link_bytes32(ctx)));
    ctx->u32_bytes = link_bytes32(ctx);
    TRY(dalloc(ctx, &ctx->G32, g_bytes32(ctx)));
  }
  // measurement partials: 3 doubles per block, blocks of >= 64 threads
  const int nbx = measure_blocks_x(ctx->L, 64);
  ctx->part_cap = 3 * 2 * lt * nbx;
  const int plaq_blocks = 2 * ((ctx->L.vh + 127) / 128);
  const int v3 = lx * ly * lz;
  if (3 * plaq_blocks > ctx->part_cap) ctx->part_cap = 3 * plaq_blocks;
  if (3 * ((v3 + 127) / 128) > ctx->part_cap) ctx->part_cap = 3 * ((v3 + 127) / 128);
  TRY(dalloc(ctx, (void**)&ctx->partials, sizeof(double) * (size_t)ctx->part_cap));
  TRY(dalloc(ctx, (void**)&ctx->slice_sums, sizeof(double) * 3 * (size_t)lt));
  TRY(dalloc(ctx, (void**)&ctx->reduced, sizeof(Reduced)));
  TRY(dalloc(ctx, (void**)&ctx->loop, sizeof(LoopState)));
  {
    cudaError_t e1 = cudaMallocHost((void**)&ctx->loop_host, sizeof(LoopState));
    cudaError_t e2 = cudaMallocHost((void**)&ctx->reduced_host, sizeof(Reduced));
    if (e1 != cudaSuccess || e2 != cudaSuccess) {
      gfx_destroy(ctx);
      return fail(nullptr, GFX_ERR_OOM, "cudaMallocHost failed");
    }
  }
  TRY(ensure_hist(ctx, 64));
#undef TRY
  *out = ctx;
  gfx_status r = gfx_unit_trafo(ctx);
  if (r != GFX_OK) {
    gfx_destroy(ctx);
    *out = nullptr;
    return r;
  }
  return GFX_OK;
}

gfx_status gfx_set_device(int device) {
  cudaError_t e = cudaSetDevice(device);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return fail(nullptr, GFX_ERR_CUDA, std::string("cudaSetDevice: ") + cudaGetErrorString(e));
  }
  return GFX_OK;
}

gfx_status gfx_set_fused_check(gfx_ctx* ctx, int fused) {
  if (!ctx) return fail(nullptr, GFX_ERR_ARG, "NULL context");
  ctx->fuse_check = fused ? 1 : 0;
  destroy_graphs(ctx);  // loop bodies captured with the other check
  return GFX_OK;
}

gfx_status gfx_synchronize(gfx_ctx* ctx) {
  if (!ctx) return fail(nullptr, GFX_ERR_ARG, "NULL context");
  CK(cudaStreamSynchronize(ctx->stream));
  return GFX_OK;
}

size_t gfx_device_bytes(const gfx_ctx* ctx) { return ctx ? ctx->dev_bytes : 0; }

gfx_status gfx_set_block(gfx_ctx* ctx, int block) {
  if (!ctx) return fail(nullptr, GFX_ERR_ARG, "NULL context");
  if (block == 0) block = 128;
  if (block < 32 || block > 256 || block % 32)
    return fail(ctx, GFX_ERR_ARG, "block must be a multiple of 32 in [32, 256]");
  ctx->block = block;
  ctx->or_block[0] = ctx->or_block[1] = block;
  destroy_graphs(ctx);  // captured loops hold the old launch shape
  return GFX_OK;
}

// ---------------------------------------------------------------------------
// fields
// ---------------------------------------------------------------------------
// Host arrays in page-locked memory from gfx_host_alloc: the layout kernels read and
// write them directly (over the CPU-GPU link, coherent on Grace systems), so a host
// transfer is one pass with no staging copy.  Other host memory goes through the
// device scratch buffer with cudaMemcpyAsync.
static gfx_status io_begin(gfx_ctx* ctx, int k) {
  CK(cudaEventRecord(ctx->io_ev[0], ctx->stream));
  ctx->io_direct[k] = 0;
  return GFX_OK;
}
static gfx_status io_end(gfx_ctx* ctx, int k) {
  CK(cudaEventRecord(ctx->io_ev[2], ctx->stream));
  CK(cudaGetLastError());
  CK(cudaEventSynchronize(ctx->io_ev[2]));
  float a = 0.f, b = 0.f;
  if (ctx->io_direct[k]) {
    CK(cudaEventElapsedTime(&b, ctx->io_ev[0], ctx->io_ev[2]));
  } else {
    CK(cudaEventElapsedTime(&a, ctx->io_ev[0], ctx->io_ev[1]));
    CK(cudaEventElapsedTime(&b, ctx->io_ev[1], ctx->io_ev[2]));
  }
  ctx->io_ms[k][0] = a;
  ctx->io_ms[k][1] = b;
  return GFX_OK;
}

gfx_status gfx_set_links(gfx_ctx* ctx, const double* su3) {
  if (!ctx || !su3) return fail(ctx, GFX_ERR_ARG, "gfx_set_links: NULL argument");
  const size_t bytes = sizeof(double) * 18 * 4 * (size_t)ctx->vol;
  gfx_status s = io_begin(ctx, 0);
  if (s) return s;
  const void* src = host_direct_ptr(su3, bytes);
  if (!src) {
    if ((s = ensure_scratch(ctx, bytes))) return s;
    CK(cudaMemcpyAsync(ctx->scratch_aos, su3, bytes, cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaEventRecord(ctx->io_ev[1], ctx->stream));
    src = ctx->scratch_aos;
  } else {
    ctx->io_direct[0] = 1;
  }
  ctx->udf_valid = false;
  ctx->rb_valid = false;  // the rebased links follow the FP64 links too
  // the FP32 12-real copy is written in the same pass (the 8-real one from U64 after)
  const bool with32 = ctx->U32 && ctx->link_nr32 == 12;
  launch_pack_links_tiled(ctx->link_nr, ctx->L, src, ctx->U64, with32 ? ctx->U32 : nullptr,
                          ctx->stream);
  if (ctx->U32 && !with32) {
    gfx_status rs = refresh_u32(ctx);
    if (rs) return rs;
  }
  return io_end(ctx, 0);
}



gfx_status gfx_get_links(gfx_ctx* ctx, double* su3) {
  if (!ctx || !su3) return fail(ctx, GFX_ERR_ARG, "gfx_get_links: NULL argument");
  const size_t bytes = sizeof(double) * 18 * 4 * (size_t)ctx->vol;
  gfx_status s = ensure_scratch(ctx, bytes);
  if (s) return s;
  launch_unpack_links(ctx->link_nr, ctx->L, ctx->U64, ctx->scratch_aos, ctx->stream);
  CK(cudaGetLastError());
  CK(cudaMemcpyAsync(su3, ctx->scratch_aos, bytes, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  return GFX_OK;
}

gfx_status gfx_set_trafo(gfx_ctx* ctx, const double* su3) {
  if (!ctx || !su3) return fail(ctx, GFX_ERR_ARG, "gfx_set_trafo: NULL argument");
  const size_t bytes = sizeof(double) * 18 * (size_t)ctx->vol;
  gfx_status s = io_begin(ctx, 1);
  if (s) return s;
  const void* src = host_direct_ptr(su3, bytes);
  if (!src) {
    if ((s = ensure_scratch(ctx, bytes))) return s;
    CK(cudaMemcpyAsync(ctx->scratch_aos, su3, bytes, cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaEventRecord(ctx->io_ev[1], ctx->stream));
    src = ctx->scratch_aos;
  } else {
    ctx->io_direct[1] = 1;
  }
  launch_pack_g_tiled(ctx->L, src, ctx->G64, ctx->stream);
  ctx->g_active = 1;
  return io_end(ctx, 1);
}

gfx_status gfx_get_trafo(gfx_ctx* ctx, double* su3) {
  if (!ctx || !su3) return fail(ctx, GFX_ERR_ARG, "gfx_get_trafo: NULL argument");
  const size_t bytes = sizeof(double) * 18 * (size_t)ctx->vol;
  gfx_status s = io_begin(ctx, 2);
  if (s) return s;
  if ((s = sync_g64(ctx))) return s;
  void* dst = host_direct_ptr(su3, bytes);
  if (dst) {
    ctx->io_direct[2] = 1;
    launch_unpack_g_tiled(ctx->L, ctx->G64, dst, ctx->stream);
  } else {
    if ((s = ensure_scratch(ctx, bytes))) return s;
    launch_unpack_g_tiled(ctx->L, ctx->G64, ctx->scratch_aos, ctx->stream);
    // here the layout kernel comes first: [0] is the copy, so time it second
    CK(cudaEventRecord(ctx->io_ev[1], ctx->stream));
    CK(cudaMemcpyAsync(su3, ctx->scratch_aos, bytes, cudaMemcpyDeviceToHost, ctx->stream));
  }
  s = io_end(ctx, 2);
  if (s == GFX_OK && !ctx->io_direct[2]) std::swap(ctx->io_ms[2][0], ctx->io_ms[2][1]);
  return s;
}

gfx_status gfx_transfer_times(const gfx_ctx* ctx, double* ms, int* direct) {
  if (!ctx || !ms) return fail(nullptr, GFX_ERR_ARG, "gfx_transfer_times: NULL argument");
  for (int k = 0; k < 3; k++) {
    ms[2 * k] = ctx->io_ms[k][0];
    ms[2 * k + 1] = ctx->io_ms[k][1];
    if (direct) direct[k] = ctx->io_direct[k];
  }
  return GFX_OK;
}

gfx_status gfx_random_trafo_haar(gfx_ctx* ctx, uint64_t seed) {
  if (!ctx) return fail(nullptr, GFX_ERR_ARG, "NULL context");
  launch_haar_g(ctx->L, (double2*)ctx->G64, seed, ctx->stream);
  CK(cudaGetLastError());
  ctx->g_active = 1;
  CK(cudaStreamSynchronize(ctx->stream));
  return GFX_OK;
}

gfx_status gfx_unit_trafo(gfx_ctx* ctx) {
  if (!ctx) return fail(nullptr, GFX_ERR_ARG, "NULL context");
  std::vector<double> h(18 * (size_t)ctx->vol);
  gfx_unit_init(h.data(), ctx->vol);
  return gfx_set_trafo(ctx, h.data());
}







gfx_status gfx_or_halfsweep(gfx_ctx* ctx, int parity, double omega, int gauge, int precision) {
  if (!ctx) return fail(nullptr, GFX_ERR_ARG, "NULL context");
  if (parity < 0 || parity > 1) return fail(ctx, GFX_ERR_ARG, "parity must be 0 or 1");
  // 2: double-float, 3: rebased FP32
  const int prec = precision == 0 ? 0 : precision == 2 ? 2 : precision == 3 ? 3 : 1;
  const int ndir = gauge == GFX_GAUGE_COULOMB ? 3 : 4;
  gfx_status s = prec == 3 ? prepare_rebased(ctx, ndir) : prepare_g(ctx, prec);
  if (s) return s;
  if (prec == 3) {
    launch_or_rebased(ndir, ctx->L, ctx->Ur, ctx->W0, ctx->G32, parity, omega, ctx->stream);
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(ctx->stream));
    return GFX_OK;
  }
  launch_or_halfsweep(prec, lnr(ctx, prec), ndir, ctx->L, prec == 0 ? ctx->U32 : ctx->U64,
                      prec == 0 ? ctx->G32 : ctx->G64, parity, omega, ctx->or_block[prec],
                      ctx->or_pf[prec], ctx->stream, ctx->or_wide);
  CK(cudaGetLastError());
  CK(cudaStreamSynchronize(ctx->stream));
  return GFX_OK;
}

gfx_status gfx_or_sweeps(gfx_ctx* ctx, int nsweeps, double omega, int gauge, int precision) {
  if (!ctx) return fail(nullptr, GFX_ERR_ARG, "NULL context");
  // 2: double-float, 3: rebased FP32
  const int prec = precision == 0 ? 0 : precision == 2 ? 2 : precision == 3 ? 3 : 1;
  const int ndir = gauge == GFX_GAUGE_COULOMB ? 3 : 4;
  gfx_status s = prec == 3 ? prepare_rebased(ctx, ndir) : prepare_g(ctx, prec);
  if (s) return s;
  enqueue_sweeps(ctx, prec, ndir, omega, nsweeps);
  CK(cudaGetLastError());
  CK(cudaStreamSynchronize(ctx->stream));
  return GFX_OK;
}

gfx_status gfx_functional(gfx_ctx* ctx, int gauge, int precision, gfx_functional_t* out) {
  if (!ctx || !out) return fail(ctx, GFX_ERR_ARG, "gfx_functional: NULL argument");
  const int ndir = gauge == GFX_GAUGE_COULOMB ? 3 : 4;
  int cprec = precision == 0 ? 0 : precision == 3 ? 3 : 1;
  if (cprec == 0 && !ctx->U32) cprec = 1;
  if (cprec == 3) {
    gfx_status s = prepare_rebased(ctx, ndir);
    if (s) return s;
  } else if (cprec == 0 || ctx->g_active >= 2) {
    gfx_status s = prepare_g(ctx, cprec);
    if (s) return s;
  }
  const int gprec = cprec == 0 ? 0 : cprec == 3 ? 3 : ctx->g_active;
  enqueue_measure(ctx, cprec, gprec, ndir);
  enqueue_reduce(ctx, ndir, false, 0, 0, 0);
  CK(cudaGetLastError());
  CK(cudaMemcpyAsync(ctx->reduced_host, ctx->reduced, sizeof(Reduced), cudaMemcpyDeviceToHost,
                     ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  const Reduced& r = *ctx->reduced_host;
  out->F = r.F;
  out->dAdA = r.dAdA;
  out->maxdAdA = r.maxdAdA;
  out->theta = r.theta;
  out->theta_slice_max = r.theta_slice_max;
  return GFX_OK;
}

gfx_status gfx_plaquette(gfx_ctx* ctx, double* plaq) {
  if (!ctx || !plaq) return fail(ctx, GFX_ERR_ARG, "gfx_plaquette: NULL argument");
  launch_plaquette(ctx->link_nr, ctx->L, ctx->U64, ctx->partials, (double*)ctx->reduced,
                   ctx->stream);
  CK(cudaGetLastError());
  CK(cudaMemcpyAsync(plaq, ctx->reduced, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  return GFX_OK;
}

gfx_status gfx_polyakov(gfx_ctx* ctx, double* re_im) {
  if (!ctx || !re_im) return fail(ctx, GFX_ERR_ARG, "gfx_polyakov: NULL argument");
  launch_polyakov(ctx->link_nr, ctx->L, ctx->U64, ctx->partials, (double*)ctx->reduced,
                  ctx->stream);
  CK(cudaGetLastError());
  CK(cudaMemcpyAsync(re_im, ctx->reduced, 2 * sizeof(double), cudaMemcpyDeviceToHost,
                     ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  return GFX_OK;
}

gfx_status gfx_apply_trafo(gfx_ctx* ctx) {
  if (!ctx) return fail(nullptr, GFX_ERR_ARG, "NULL context");
  gfx_status s = sync_g64(ctx);
  if (s) return s;
  launch_apply_trafo(ctx->link_nr, ctx->L, ctx->U64, ctx->G64, ctx->stream);
  {
    ctx->udf_valid = false;
    gfx_status rs = refresh_u32(ctx);
    if (rs) return rs;
  }
  CK(cudaGetLastError());
  return gfx_unit_trafo(ctx);
}

// ---------------------------------------------------------------------------
// convergence loop (overrelax_gauge, overrelax.cu:677-823)
// ---------------------------------------------------------------------------
void gfx_or_params_default(gfx_or_params* p) {
  std::memset(p, 0, sizeof(*p));
  p->maxit = 20000;
  p->eps = 1e-14;
  p->checkinterval = 50;
  p->omega = 1.68;
  p->criterion = GFX_CRIT_MAXDADA;
  p->gauge = GFX_GAUGE_LANDAU;
  p->switch_eps = 1e-10;
  p->plateau_ratio = 0.998;
  p->checkinterval_double = 2;
  p->use_graph = 1;
  p->record_history = 1;
}

// body of the device-side loop: ck sweeps, measurement, reduction + check
static void enqueue_body(gfx_ctx* ctx, int prec, int ndir, int ck, double omega,
                         unsigned long long handle, int use_handle) {
  const bool odd = odd_only_checks(ctx, prec);
  enqueue_sweeps_measure(ctx, prec, ndir, omega, ck, odd);
  enqueue_reduce(ctx, ndir, true, ck, handle, use_handle, odd);
}

static gfx_status get_graph(gfx_ctx* ctx, int prec, int ndir, int ck, double omega,
                            cudaGraphExec_t* exec, unsigned long long* body_out = nullptr) {
  const int odd = odd_only_checks(ctx, prec) ? 1 : 0;
  for (auto& g : ctx->graphs)
    if (g.cprec == prec && g.ndir == ndir && g.ck == ck && g.omega == omega && g.odd == odd) {
      *exec = g.exec;
      if (body_out) *body_out = g.body_launches;
      return GFX_OK;
    }
  cudaGraph_t graph;
  CK(cudaGraphCreate(&graph, 0));
  cudaGraphConditionalHandle handle;
  CK(cudaGraphConditionalHandleCreate(&handle, graph, 1, cudaGraphCondAssignDefault));
  cudaGraphNodeParams cp = {cudaGraphNodeTypeConditional};
  cp.conditional.handle = handle;
  cp.conditional.type = cudaGraphCondTypeWhile;
  cp.conditional.size = 1;
  cudaGraphNode_t node;
  CK(cudaGraphAddNode(&node, graph, nullptr, nullptr, 0, &cp));
  cudaGraph_t body = cp.conditional.phGraph_out[0];
  CK(cudaStreamBeginCaptureToGraph(ctx->stream, body, nullptr, nullptr, 0,
                                   cudaStreamCaptureModeThreadLocal));
  const unsigned long long l0 = ctx->launches;
  enqueue_body(ctx, prec, ndir, ck, omega, (unsigned long long)handle, 1);
  const unsigned long long nbody = ctx->launches - l0;
  cudaGraph_t captured;
  cudaError_t e = cudaStreamEndCapture(ctx->stream, &captured);
  if (e != cudaSuccess) {
    cudaGraphDestroy(graph);
    return fail(ctx, GFX_ERR_CUDA, std::string("stream capture: ") + cudaGetErrorString(e));
  }
  cudaGraphExec_t ex;
  CK(cudaGraphInstantiate(&ex, graph, 0));
  gfx_ctx::GraphEntry ge;
  ge.cprec = prec;
  ge.ndir = ndir;
  ge.ck = ck;
  ge.gprec = prec;
  ge.omega = omega;
  ge.exec = ex;
  ge.graph = graph;
  ge.body_launches = nbody;
  ge.odd = odd;
  ctx->graphs.push_back(ge);
  if (body_out) *body_out = nbody;
  *exec = ex;
  return GFX_OK;
}

// sweeps between two bases of the rebased FP32 polish: |a| grows slowly near
// convergence, and a new base (about one FP64 sweep of work) keeps it small
constexpr int kRebaseSweeps = 1000;

static gfx_status read_loop(gfx_ctx* ctx) {
  CK(cudaMemcpyAsync(ctx->loop_host, ctx->loop, sizeof(LoopState), cudaMemcpyDeviceToHost,
                     ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  return GFX_OK;
}
static gfx_status write_loop(gfx_ctx* ctx) {
  CK(cudaMemcpyAsync(ctx->loop, ctx->loop_host, sizeof(LoopState), cudaMemcpyHostToDevice,
                     ctx->stream));
  return GFX_OK;
}

gfx_status gfx_overrelax(gfx_ctx* ctx, const gfx_or_params* pin, gfx_or_result* res) {
  if (!ctx || !pin) return fail(ctx, GFX_ERR_ARG, "gfx_overrelax: NULL argument");
  gfx_or_params p = *pin;
  if (p.maxit < 1 || p.checkinterval < 1)
    return fail(ctx, GFX_ERR_ARG, "maxit and checkinterval must be positive");
  if (p.checkinterval_double <= 0) p.checkinterval_double = p.checkinterval;
  const int ndir = p.gauge == GFX_GAUGE_COULOMB ? 3 : 4;
  int prec = ctx->precision == GFX_PREC_DOUBLE ? 1 : 0;
  const bool handover = ctx->precision == GFX_PREC_MIXED;
  gfx_status s = prepare_g(ctx, prec);
  if (s) return s;
  if (p.checkinterval_near < 0) return fail(ctx, GFX_ERR_ARG, "checkinterval_near must be >= 0");
  if (p.polish < 0 || p.polish > 2) return fail(ctx, GFX_ERR_ARG, "polish must be 0, 1 or 2");
  ctx->odd_checks = p.fp32_checks_all_sites ? 0 : 1;
  const int ck_min = std::min(std::min(p.checkinterval, p.checkinterval_double),
                              p.checkinterval_near > 0 ? p.checkinterval_near : p.checkinterval);
  const int hist_need = p.maxit / ck_min + 8;
  s = ensure_hist(ctx, hist_need);
  if (s) return s;

  EventPair ev;
  CK(ev.create());
  cudaEvent_t e0 = ev.e0, e1 = ev.e1;
  CK(cudaEventRecord(e0, ctx->stream));

  LoopState& H = *ctx->loop_host;
  std::memset(&H, 0, sizeof(H));
  H.iter = 0;
  // checkinterval_double applies to the polish after a mixed-precision handover;
  // a single-precision-mode run checks every checkinterval sweeps (overrelax.cu:775)
  H.ck = p.checkinterval;
  H.ck_near = p.checkinterval_near;
  H.maxit = p.maxit;
  H.criterion = p.criterion;
  H.phase = handover ? 0 : 1;
  H.hist_cap = ctx->hist_cap;
  H.eps = p.eps;
  H.switch_eps = p.switch_eps;
  // plateau_ratio is per sweep: the threshold between checks k sweeps apart is ratio^k
  H.plateau_ratio = p.plateau_ratio > 0 ? std::pow(p.plateau_ratio, p.checkinterval) : 1e300;
  H.plateau_near = p.plateau_ratio > 0 && p.checkinterval_near > 0
                       ? std::pow(p.plateau_ratio, p.checkinterval_near)
                       : H.plateau_ratio;
  s = write_loop(ctx);
  if (s) return s;

  int sweeps_single = 0, sweeps_double = 0, sweeps_df = 0, sweeps_rb = 0;
  // iteration 0: sweep, then the first check (overrelax.cu:710-789)
  {
    const bool odd = odd_only_checks(ctx, prec);
    enqueue_sweeps_measure(ctx, prec, ndir, p.omega, 1, odd);
    enqueue_reduce(ctx, ndir, true, 0, 0, 0, odd);
  }
  (prec == 0 ? sweeps_single : sweeps_double)++;
  CK(cudaGetLastError());
  s = read_loop(ctx);
  if (s) return s;

  for (;;) {
    if (H.done == 0) {
      const int it0 = H.iter;
      if (p.use_graph) {
        cudaGraphExec_t ex = nullptr;
        unsigned long long nbody = 0;
        const unsigned long long before = ctx->launches;
        s = get_graph(ctx, prec, ndir, H.ck, p.omega, &ex, &nbody);
        if (s) return s;
        CK(cudaGraphLaunch(ex, ctx->stream));
        s = read_loop(ctx);
        if (s) return s;
        // one body per executed iteration (a capture counts nothing that runs)
        ctx->launches = before + (unsigned long long)((H.iter - it0) / H.ck) * nbody;
      } else {
        while (H.done == 0) {
          enqueue_body(ctx, prec, ndir, H.ck, p.omega, 0, 0);
          CK(cudaGetLastError());
          s = read_loop(ctx);
          if (s) return s;
        }
      }
      (prec == 0 ? sweeps_single : sweeps_double) += H.iter - it0;
      if (prec == 2) sweeps_df += H.iter - it0;
      if (prec == 3) sweeps_rb += H.iter - it0;
    }
    if (H.done == 4) {
      // below switch_eps: the same phase continues with the shorter interval
      H.ck = H.ck_near;
      H.done = 0;
      s = write_loop(ctx);
      if (s) return s;
      continue;
    }
    if (H.done == 5) {
      // rebased FP32 polish: a new base from the current g
      if (prec == 3 && (s = rebase(ctx, ndir))) return s;
      H.rebase_at = prec == 3 ? H.iter + kRebaseSweeps : 0;
      H.done = 0;
      s = write_loop(ctx);
      if (s) return s;
      continue;
    }
    if (H.done == 1 && prec >= 2) {
      // the double-float or rebased FP32 polish reached eps: confirm with an FP64
      // measurement; if it does not, FP64 sweeps continue
      s = prepare_g(ctx, 1);
      if (s) return s;
      prec = 1;
      H.done = 0;
      H.rebase_at = 0;
      s = write_loop(ctx);
      if (s) return s;
      enqueue_measure(ctx, 1, 1, ndir);
      enqueue_reduce(ctx, ndir, true, 0, 0, 0);
      CK(cudaGetLastError());
      s = read_loop(ctx);
      if (s) return s;
      continue;
    }
    if (H.done == 2) {
      // FP32 phase finished: widen g (reunitarized in FP64), then polish in FP64,
      // double-float or rebased FP32 (a new base from the widened g); the first check
      // verifies the handover state
      s = prepare_g(ctx, 1);
      if (s) return s;
      prec = p.polish == 2 ? 3 : p.polish == 1 ? 2 : 1;
      if (prec == 2 && (s = prepare_g(ctx, 2))) return s;
      if (prec == 3 && (s = rebase(ctx, ndir))) return s;
      H.rebase_at = prec == 3 ? H.iter + kRebaseSweeps : 0;
      H.phase = 1;
      H.done = 0;
      H.prev = 0.0;
      H.ck = p.checkinterval_double;
      H.ck_near = 0;
      s = write_loop(ctx);
      if (s) return s;
      enqueue_measure(ctx, prec, prec, ndir);
      enqueue_reduce(ctx, ndir, true, 0, 0, 0);
      CK(cudaGetLastError());
      s = read_loop(ctx);
      if (s) return s;
      continue;
    }
    break;
  }
  bool converged = H.done == 1;
  if (!converged) {
    // tail: the iterations after the last check run without a check (overrelax.cu:710-805)
    const int tail = p.maxit - 1 - H.iter;
    enqueue_sweeps(ctx, prec, ndir, p.omega, tail);
    (prec == 0 ? sweeps_single : sweeps_double) += tail > 0 ? tail : 0;
    if (prec == 2) sweeps_df += tail > 0 ? tail : 0;
    if (prec == 3) sweeps_rb += tail > 0 ? tail : 0;
    if (prec == 0 && handover) {
      s = prepare_g(ctx, 1);
      if (s) return s;
      prec = 1;
    }
  }
  CK(cudaEventRecord(e1, ctx->stream));
  CK(cudaGetLastError());
  CK(cudaEventSynchronize(e1));
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);

  const int nrec = std::min(H.nhist, H.hist_cap);
  ctx->last_hist.resize(nrec);
  if (nrec > 0 && p.record_history)
    CK(cudaMemcpy(ctx->last_hist.data(), ctx->hist, sizeof(CheckRecord) * nrec,
                  cudaMemcpyDeviceToHost));
  if (!p.record_history) ctx->last_hist.clear();
  if (res) {
    std::memset(res, 0, sizeof(*res));
    res->converged = converged ? 1 : 0;
    // reference semantics: the converging check's iteration, or -1 (maxit when the
    // last value equals eps exactly, overrelax.cu:816-822)
    double last = H.criterion == 0 ? H.last_max : H.criterion == 1 ? H.last_theta
                                                                    : H.last_theta_slice_max;
    res->iterations = converged ? H.iter : (last > p.eps ? -1 : p.maxit);
    res->sweeps_single = sweeps_single;
    res->sweeps_double = sweeps_double;
    res->sweeps = sweeps_single + sweeps_double;
    res->sweeps_polish_df = sweeps_df;
    res->sweeps_polish_fp32 = sweeps_rb;
    res->checks = H.nhist;
    res->final_values.F = H.last_F;
    res->final_values.dAdA = H.last_dAdA;
    res->final_values.maxdAdA = H.last_max;
    res->final_values.theta = H.last_theta;
    res->final_values.theta_slice_max = H.last_theta_slice_max;
    res->ms = ms;
  }
  return converged ? GFX_OK : GFX_ERR_NOT_CONVERGED;
}

int gfx_or_history(const gfx_ctx* ctx, gfx_check_record* out, int cap) {
  if (!ctx) return 0;
  const int n = std::min((int)ctx->last_hist.size(), cap);
  for (int k = 0; k < n; k++) {
    const CheckRecord& r = ctx->last_hist[k];
    out[k].iter = r.iter;
    out[k].phase = r.phase;
    out[k].F = r.F;
    out[k].dAdA = r.dAdA;
    out[k].maxdAdA = r.maxdAdA;
    out[k].theta = r.theta;
    out[k].theta_slice_max = r.theta_slice_max;
  }
  return (int)ctx->last_hist.size();
}

// ---------------------------------------------------------------------------
// Mersenne Twister bank
// ---------------------------------------------------------------------------
static gfx_status mt_alloc(gfx_ctx* ctx) {
  if (ctx->bank.a) return GFX_OK;
  gfx_status s;
  if ((s = dalloc(ctx, (void**)&ctx->bank.a, 4 * kMTCount))) return s;
  if ((s = dalloc(ctx, (void**)&ctx->bank.b, 4 * kMTCount))) return s;
  if ((s = dalloc(ctx, (void**)&ctx->bank.c, 4 * kMTCount))) return s;
  if ((s = dalloc(ctx, (void**)&ctx->bank.seed, 4 * kMTCount))) return s;
  if ((s = dalloc(ctx, (void**)&ctx->bank.status, 4 * kMTCount * kMTN))) return s;
  return GFX_OK;
}

static gfx_status mt_upload(gfx_ctx* ctx) {
  std::vector<uint32_t> a(kMTCount), b(kMTCount), c(kMTCount), sd(kMTCount);
  for (int r = 0; r < kMTCount; r++) {
    a[r] = ctx->h_params[4 * r];
    b[r] = ctx->h_params[4 * r + 1];
    c[r] = ctx->h_params[4 * r + 2];
    sd[r] = ctx->h_params[4 * r + 3];
  }
  CK(cudaMemcpy(ctx->bank.a, a.data(), 4 * kMTCount, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(ctx->bank.b, b.data(), 4 * kMTCount, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(ctx->bank.c, c.data(), 4 * kMTCount, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(ctx->bank.seed, sd.data(), 4 * kMTCount, cudaMemcpyHostToDevice));
  return GFX_OK;
}

gfx_status gfx_mt_load_params(gfx_ctx* ctx, const uint32_t* params) {
  if (!ctx || !params) return fail(ctx, GFX_ERR_ARG, "gfx_mt_load_params: NULL argument");
  gfx_status s = mt_alloc(ctx);
  if (s) return s;
  std::memcpy(ctx->h_params, params, sizeof(ctx->h_params));
  ctx->mt_params = true;
  ctx->mt_seeded = false;
  ctx->mt_init = false;
  return mt_upload(ctx);
}

// loadMTGPU (MersenneTwister.cu:79-92): 4096 x {matrix_a, mask_b, mask_c, seed},
// little-endian uint32
gfx_status gfx_mt_load_file(gfx_ctx* ctx, const char* path) {
  if (!ctx || !path) return fail(ctx, GFX_ERR_ARG, "gfx_mt_load_file: NULL argument");
  FILE* f = std::fopen(path, "rb");
  if (!f) return fail(ctx, GFX_ERR_IO, std::string("cannot open twister parameters ") + path);
  std::vector<uint32_t> buf(4 * kMTCount);
  unsigned char raw[16 * kMTCount];
  size_t n = std::fread(raw, 1, sizeof(raw), f);
  std::fclose(f);
  if (n != sizeof(raw))
    return fail(ctx, GFX_ERR_IO, std::string("twister parameter file truncated: ") + path);
  for (int k = 0; k < 4 * kMTCount; k++)
    buf[k] = (uint32_t)raw[4 * k] | ((uint32_t)raw[4 * k + 1] << 8) |
             ((uint32_t)raw[4 * k + 2] << 16) | ((uint32_t)raw[4 * k + 3] << 24);
  return gfx_mt_load_params(ctx, buf.data());
}

gfx_status gfx_mt_set_seeds(gfx_ctx* ctx, const uint32_t* seeds) {
  if (!ctx || !seeds) return fail(ctx, GFX_ERR_ARG, "gfx_mt_set_seeds: NULL argument");
  if (!ctx->mt_params) return fail(ctx, GFX_ERR_STATE, "twister parameters not loaded");
  for (int r = 0; r < kMTCount; r++) ctx->h_params[4 * r + 3] = seeds[r];
  ctx->mt_seeded = true;
  return mt_upload(ctx);
}

gfx_status gfx_mt_seed(gfx_ctx* ctx, unsigned int mtseed) {
  std::vector<int32_t> r(kMTCount);
  gfx_glibc_rand(mtseed, kMTCount, r.data());
  std::vector<uint32_t> s(kMTCount);
  for (int k = 0; k < kMTCount; k++) s[k] = (uint32_t)r[k];
  return gfx_mt_set_seeds(ctx, s.data());
}

static int align_up2(int q) { return (q % 2) ? q + 1 : q; }
static int nper_of(int n) { return align_up2(n % kMTCount ? n / kMTCount + 1 : n / kMTCount); }

gfx_status gfx_mt_init(gfx_ctx* ctx, int n_gauss, int n_unif) {
  if (!ctx) return fail(nullptr, GFX_ERR_ARG, "NULL context");
  if (!ctx->mt_params || !ctx->mt_seeded)
    return fail(ctx, GFX_ERR_STATE, "twister bank needs parameters and seeds before init");
  if (n_gauss < 1 || n_unif < 1) return fail(ctx, GFX_ERR_ARG, "field sizes must be positive");
  if (ctx->gauss) {
    cudaFree(ctx->gauss);
    ctx->dev_bytes -= sizeof(float) * (size_t)kMTCount * ctx->nper_g;
    ctx->gauss = nullptr;
  }
  if (ctx->unif) {
    cudaFree(ctx->unif);
    ctx->dev_bytes -= sizeof(float) * (size_t)kMTCount * ctx->nper_u;
    ctx->unif = nullptr;
  }
  ctx->n_gauss = n_gauss;
  ctx->n_unif = n_unif;
  ctx->nper_g = nper_of(n_gauss);
  ctx->nper_u = nper_of(n_unif);
  gfx_status s;
  if ((s = dalloc(ctx, (void**)&ctx->gauss, sizeof(float) * (size_t)kMTCount * ctx->nper_g))) return s;
  if ((s = dalloc(ctx, (void**)&ctx->unif, sizeof(float) * (size_t)kMTCount * ctx->nper_u))) return s;
  s = mt_upload(ctx);
  if (s) return s;
  launch_mt_generate(ctx->bank, ctx->gauss, ctx->nper_g, 0, 1, ctx->stream);
  launch_mt_generate(ctx->bank, ctx->unif, ctx->nper_u, 0, 0, ctx->stream);
  CK(cudaGetLastError());
  CK(cudaStreamSynchronize(ctx->stream));
  ctx->mt_init = true;
  return GFX_OK;
}

static void enqueue_mt_update(gfx_ctx* ctx) {
  launch_mt_generate(ctx->bank, ctx->gauss, ctx->nper_g, 1, 1, ctx->stream);
  launch_mt_generate(ctx->bank, ctx->unif, ctx->nper_u, 1, 0, ctx->stream);
}

gfx_status gfx_mt_update(gfx_ctx* ctx) {
  if (!ctx) return fail(nullptr, GFX_ERR_ARG, "NULL context");
  if (!ctx->mt_init) return fail(ctx, GFX_ERR_STATE, "update_MT before init_MT");
  enqueue_mt_update(ctx);
  CK(cudaGetLastError());
  CK(cudaStreamSynchronize(ctx->stream));
  return GFX_OK;
}

gfx_status gfx_mt_sizes(const gfx_ctx* ctx, int* nper_gauss, int* nper_unif) {
  if (!ctx) return GFX_ERR_ARG;
  if (nper_gauss) *nper_gauss = ctx->nper_g;
  if (nper_unif) *nper_unif = ctx->nper_u;
  return GFX_OK;
}

gfx_status gfx_mt_read(gfx_ctx* ctx, float* gauss, float* unif, uint32_t* state,
                       uint32_t* seeds) {
  if (!ctx) return fail(nullptr, GFX_ERR_ARG, "NULL context");
  if (!ctx->mt_init) return fail(ctx, GFX_ERR_STATE, "twister bank not initialized");
  if (gauss)
    CK(cudaMemcpyAsync(gauss, ctx->gauss, sizeof(float) * (size_t)kMTCount * ctx->nper_g,
                       cudaMemcpyDeviceToHost, ctx->stream));
  if (unif)
    CK(cudaMemcpyAsync(unif, ctx->unif, sizeof(float) * (size_t)kMTCount * ctx->nper_u,
                       cudaMemcpyDeviceToHost, ctx->stream));
  if (state)
    CK(cudaMemcpyAsync(state, ctx->bank.status, 4 * (size_t)kMTCount * kMTN,
                       cudaMemcpyDeviceToHost, ctx->stream));
  if (seeds)
    CK(cudaMemcpyAsync(seeds, ctx->bank.seed, 4 * (size_t)kMTCount, cudaMemcpyDeviceToHost,
                       ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  return GFX_OK;
}

// ---------------------------------------------------------------------------
// simulated annealing (simulated_annealing.cu:265-476)
// ---------------------------------------------------------------------------
double gfx_sa_temperature(const gfx_sa_params* p, int i) {
  double a, temperature;
  if (p->Tmax == p->Tmin) {
    temperature = p->Tmax;
  } else if (p->expo == 0) {
    a = (double)i / (double)(p->N - 1);
    temperature = std::pow(p->Tmin / p->Tmax, a) * p->Tmax;
  } else if (p->expo == -1) {
    a = (p->Tmin - p->Tmax) / (double)(p->N - 1);
    temperature = a * i + p->Tmax;
  } else {
    a = std::pow(p->Tmin, -p->expo) - std::pow(p->Tmax, -p->expo);
    a = a / (double)(p->N - 1);
    temperature = std::pow(a * i + std::pow(p->Tmax, -p->expo), -1.0 / p->expo);
  }
  return temperature;
}

static gfx_status check_sa_fields(gfx_ctx* ctx) {
  if (!ctx->mt_init) return fail(ctx, GFX_ERR_STATE, "simulated annealing needs init_MT");
  if ((long long)kMTCount * ctx->nper_g < ctx->vol / 2 ||
      (long long)kMTCount * ctx->nper_u < 2 * ctx->vol)
    return fail(ctx, GFX_ERR_STATE, "random fields smaller than V/2 gauss + 2V uniform");
  return GFX_OK;
}

gfx_status gfx_sa_halfsweep(gfx_ctx* ctx, int parity, double beta, int precision) {
  if (!ctx) return fail(nullptr, GFX_ERR_ARG, "NULL context");
  gfx_status s = check_sa_fields(ctx);
  if (s) return s;
  const int prec = precision == 0 ? 0 : 1;
  if ((s = prepare_g(ctx, prec))) return s;
  launch_sa_heatbath(prec, lnr(ctx, prec), ctx->L, prec == 0 ? ctx->U32 : ctx->U64,
                     prec == 0 ? ctx->G32 : ctx->G64, parity, beta, ctx->gauss, ctx->unif,
                     ctx->block, ctx->stream);
  CK(cudaGetLastError());
  CK(cudaStreamSynchronize(ctx->stream));
  return GFX_OK;
}

gfx_status gfx_micro_halfsweep(gfx_ctx* ctx, int parity, int gauge, int precision) {
  if (!ctx) return fail(nullptr, GFX_ERR_ARG, "NULL context");
  const int prec = precision == 0 ? 0 : 1;
  gfx_status s = prepare_g(ctx, prec);
  if (s) return s;
  launch_micro(prec, lnr(ctx, prec), gauge == GFX_GAUGE_COULOMB ? 3 : 4, ctx->L,
               prec == 0 ? ctx->U32 : ctx->U64, prec == 0 ? ctx->G32 : ctx->G64, parity,
               ctx->block, ctx->stream);
  CK(cudaGetLastError());
  CK(cudaStreamSynchronize(ctx->stream));
  return GFX_OK;
}

gfx_status gfx_simanneal_range(gfx_ctx* ctx, const gfx_sa_params* p, int first, int count) {
  if (!ctx || !p) return fail(ctx, GFX_ERR_ARG, "gfx_simanneal_range: NULL argument");
  if (p->N < 1 || first < 0 || count < 0 || first + count > p->N)
    return fail(ctx, GFX_ERR_ARG, "SA step range outside [0, N)");
  gfx_status s = check_sa_fields(ctx);
  if (s) return s;
  const int prec = ctx->precision == GFX_PREC_DOUBLE ? 1 : 0;
  if ((s = prepare_g(ctx, prec))) return s;
  const void* U = prec == 0 ? ctx->U32 : ctx->U64;
  void* G = prec == 0 ? ctx->G32 : ctx->G64;
  for (int i = first; i < first + count; i++) {
    // set_sa_temperature: beta = 1/T (simulated_annealing.cu:292)
    const double beta = 1.0 / gfx_sa_temperature(p, i);
    for (int par = 0; par < 2; par++) {
      launch_sa_heatbath(prec, lnr(ctx, prec), ctx->L, U, G, par, beta, ctx->gauss, ctx->unif,
                         ctx->block, ctx->stream);
      enqueue_mt_update(ctx);
    }
    for (int m = 0; m < p->nmicro; m++)
      for (int par = 0; par < 2; par++)
        launch_micro(prec, lnr(ctx, prec), 4, ctx->L, U, G, par, ctx->block, ctx->stream);
  }
  CK(cudaGetLastError());
  CK(cudaStreamSynchronize(ctx->stream));
  return GFX_OK;
}

gfx_status gfx_simanneal(gfx_ctx* ctx, const gfx_sa_params* p, gfx_functional_t* last) {
  gfx_status s = gfx_simanneal_range(ctx, p, 0, p ? p->N : 0);
  if (s) return s;
  if (last) return gfx_functional(ctx, GFX_GAUGE_LANDAU, 1, last);
  return GFX_OK;
}

// ---------------------------------------------------------------------------
// thermalization (heatbath_thermalization.cu:557-841)
// ---------------------------------------------------------------------------
gfx_status gfx_link_heatbath_halfsweep(gfx_ctx* ctx, int parity, int nu, double beta,
                                       int variant) {
  if (!ctx) return fail(nullptr, GFX_ERR_ARG, "NULL context");
  if (!ctx->mt_init) return fail(ctx, GFX_ERR_STATE, "link heatbath needs init_MT");
  if ((long long)kMTCount * ctx->nper_g < 2 * ctx->vol ||
      (long long)kMTCount * ctx->nper_u < 8 * ctx->vol)
    return fail(ctx, GFX_ERR_STATE, "random fields smaller than 2V gauss + 8V uniform");
  launch_link_heatbath(ctx->link_nr, ctx->L, ctx->U64, parity, nu, beta / 3.0, ctx->gauss,
                       ctx->unif, variant, 128, ctx->stream);
  {
    ctx->udf_valid = false;
    gfx_status rs = refresh_u32(ctx);
    if (rs) return rs;
  }
  CK(cudaGetLastError());
  CK(cudaStreamSynchronize(ctx->stream));
  return GFX_OK;
}

gfx_status gfx_thermalize(gfx_ctx* ctx, const gfx_therm_params* p, double* plaq, int plaq_cap) {
  if (!ctx || !p) return fail(ctx, GFX_ERR_ARG, "gfx_thermalize: NULL argument");
  if (!ctx->mt_init) return fail(ctx, GFX_ERR_STATE, "thermalization needs init_MT");
  if ((long long)kMTCount * ctx->nper_g < 2 * ctx->vol ||
      (long long)kMTCount * ctx->nper_u < 8 * ctx->vol)
    return fail(ctx, GFX_ERR_STATE, "random fields smaller than 2V gauss + 8V uniform");
  if (p->precision < 0 || p->precision > 1) return fail(ctx, GFX_ERR_ARG, "thermalize precision must be 0 or 1");
  const bool f32 = p->precision == 1;
  const int nr32 = ctx->link_nr32;
  if (f32) {
    if (!ctx->U32) return fail(ctx, GFX_ERR_STATE, "FP32 thermalization needs a SINGLE or MIXED context");
    // the FP32 copy in 12 reals while the heatbath keeps it in step with the FP64 links
    gfx_status s = nr32 != 12 ? set_link_layout32(ctx, 12) : refresh_u32(ctx);
    if (s) return s;
  }
  const double beta3 = p->beta / 3.0;
  const int checkint = p->checkint > 0 ? p->checkint : p->Nsweep + 1;
  int np = 0;
  for (int i = 0; i < p->Nsweep; i++) {
    for (int nu = 0; nu < 4; nu++)
      for (int par = 0; par < 2; par++) {
        if (f32)
          launch_link_heatbath_f32(ctx->link_nr, ctx->L, ctx->U64, ctx->U32, par, nu, beta3,
                                   ctx->gauss, ctx->unif, p->variant, ctx->stream);
        else
          launch_link_heatbath(ctx->link_nr, ctx->L, ctx->U64, par, nu, beta3, ctx->gauss,
                               ctx->unif, p->variant, 128, ctx->stream);
        enqueue_mt_update(ctx);
      }
    if (i % checkint == 0 && plaq && np < plaq_cap) {
      launch_plaquette(ctx->link_nr, ctx->L, ctx->U64, ctx->partials, (double*)ctx->reduced,
                       ctx->stream);
      CK(cudaMemcpyAsync(plaq + np, ctx->reduced, sizeof(double), cudaMemcpyDeviceToHost,
                         ctx->stream));
      np++;
    }
  }
  {
    ctx->udf_valid = false;
    gfx_status rs = f32 && nr32 != 12 ? set_link_layout32(ctx, nr32) : refresh_u32(ctx);
    if (rs) return rs;
  }
  CK(cudaGetLastError());
  CK(cudaStreamSynchronize(ctx->stream));
  return GFX_OK;
}

gfx_status gfx_time_sweeps(gfx_ctx* ctx, int nsweeps, double omega, int gauge, int precision,
                           double* ms) {
  if (!ctx || !ms || nsweeps < 1) return fail(ctx, GFX_ERR_ARG, "gfx_time_sweeps: bad argument");
  // 2: double-float, 3: rebased FP32
  const int prec = precision == 0 ? 0 : precision == 2 ? 2 : precision == 3 ? 3 : 1;
  const int ndir = gauge == GFX_GAUGE_COULOMB ? 3 : 4;
  gfx_status s = prec == 3 ? prepare_rebased(ctx, ndir) : prepare_g(ctx, prec);
  if (s) return s;
  // the sweeps run as one CUDA graph, back to back as inside the solve's device loop
  CK(cudaStreamSynchronize(ctx->stream));
  CK(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
  enqueue_sweeps(ctx, prec, ndir, omega, nsweeps);
  cudaGraph_t graph;
  CK(cudaStreamEndCapture(ctx->stream, &graph));
  cudaGraphExec_t exec;
  cudaError_t ge = cudaGraphInstantiate(&exec, graph, 0);
  cudaGraphDestroy(graph);
  CK(ge);
  EventPair ev;
  cudaError_t err = ev.create();
  if (err == cudaSuccess) err = cudaEventRecord(ev.e0, ctx->stream);
  if (err == cudaSuccess) err = cudaGraphLaunch(exec, ctx->stream);
  if (err == cudaSuccess) err = cudaEventRecord(ev.e1, ctx->stream);
  if (err == cudaSuccess) err = cudaEventSynchronize(ev.e1);
  float t = 0.f;
  if (err == cudaSuccess) err = cudaEventElapsedTime(&t, ev.e0, ev.e1);
  cudaGraphExecDestroy(exec);
  CK(err);
  *ms = t;
  return GFX_OK;
}

unsigned long long gfx_launch_count(const gfx_ctx* ctx) { return ctx ? ctx->launches : 0; }

void* gfx_host_alloc(size_t bytes) {
  void* p = nullptr;
  // portable and mapped: every context of the process may read and write it directly
  if (cudaHostAlloc(&p, bytes, cudaHostAllocPortable | cudaHostAllocMapped) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  std::lock_guard<std::mutex> lk(g_pinned_mu);
  g_pinned[(uintptr_t)p] = bytes;
  return p;
}

void gfx_host_free(void* p) {
  if (!p) return;
  {
    std::lock_guard<std::mutex> lk(g_pinned_mu);
    g_pinned.erase((uintptr_t)p);
  }
  cudaFreeHost(p);
}

}  // extern "C"
