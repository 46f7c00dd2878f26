// gfx_context.h -- the context behind a gfx_ctx handle and the helpers that the
// context's translation units share (gfx_api.cu: lifecycle, fields, sweeps and the
// solve loop; gfx_tune.cu: launch tuning; gfx_ctx_files.cu: files and checkpoints).
#pragma once

#include <string>
#include <vector>

#include "../../include/gfx.h"
#include "gfx_internal.h"

// One context = one lattice on the current device, with
//   U64 : links, FP64, 12 or 18 reals, even/odd SoA (authoritative copy)
//   G64 : gauge transformation, FP64, 12 reals
//   U32, G32 : FP32 copies for the single/mixed-precision sweeps (links 12 or 8 reals)
//   Udf, Gdf : double-float copies for the polish sweeps
//   Ur, W0 : the base of the rebased FP32 polish sweeps (gfx_rebased.cu)
// and the work buffers of the reductions, the convergence loop and the twister bank.
struct gfx_ctx {
  int lx, ly, lz, lt;
  long long vol;
  gfx::Lattice L;
  int precision;
  int link_nr;    // FP64 link storage: 12 or 18
  int link_nr32;  // FP32 link copy: 12 or 8
  size_t u32_bytes;
  int block;
  int or_block[3];  // OR/SA half-sweep block size, FP32 [0], FP64 [1], double-float [2]
  int or_wide;      // FP32 half-sweep kernel with its full register set (1) or 64 (0)
  int or_pf[3];     // OR half-sweep loads: 0 plain, 1 after an L2 bulk prefetch, 2 plain
                    // with the odd half-sweep's blocks in reverse order (the default), 3 and
                    // 4 as 2 with FP32 12-real g as L2 evict_last (4: links evict_first)
  int fuse_check;   // FP32 checks fused into the last odd half-sweep when possible (default 1)
  int odd_checks;   // the FP32-phase checks of a mixed solve may measure the odd sites only
                    // (gfx_or_params.fp32_checks_all_sites = 0); set per gfx_overrelax
  double tune_sweep_ms[2], tune_measure_ms[2];
  int tune_ck;
  cudaStream_t stream;
  bool own_stream;
  int g_active;  // 0: G32 holds the current g, 1: G64 does, 2: Gdf does,
                 // 3: g = (1 + a) G64 with a in G32 (rebased FP32 sweeps)
  void* Udf;     // double-float links (18 reals) and g (12 reals) of the polish sweeps
  void* Gdf;
  bool udf_valid;
  void* Ur;      // rebased FP32 sweeps: links g_c U g_c^+ (FP32, 12 reals) and split star
  void* W0;
  bool rb_valid;  // Ur and W0 belong to the current base, links and rb_ndir
  int rb_ndir;
  // fields
  void* U64;
  void* G64;
  void* U32;
  void* G32;
  // reductions
  double* partials;
  int part_cap;  // doubles
  double* slice_sums;
  gfx::Reduced* reduced;
  gfx::LoopState* loop;
  gfx::CheckRecord* hist;
  int hist_cap;
  gfx::LoopState* loop_host;  // pinned
  gfx::Reduced* reduced_host; // pinned
  double* scratch_aos;   // device staging for host<->device layout conversion
  size_t scratch_bytes;
  // twister bank
  gfx::MTBank bank;
  bool mt_params;
  bool mt_seeded;
  bool mt_init;
  int n_gauss, n_unif, nper_g, nper_u;
  float* gauss;
  float* unif;
  uint32_t h_params[4 * gfx::kMTCount];
  // graph cache for the convergence loop
  struct GraphEntry {
    int cprec, ndir, ck, gprec;
    double omega;
    cudaGraphExec_t exec;
    cudaGraph_t graph;
    unsigned long long body_launches;  // kernels in one execution of the loop body
    int odd;                           // captured with odd-site FP32 checks
  };
  std::vector<GraphEntry> graphs;
  std::vector<gfx::CheckRecord> last_hist;
  size_t dev_bytes;
  unsigned long long launches;  // kernels enqueued by this context (graph bodies included)
  // device times of the last set_links, set_trafo, get_trafo: [k][0] the host<->device
  // copy (0 when the GPU reached the caller's page-locked buffer directly), [k][1] the
  // layout kernels; io_direct[k] = 1 for the direct path
  cudaEvent_t io_ev[3];
  double io_ms[3][2];
  int io_direct[3];
  std::string err;
};

// return a CUDA failure as GFX_ERR_CUDA from a function with a `ctx` in scope
#define CK(call)                                                                     \
  do {                                                                               \
    cudaError_t e_ = (call);                                                         \
    if (e_ != cudaSuccess) {                                                         \
      return fail(ctx, GFX_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    }                                                                                \
  } while (0)

namespace gfx {

// the device address of caller memory inside one gfx_host_alloc allocation (16-byte
// aligned), or nullptr
void* host_direct_ptr(const void* p, size_t bytes);
// record msg as the context's and the library's last error; returns s
gfx_status fail(gfx_ctx* ctx, gfx_status s, const std::string& msg);
const std::string& global_error();

// buffer sizes (8 link blocks or 2 g parities x 16-byte planes x Vh)
inline size_t link_bytes64(const gfx_ctx* c) { return (size_t)8 * (c->link_nr / 2) * 16 * (size_t)c->L.vh; }
inline size_t link_bytes32(const gfx_ctx* c) { return (size_t)8 * 3 * 16 * (size_t)c->L.vh; }
inline size_t g_bytes64(const gfx_ctx* c) { return (size_t)2 * 6 * 16 * (size_t)c->L.vh; }
inline size_t g_bytes32(const gfx_ctx* c) { return (size_t)2 * 3 * 16 * (size_t)c->L.vh; }
// FP32 links: 12 reals = 3 planes; 8 reals = 2 planes + the 3 planes of exact rows
// kept for the links the 8-parameter form declines
inline size_t link_bytes32_for(const gfx_ctx* c, int nr32) {
  return (size_t)8 * (nr32 == 8 ? 5 : 3) * 16 * (size_t)c->L.vh;
}
// the layout of the link field that precision prec (0 FP32, 1 FP64) reads
inline int lnr(const gfx_ctx* c, int prec) { return prec == 0 ? c->link_nr32 : c->link_nr; }
inline void ctx_dims(const gfx_ctx* ctx, int d[4]) {
  d[0] = ctx->lx;
  d[1] = ctx->ly;
  d[2] = ctx->lz;
  d[3] = ctx->lt;
}

gfx_status dalloc(gfx_ctx* ctx, void** p, size_t bytes);
gfx_status ensure_scratch(gfx_ctx* ctx, size_t bytes);
void destroy_graphs(gfx_ctx* ctx);
// the FP32 link copy from the FP64 links, in the current FP32 layout
gfx_status refresh_u32(gfx_ctx* ctx);
// make G64 the current g (from G32, from Gdf, or composed as (1 + a) G64 on a rebased base)
gfx_status sync_g64(gfx_ctx* ctx);
gfx_status ensure_df(gfx_ctx* ctx);
// make the g of precision prec (0 FP32, 1 FP64, 2 double-float) the current one; the
// rebased FP32 state comes from prepare_rebased
gfx_status prepare_g(gfx_ctx* ctx, int prec);
// a new base for the rebased FP32 sweeps over ndir directions: g_c = g, a = 0
gfx_status rebase(gfx_ctx* ctx, int ndir);
// the rebased state for ndir directions, keeping a valid base
gfx_status prepare_rebased(gfx_ctx* ctx, int ndir);
void enqueue_sweep(gfx_ctx* ctx, int prec, int ndir, double omega);
void enqueue_sweeps(gfx_ctx* ctx, int prec, int ndir, double omega, int n);
void enqueue_measure(gfx_ctx* ctx, int cprec, int gprec, int ndir);
// n sweeps followed by the check's measurement (the same partials either way; FP32
// with fused_check_ok: the last odd half-sweep writes the odd sites' partials)
void enqueue_sweeps_measure(gfx_ctx* ctx, int prec, int ndir, double omega, int n,
                            bool odd_only = false);
// the FP32-phase checks of a mixed solve measure the odd sites only (gfx_internal.h)
bool odd_only_checks(const gfx_ctx* ctx, int prec);
void enqueue_reduce(gfx_ctx* ctx, int ndir, bool with_loop, int advance,
                    unsigned long long handle, int use_handle, bool odd_only = false);
// re-pack the FP64 links as nr reals per link (12 or 18)
gfx_status relayout_links(gfx_ctx* ctx, int nr);
// FP32 link layout 12 or 8
gfx_status set_link_layout32(gfx_ctx* ctx, int nr32);
// the links of U64 (or of src, a device field in U64's layout) as host su3
gfx_status links_to_host(gfx_ctx* ctx, const void* src, std::vector<double>& out);

}  // namespace gfx
