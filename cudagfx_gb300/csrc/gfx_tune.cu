// gfx_tune.cu -- launch tuning of a context: gfx_get_tuning, gfx_set_tuning and
// gfx_autotune (block size, L2 prefetch, FP64 and FP32 link layouts, check interval),
// with the on-disk result cache.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <string>
#include <vector>

#include "../../include/gfx.h"
#include "gfx_context.h"

using namespace gfx;

extern "C" {

// ---------------------------------------------------------------------------
// launch tuning
// ---------------------------------------------------------------------------
gfx_status gfx_get_tuning(const gfx_ctx* ctx, gfx_tuning* t) {
  if (!ctx || !t) return fail(nullptr, GFX_ERR_ARG, "gfx_get_tuning: NULL argument");
  for (int p = 0; p < 2; p++) {
    t->block[p] = ctx->or_block[p];
    t->staging[p] = ctx->or_pf[p];
    t->sweep_ms[p] = ctx->tune_sweep_ms[p];
    t->check_ms[p] = ctx->tune_measure_ms[p];
  }
  t->link_reals64 = ctx->link_nr;
  t->link_reals32 = ctx->link_nr32;
  t->checkinterval = ctx->tune_ck;
  t->wide_regs = ctx->or_wide;
  return GFX_OK;
}


static bool valid_block(int b) { return b >= 32 && b <= 256 && b % 32 == 0; }


gfx_status gfx_set_tuning(gfx_ctx* ctx, const gfx_tuning* t) {
  if (!ctx || !t) return fail(ctx, GFX_ERR_ARG, "gfx_set_tuning: NULL argument");
  for (int p = 0; p < 2; p++) {
    if (!valid_block(t->block[p]))
      return fail(ctx, GFX_ERR_ARG, "gfx_set_tuning: block must be a multiple of 32 in [32, 256]");
    if (t->staging[p] < 0 || t->staging[p] > 4)
      return fail(ctx, GFX_ERR_ARG, "gfx_set_tuning: staging must be 0 to 4");
  }
  if (t->link_reals64 != 0 && t->link_reals64 != 12 && t->link_reals64 != 18)
    return fail(ctx, GFX_ERR_ARG, "gfx_set_tuning: link_reals64 must be 0, 12 or 18");
  if (t->checkinterval < 0) return fail(ctx, GFX_ERR_ARG, "gfx_set_tuning: checkinterval < 0");
  if (t->link_reals32 != 0 && t->link_reals32 != 12 && t->link_reals32 != 8)
    return fail(ctx, GFX_ERR_ARG, "gfx_set_tuning: link_reals32 must be 0, 12 or 8");
  if (t->wide_regs != 0 && t->wide_regs != 1)
    return fail(ctx, GFX_ERR_ARG, "gfx_set_tuning: wide_regs must be 0 or 1");
  if (t->link_reals64) {
    gfx_status s = relayout_links(ctx, t->link_reals64);
    if (s) return s;
  }
  if (t->link_reals32 && t->link_reals32 != ctx->link_nr32 && ctx->U32) {
    gfx_status s = set_link_layout32(ctx, t->link_reals32);
    if (s) return s;
  }
  for (int p = 0; p < 2; p++) {
    ctx->or_block[p] = t->block[p];
    ctx->or_pf[p] = t->staging[p];
  }
  ctx->or_wide = t->wide_regs;
  ctx->tune_ck = t->checkinterval;
  destroy_graphs(ctx);
  return GFX_OK;
}

// device time of n repetitions of enqueue(), after one untimed repetition
static gfx_status time_reps(gfx_ctx* ctx, int n, const std::function<void()>& enqueue,
                            double* ms) {
  EventPair ev;
  CK(ev.create());
  enqueue();
  CK(cudaEventRecord(ev.e0, ctx->stream));
  for (int k = 0; k < n; k++) enqueue();
  CK(cudaEventRecord(ev.e1, ctx->stream));
  CK(cudaEventSynchronize(ev.e1));
  float t = 0.f;
  CK(cudaEventElapsedTime(&t, ev.e0, ev.e1));
  CK(cudaGetLastError());
  *ms = t / n;
  return GFX_OK;
}

static std::string tune_key(const gfx_ctx* ctx, int ndir) {
  int dev = 0;
  cudaGetDevice(&dev);
  cudaDeviceProp prop;
  if (cudaGetDeviceProperties(&prop, dev) != cudaSuccess) {
    cudaGetLastError();
    std::snprintf(prop.name, sizeof(prop.name), "unknown");
    prop.multiProcessorCount = 0;
  }
  char key[512];
  std::snprintf(key, sizeof(key), "%s|%d|%dx%dx%dx%d|prec%d|ndir%d", prop.name,
                prop.multiProcessorCount, ctx->lx, ctx->ly, ctx->lz, ctx->lt, ctx->precision, ndir);
  for (char* c = key; *c; c++)
    if (*c == '\t' || *c == '\n') *c = ' ';
  return key;
}

// cache line: key TAB block0 staging0 block1 staging1 link_reals64 link_reals32 sweep_ms0
// sweep_ms1 check_ms0 check_ms1 wide_regs
static bool cache_lookup(const char* path, const std::string& key, gfx_tuning* t) {
  FILE* f = std::fopen(path, "r");
  if (!f) return false;
  char line[1024];
  bool hit = false;
  while (std::fgets(line, sizeof(line), f)) {
    char* tab = std::strchr(line, '\t');
    if (!tab || std::string(line, tab - line) != key) continue;
    gfx_tuning c;
    std::memset(&c, 0, sizeof(c));
    if (std::sscanf(tab + 1, "%d %d %d %d %d %d %lf %lf %lf %lf %d", &c.block[0], &c.staging[0],
                    &c.block[1], &c.staging[1], &c.link_reals64, &c.link_reals32, &c.sweep_ms[0],
                    &c.sweep_ms[1], &c.check_ms[0], &c.check_ms[1], &c.wide_regs) == 11 &&
        (c.wide_regs == 0 || c.wide_regs == 1) && (c.link_reals32 == 12 || c.link_reals32 == 8) &&
        valid_block(c.block[0]) && valid_block(c.block[1]) &&
        (c.link_reals64 == 12 || c.link_reals64 == 18)) {
      *t = c;  // the last valid line for a key wins
      hit = true;
    }
  }
  std::fclose(f);
  return hit;
}

static void cache_append(const char* path, const std::string& key, const gfx_tuning& t) {
  FILE* f = std::fopen(path, "a");
  if (!f) return;  // the cache is an optimisation; an unwritable path only costs a re-tune
  std::fprintf(f, "%s\t%d %d %d %d %d %d %.6g %.6g %.6g %.6g %d\n", key.c_str(), t.block[0],
               t.staging[0], t.block[1], t.staging[1], t.link_reals64, t.link_reals32,
               t.sweep_ms[0], t.sweep_ms[1], t.check_ms[0], t.check_ms[1], t.wide_regs);
  std::fclose(f);
}

static int suggest_checkinterval(const gfx_ctx* ctx, int expected_sweeps) {
  const int p = ctx->G32 ? 0 : 1;
  if (expected_sweeps <= 0 || ctx->tune_sweep_ms[p] <= 0.0) return 0;
  // checks every k sweeps cost (n/k) c; stopping at the first check past
  // convergence wastes k/2 sweeps s on average: k* = sqrt(2 n c / s)
  const double k = std::sqrt(2.0 * expected_sweeps * ctx->tune_measure_ms[p] / ctx->tune_sweep_ms[p]);
  return std::min(100, std::max(5, (int)std::lround(k)));
}

gfx_status gfx_autotune(gfx_ctx* ctx, int gauge, int expected_sweeps, const char* cache_path,
                        gfx_tuning* out) {
  if (!ctx) return fail(nullptr, GFX_ERR_ARG, "NULL context");
  const int ndir = gauge == GFX_GAUGE_COULOMB ? 3 : 4;
  const std::string key = tune_key(ctx, ndir);
  gfx_tuning t;
  gfx_status s;
  if (cache_path && cache_lookup(cache_path, key, &t)) {
    s = gfx_set_tuning(ctx, &t);
    if (s) return s;
    for (int p = 0; p < 2; p++) {
      ctx->tune_sweep_ms[p] = t.sweep_ms[p];
      ctx->tune_measure_ms[p] = t.check_ms[p];
    }
    ctx->tune_ck = suggest_checkinterval(ctx, expected_sweeps);
    return out ? gfx_get_tuning(ctx, out) : GFX_OK;
  }
  // keep the current g: the candidate sweeps run on it (from G64 when it is held as
  // double-float or on a rebased base)
  if (ctx->g_active >= 2 && (s = sync_g64(ctx))) return s;
  const int active = ctx->g_active;
  void* gsrc = active ? ctx->G64 : ctx->G32;
  const size_t gbytes = active ? g_bytes64(ctx) : g_bytes32(ctx);
  void* saved = nullptr;
  if (cudaMalloc(&saved, gbytes) != cudaSuccess) {
    cudaGetLastError();
    return fail(ctx, GFX_ERR_OOM, "gfx_autotune: no room to keep g during tuning");
  }
  if (cudaMemcpyAsync(saved, gsrc, gbytes, cudaMemcpyDeviceToDevice, ctx->stream) != cudaSuccess) {
    cudaGetLastError();
    cudaFree(saved);
    return fail(ctx, GFX_ERR_CUDA, "gfx_autotune: copy of g failed");
  }
  const int blocks[4] = {64, 128, 192, 256};
  s = GFX_OK;
  for (int prec = 0; prec < 2 && s == GFX_OK; prec++) {
    if (prec == 0 && !ctx->G32) continue;
    if (prec == 1 && ctx->precision == GFX_PREC_SINGLE) continue;  // FP64 sweeps never run
    // link layouts: FP64 12/18 reals, FP32 12/8 reals
    int layouts[2] = {ctx->link_nr, ctx->link_nr == 12 ? 18 : 12};
    const int nlayouts = 2;
    if (prec == 0) {
      layouts[0] = 12;
      layouts[1] = 8;
    }
    double best = 1e30;
    int bb = ctx->or_block[prec], bp = ctx->or_pf[prec], bnr = layouts[0], bw = ctx->or_wide;
    int n = 0;
    for (int li = 0; li < nlayouts && s == GFX_OK; li++) {
      if (prec == 1 && (s = relayout_links(ctx, layouts[li]))) break;
      if (prec == 0 && (s = set_link_layout32(ctx, layouts[li]))) break;
      if ((s = prepare_g(ctx, prec))) break;
      if (n == 0) {
        double t1 = 0.0;
        s = time_reps(ctx, 2, [&]() { enqueue_sweep(ctx, prec, ndir, 1.7); }, &t1);
        if (s) break;
        n = std::min(40, std::max(2, (int)std::ceil(3.0 / std::max(t1, 1e-3))));
      }
      auto sweep = [&]() { enqueue_sweeps(ctx, prec, ndir, 1.7, n); };
      // modes 3 and 4 (L2 eviction priorities) exist for the FP32 12-real sweep only
      const int nmodes = prec == 0 && layouts[li] == 12 ? 5 : 3;
      // FP32 12-real sweeps: both register budgets of the kernel
      const int nwide = prec == 0 && layouts[li] == 12 ? 2 : 1;
      for (int round = 0; round < 2 && s == GFX_OK; round++)
        for (int w = 0; w < nwide && s == GFX_OK; w++)
          for (int bi = 0; bi < 4 && s == GFX_OK; bi++)
            for (int pf = 0; pf < nmodes && s == GFX_OK; pf++) {
              ctx->or_block[prec] = blocks[bi];
              ctx->or_pf[prec] = pf;
              if (prec == 0) ctx->or_wide = nwide == 2 ? w : 0;
              double ms = 0.0;
              s = time_reps(ctx, 2, sweep, &ms);
              ms /= n;
              if (s == GFX_OK && ms < best) {
                best = ms;
                bb = blocks[bi];
                bp = pf;
                bnr = layouts[li];
                if (prec == 0) bw = ctx->or_wide;
              }
            }
    }
    if (s) break;
    ctx->or_block[prec] = bb;
    ctx->or_pf[prec] = bp;
    if (prec == 0) ctx->or_wide = bw;
    if (prec == 1 && (s = relayout_links(ctx, bnr))) break;
    if (prec == 0 && (s = set_link_layout32(ctx, bnr))) break;
    ctx->tune_sweep_ms[prec] = best;
    if ((s = prepare_g(ctx, prec))) break;
    // the check's cost: a sweep with its check (fused when the loop fuses it) minus
    // a plain sweep
    const bool odd = odd_only_checks(ctx, prec);
    auto check = [&]() {
      enqueue_sweeps_measure(ctx, prec, ndir, 1.7, 1, odd);
      enqueue_reduce(ctx, ndir, false, 0, 0, 0, odd);
    };
    s = time_reps(ctx, std::max(2, n), check, &ctx->tune_measure_ms[prec]);
    ctx->tune_measure_ms[prec] = std::max(0.0, ctx->tune_measure_ms[prec] - best);
  }
  // put g back where it was
  cudaError_t e = cudaMemcpyAsync(gsrc, saved, gbytes, cudaMemcpyDeviceToDevice, ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  cudaFree(saved);
  ctx->g_active = active;
  destroy_graphs(ctx);
  if (s) return s;
  if (e != cudaSuccess) return fail(ctx, GFX_ERR_CUDA, std::string("gfx_autotune: ") + cudaGetErrorString(e));
  ctx->tune_ck = suggest_checkinterval(ctx, expected_sweeps);
  gfx_tuning res;
  gfx_get_tuning(ctx, &res);
  if (cache_path) cache_append(cache_path, key, res);
  if (out) *out = res;
  return GFX_OK;
}

}  // extern "C"
