// gfx_batch.cu -- many gauge copies of several configurations, fixed together.
//
// A batch holds nconf configurations (each with its own lattice extents and links) and
// ncopies[c] gauge transformations per configuration (Gribov copies).  Every half-sweep
// of every active copy of every configuration is one kernel launch: a work item is
// (configuration, block of 128 sites, copy), ordered copy-minor, so the copies of a site
// block run side by side and share its links through L2 -- each link read from HBM
// serves all copies of its configuration.  The
// checks, their per-copy reductions and the per-copy convergence bookkeeping run on
// the device; the whole loop is one CUDA graph with a conditional while node, as for a
// single lattice.  Per copy, the arithmetic and the reduction order are those of the
// single-lattice kernels (gfx_common.cuh), so a copy's trajectory, iteration count and
// final functional equal those of the same start fixed alone.
#include <algorithm>
#include <cmath>
#include <array>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/gfx.h"
#include "gfx_common.cuh"
#include "gfx_internal.h"
#include "gfx_rebased.cuh"

namespace gfx {

constexpr int kBatchBlock = 128;
constexpr int kMaxConf = 8;

struct BConf {
  Lattice L;
  const void* U32;   // FP32 12-real links
  void* U32P;        // the same links in both lanes of the pair layout (P12)
  const void* U64;   // FP64 12-real links
  void* G32;         // copy 0's g (FP32), copy k at + k * gstride32 vectors; while the
                     // FP32 sweeps run two copies per thread, pair k (copies 2k, 2k+1)
                     // in the P12 layout at + 2 k * gstride32
  void* G64;         // copy 0's g (FP64), copy k at + k * gstride64 vectors
  size_t gstride32, gstride64;
  void* Ur;          // rebased FP32 polish (polish = 2): copy k's rebased links at
  void* W0;          // + k * urstride vectors, its split star at + k * w0stride
  size_t urstride, w0stride;
  int ncopies;
  int copy_base;     // index of copy 0 among all copies of the batch
  int item_base;     // first sweep work item
  int nblk;          // site blocks per parity
  int mitem_base;    // first measurement item
  int nbx;           // measurement blocks per time slice
  size_t part_base;  // first partial triple of copy 0 (copy k: + k * 2 * lt * nbx)
  int slice_base;    // first slice triple of copy 0 (copy k: + k * lt)
  int sitem_base;    // first slice-reduce item
  int odd_only;      // FP32-phase checks measure the odd sites only, as a single
                     // mixed solve of this lattice does (gfx_internal.h)
  int npairs;        // copy pairs (copies 2k, 2k+1; the last one alone when ncopies is odd)
  int pitem_base;    // first paired-sweep work item
};

struct BDesc {
  BConf c[kMaxConf];
  int nconf;
  int ncopies;  // all configurations
  int paired;   // FP32 g of the sweeps in the pair layout (or_batch_pair_kernel)
  LoopState* states;
  double* partials;
  double* slice_sums;
  Reduced* reduced;
};

__device__ __forceinline__ int conf_of(const BDesc& d, int item, int BConf::*base) {
  int ci = 0;
  while (ci + 1 < d.nconf && item >= d.c[ci + 1].*base) ci++;
  return ci;
}

// One half-sweep of parity `parity` for all active copies (or_halfsweep_kernel per
// copy).  Work items run copy-minor: the ncopies blocks of one site block are adjacent
// in the grid, so they run at about the same time and the site block's links (8 per
// site) come from L2 for all but the first copy; each link crosses HBM about once per
// half-sweep whatever the number of copies.
template <typename T, int NDIR>
__global__ void __launch_bounds__(kBatchBlock, sizeof(T) == 4 ? 8 : 4) or_batch_kernel(BDesc d, int parity, T omega) {
  typedef typename VecOf<T>::type V;
  // parity 1 runs the work items in reverse order: it starts on the ranges parity 0
  // touched last, which L2 may still hold (the order does not change any result)
  const int item = parity ? (int)gridDim.x - 1 - (int)blockIdx.x : (int)blockIdx.x;
  const int ci = conf_of(d, item, &BConf::item_base);
  const BConf& C = d.c[ci];
  const int local = item - C.item_base;
  const int blk = local / C.ncopies, copy = local - blk * C.ncopies;
  if (d.states[C.copy_base + copy].done != 0) return;  // uniform over the block
  const int i = blk * kBatchBlock + threadIdx.x;
  if (i >= C.L.vh) return;
  const Site s = site_of(C.L, i, parity);
  const V* U = (const V*)(sizeof(T) == 4 ? C.U32 : C.U64);
  V* G = (V*)(sizeof(T) == 4 ? C.G32 : C.G64) +
         (size_t)copy * (sizeof(T) == 4 ? C.gstride32 : C.gstride64);
  or_site_update<T, 12, NDIR>(C.L, s, parity, U, G, i, omega);
}

// The last odd half-sweep before an FP32 check (or_batch_kernel<float> with parity 1),
// writing the check's partials of the configurations whose FP32-phase checks read the
// odd sites only (BConf::odd_only), as or_halfsweep_measure_kernel does for one
// lattice: the odd sites' star depends on the even sites only, so the partials are
// those measure_batch_kernel would form after the sweep, bit for bit.  With odd_only
// the slice holds whole 128-site blocks, so every block is full and lies in one slice.
template <int NDIR>
__global__ void __launch_bounds__(kBatchBlock, 6) or_batch_measure_kernel(BDesc d, float omega) {
  const int parity = 1;
  const int item = (int)gridDim.x - 1 - (int)blockIdx.x;  // parity 1's order
  const int ci = conf_of(d, item, &BConf::item_base);
  const BConf& C = d.c[ci];
  const int local = item - C.item_base;
  const int blk = local / C.ncopies, copy = local - blk * C.ncopies;
  if (d.states[C.copy_base + copy].done != 0) return;  // uniform over the block
  const int i = blk * kBatchBlock + threadIdx.x;
  const float4* U = (const float4*)C.U32;
  float4* G = (float4*)C.G32 + (size_t)copy * C.gstride32;
  if (!C.odd_only) {  // uniform over the block: the sweep alone
    if (i >= C.L.vh) return;
    or_site_update<float, 12, NDIR>(C.L, site_of(C.L, i, parity), parity, U, G, i, omega);
    return;
  }
  const size_t vh = (size_t)C.L.vh;
  const Site s = site_of(C.L, i, parity);
  float4* Gp = G + (size_t)parity * 3 * vh;
  Mat3<float> star, gold, gn;
  compute_star_f32<NDIR>(C.L, s, parity, U, G, star);
  Field<float, 12>::load(Gp, vh, i, gold);
  or_update_composed(gold, star, omega, gn);
  Field<float, 12>::store(Gp, vh, i, gn);
  row2_from_01(gn);  // as the measurement's load of the stored rows
  float f, dd;
  site_functional_f32(gn, star, f, dd);
  const int t = blk / C.nbx, bx = blk - t * C.nbx;
  const int per_copy = 2 * C.L.lt * C.nbx;
  block_reduce3_f32(f, dd,
                    d.partials + 3 * (C.part_base + (size_t)copy * per_copy +
                                      (size_t)(parity * C.L.lt + t) * C.nbx + bx));
}

// The FP32 half-sweep with two copies per thread (or_site_update_pair: packed FP32
// arithmetic, lane for lane the operations of or_batch_kernel<float>).  Work items are
// (configuration, site block, copy pair), pair-minor, so the pairs of a site block run
// side by side as in or_batch_kernel.  The pair's g and the links (held in both lanes)
// are in the P12 layout, so every operand of the packed instructions comes straight
// from a 16-byte load.  The second lane of a configuration's last pair when its copy
// count is odd holds a duplicate of the first and is never written.
template <int NDIR>
__global__ void __launch_bounds__(kBatchBlock, 4) or_batch_pair_kernel(BDesc d, int parity,
                                                                       float omega) {
  const int item = parity ? (int)gridDim.x - 1 - (int)blockIdx.x : (int)blockIdx.x;
  const int ci = conf_of(d, item, &BConf::pitem_base);
  const BConf& C = d.c[ci];
  const int local = item - C.pitem_base;
  const int blk = local / C.npairs, pair = local - blk * C.npairs;
  const int c0 = 2 * pair, c1 = c0 + 1;
  const bool run0 = d.states[C.copy_base + c0].done == 0;
  const bool run1 = c1 < C.ncopies && d.states[C.copy_base + c1].done == 0;
  if (!run0 && !run1) return;  // uniform over the block
  const int i = blk * kBatchBlock + threadIdx.x;
  if (i >= C.L.vh) return;
  P12 U, G;
  U.p = (float4*)C.U32P;
  G.p = (float4*)C.G32 + (size_t)c0 * C.gstride32;
  or_site_update_pair<NDIR>(C.L, site_of(C.L, i, parity), parity, U, G, i, omega, run0, run1);
}

// the FP32 links of configuration conf in both lanes of the pair layout
__global__ void links_pair_kernel(BDesc d, int conf) {
  const BConf& C = d.c[conf];
  const int blk = blockIdx.y;  // parity * 4 + mu
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= C.L.vh) return;
  const size_t vh = (size_t)C.L.vh;
  Mat3<float> f;
  Field<float, 12>::load((const float4*)C.U32 + (size_t)blk * 3 * vh, vh, i, f);
  float4* o = (float4*)C.U32P + (size_t)blk * kPairPlanes * vh;
#pragma unroll
  for (int e = 0; e < 6; e++) {
    const cplx<float> z = f.e[e / 3][e % 3];
    o[e * vh + i] = make_float4(z.re, z.re, z.im, z.im);
  }
}

// The rebased FP32 polish sweep for all active copies (or_rebased_kernel per copy, the
// same work-item order as or_batch_kernel); a copy's a lives in its G32 slot
template <int NDIR>
__global__ void __launch_bounds__(kBatchBlock, 4) or_batch_rebased_kernel(BDesc d, int parity,
                                                                          float omega) {
  const int item = parity ? (int)gridDim.x - 1 - (int)blockIdx.x : (int)blockIdx.x;
  const int ci = conf_of(d, item, &BConf::item_base);
  const BConf& C = d.c[ci];
  const int local = item - C.item_base;
  const int blk = local / C.ncopies, copy = local - blk * C.ncopies;
  if (d.states[C.copy_base + copy].done != 0) return;  // uniform over the block
  const int i = blk * kBatchBlock + threadIdx.x;
  if (i >= C.L.vh) return;
  rebased_site_update<NDIR>(C.L, site_of(C.L, i, parity), parity,
                            (const float4*)C.Ur + (size_t)copy * C.urstride,
                            (const float4*)C.W0 + (size_t)copy * C.w0stride,
                            (float4*)C.G32 + (size_t)copy * C.gstride32, omega);
}

// Per-copy functional partials (measure_kernel per copy, same block grouping)
// fused: the FP32 partials of odd_only configurations came from or_batch_measure_kernel
template <typename TC, typename TSG, int NDIR>
__global__ void __launch_bounds__(kBatchBlock) measure_batch_kernel(BDesc d, int fused) {
  const int ci = conf_of(d, blockIdx.x, &BConf::mitem_base);
  const BConf& C = d.c[ci];
  int local = blockIdx.x - C.mitem_base;
  const int per_copy = 2 * C.L.lt * C.nbx;
  const int copy = local / per_copy;
  local -= copy * per_copy;
  const int parity = local / (C.L.lt * C.nbx);
  local -= parity * C.L.lt * C.nbx;
  const int t = local / C.nbx, bx = local - t * C.nbx;
  if (d.states[C.copy_base + copy].done != 0) return;  // uniform over the block
  constexpr bool F32 = sizeof(TC) == 4 && sizeof(TSG) == 4;
  // the FP32-phase checks: odd sites only, and those already written by a fused sweep
  if (F32 && C.odd_only && (parity == 0 || fused)) return;
  typedef typename VecOf<TC>::type VU;
  typedef typename VecOf<TSG>::type VG;
  const VU* U = (const VU*)(sizeof(TC) == 4 ? C.U32 : C.U64);
  const VG* G = (const VG*)(sizeof(TSG) == 4 ? C.G32 : C.G64) +
                (size_t)copy * (sizeof(TSG) == 4 ? C.gstride32 : C.gstride64);
  const int k = bx * blockDim.x + threadIdx.x;
  double f = 0.0, dd = 0.0;
  float f32 = 0.0f, d32 = 0.0f;
  if (k < C.L.st) {
    const int i = t * C.L.st + k;
    const Site c = site_of(C.L, i, parity);
    const size_t vh = (size_t)C.L.vh;
    Mat3<TC> star, g;
    if constexpr (F32) {
      if (d.paired) {
        // this copy's lane of its pair (P12 layout)
        LaneP12 Gl;
        Gl.p = (const float4*)C.G32 + (size_t)(copy & ~1) * C.gstride32;
        Gl.lane = copy & 1;
        Mat3<float> s, h;
        compute_star_12<float, const float4*, LaneP12, NDIR>(C.L, c, parity, (const float4*)U,
                                                               Gl, s);
        g_full(Gl + (size_t)parity * kPairPlanes * vh, vh, i, h);
        site_functional_f32(h, s, f32, d32);
      } else {
        compute_star_f32<NDIR>(C.L, c, parity, (const float4*)U, (const float4*)G, star);
        Load<TC, TSG, 12>::go(G + (size_t)parity * 3 * vh, vh, i, g);
        site_functional_f32(g, star, f32, d32);
      }
    } else {
      compute_star<TC, TC, 12, TSG, 12, NDIR>(C.L, c, parity, U, G, star);
      constexpr int NCG = Field<TSG, 12>::NCHUNK;
      Load<TC, TSG, 12>::go(G + (size_t)parity * NCG * vh, vh, i, g);
      site_functional(g, star, f, dd);
    }
  }
  double* out = d.partials +
                3 * (C.part_base + (size_t)copy * per_copy + (size_t)(parity * C.L.lt + t) * C.nbx + bx);
  if constexpr (F32) block_reduce3_f32(f32, d32, out);
  else block_reduce3(f, dd, dd, out);
}

// the same partials from the rebased fields (measure_rebased_kernel per copy)
template <int NDIR>
__global__ void __launch_bounds__(kBatchBlock) measure_batch_rebased_kernel(BDesc d) {
  const int ci = conf_of(d, blockIdx.x, &BConf::mitem_base);
  const BConf& C = d.c[ci];
  int local = blockIdx.x - C.mitem_base;
  const int per_copy = 2 * C.L.lt * C.nbx;
  const int copy = local / per_copy;
  local -= copy * per_copy;
  const int parity = local / (C.L.lt * C.nbx);
  local -= parity * C.L.lt * C.nbx;
  const int t = local / C.nbx, bx = local - t * C.nbx;
  if (d.states[C.copy_base + copy].done != 0) return;  // uniform over the block
  const int k = bx * blockDim.x + threadIdx.x;
  double f = 0.0, dd = 0.0;
  if (k < C.L.st)
    rebased_site_functional<NDIR>(C.L, site_of(C.L, t * C.L.st + k, parity), parity,
                                  (const float4*)C.Ur + (size_t)copy * C.urstride,
                                  (const float4*)C.W0 + (size_t)copy * C.w0stride,
                                  (const float4*)C.G32 + (size_t)copy * C.gstride32, f, dd);
  double* out = d.partials +
                3 * (C.part_base + (size_t)copy * per_copy + (size_t)(parity * C.L.lt + t) * C.nbx + bx);
  block_reduce3(f, dd, dd, out);
}

// per (copy, slice) sums, as slice_reduce_kernel (f32check: an FP32 check, odd sites
// only where the configuration's single solve does so)
__global__ void slice_batch_kernel(BDesc d, int f32check) {
  const int ci = conf_of(d, blockIdx.x, &BConf::sitem_base);
  const BConf& C = d.c[ci];
  const int local = blockIdx.x - C.sitem_base;
  const int copy = local / C.L.lt, t = local - copy * C.L.lt;
  if (d.states[C.copy_base + copy].done != 0) return;
  const double* partials = d.partials + 3 * (C.part_base + (size_t)copy * 2 * C.L.lt * C.nbx);
  const bool odd_only = f32check && C.odd_only;
  double f = 0.0, dd = 0.0, m = 0.0;
  for (int j = (odd_only ? C.nbx : 0) + threadIdx.x; j < 2 * C.nbx; j += blockDim.x) {
    const int p = j / C.nbx, bx = j % C.nbx;
    const double* q = partials + 3 * ((size_t)(p * C.L.lt + t) * C.nbx + bx);
    f += q[0];
    dd += q[1];
    m = fmax(m, q[2]);
  }
  if (odd_only) {
    f *= 2.0;
    dd *= 2.0;
  }
  block_reduce3(f, dd, m, d.slice_sums + 3 * (C.slice_base + (size_t)copy * C.L.lt + t));
}

// per-copy totals and convergence bookkeeping, as final_reduce_kernel
__global__ void check_batch_kernel(BDesc d, int ndir, int advance) {
  int ci = 0;
  while (ci + 1 < d.nconf && (int)blockIdx.x >= d.c[ci + 1].copy_base) ci++;
  const BConf& C = d.c[ci];
  const int copy = blockIdx.x - C.copy_base;
  LoopState* S = d.states + blockIdx.x;
  if (S->done != 0) return;
  const double vol = 2.0 * (double)C.L.vh;
  const double v3 = (double)C.L.lx * C.L.ly * C.L.lz;
  reduce_and_check(d.slice_sums + 3 * (C.slice_base + (size_t)copy * C.L.lt), C.L.lt, vol, v3,
                   ndir, d.reduced + blockIdx.x, S, nullptr, advance);
}

// continue the device loop while any copy is still running
__global__ void continue_batch_kernel(BDesc d, int* running, cudaGraphConditionalHandle handle,
                                      int use_handle) {
  int n = 0;
  for (int k = threadIdx.x; k < d.ncopies; k += blockDim.x) n += d.states[k].done == 0;
  __shared__ int sh[32];
  for (int o = 16; o > 0; o >>= 1) n += __shfl_xor_sync(0xffffffffu, n, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = n;
  __syncthreads();
  if (threadIdx.x == 0) {
    int tot = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) tot += sh[w];
    *running = tot;
    if (use_handle) cudaGraphSetConditional(handle, tot > 0 ? 1u : 0u);
  }
}

// FP64 <-> FP32 copies of every copy's g (g_32_to_64_kernel / g_64_to_32_kernel per copy)
__global__ void convert_batch_kernel(BDesc d, int to64, int only_state) {
  const int ci = conf_of(d, blockIdx.y, &BConf::copy_base);
  const BConf& C = d.c[ci];
  const int copy = blockIdx.y - C.copy_base;
  if (only_state >= 0 && d.states[blockIdx.y].done != only_state) return;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= C.L.vh) return;
  const size_t vh = (size_t)C.L.vh;
  for (int parity = 0; parity < 2; parity++) {
    const float4* g32 = (const float4*)C.G32 + (size_t)copy * C.gstride32 + (size_t)parity * 3 * vh;
    // the pair layout: this copy's lane of pair copy / 2
    float* g32p = (float*)((float4*)C.G32 + (size_t)(copy & ~1) * C.gstride32 +
                           (size_t)parity * kPairPlanes * vh);
    const int lane = copy & 1;
    const double2* g64 = (const double2*)C.G64 + (size_t)copy * C.gstride64 + (size_t)parity * 6 * vh;
    if (to64) {
      Mat3<double> m;
      if (d.paired) {
        LaneP12 Gl;
        Gl.p = (const float4*)g32p;
        Gl.lane = lane;
        Mat3<float> f;
        load12_rows01(Gl, vh, i, f);
#pragma unroll
        for (int r = 0; r < 2; r++)
#pragma unroll
          for (int c = 0; c < 3; c++) m.e[r][c] = cmk<double>(f.e[r][c].re, f.e[r][c].im);
        normalize<double, true>(m);  // as Load<double, float, 12>
      } else {
        Load<double, float, 12>::go(g32, vh, i, m);
      }
      Field<double, 12>::store((double2*)g64, vh, i, m);
    } else {
      Mat3<double> m;
      Field<double, 12>::load(g64, vh, i, m);
      Mat3<float> f;
#pragma unroll
      for (int r = 0; r < 3; r++)
#pragma unroll
        for (int c = 0; c < 3; c++) f.e[r][c] = cmk<float>((float)m.e[r][c].re, (float)m.e[r][c].im);
      if (d.paired) {
        // the last copy of an odd count also fills the unused second lane
        const bool both = lane == 0 && copy + 1 == C.ncopies;
#pragma unroll
        for (int e = 0; e < 6; e++) {
          float* q = g32p + 4 * (e * vh + i);
          q[lane] = f.e[e / 3][e % 3].re;
          q[2 + lane] = f.e[e / 3][e % 3].im;
          if (both) {
            q[1] = f.e[e / 3][e % 3].re;
            q[3] = f.e[e / 3][e % 3].im;
          }
        }
      } else {
        Field<float, 12>::store((float4*)g32, vh, i, f);
      }
    }
  }
}

}  // namespace gfx

using namespace gfx;

struct gfx_batch {
  int nconf;
  int ncopies;
  int precision;
  cudaStream_t stream;
  bool own_stream;
  std::vector<std::array<int, 4>> dims;
  std::vector<int> copies;
  BDesc desc;
  int nitems, nmitems, nsitems, npitems;
  int paired;  // FP32 sweeps with two copies per thread (default 1)
  std::vector<void*> allocs;
  int* running;       // device
  LoopState* h_states;  // pinned
  std::vector<double> ms;
  struct G {
    int prec, ndir, ck;
    double omega;
    cudaGraph_t graph;
    cudaGraphExec_t exec;
  };
  std::vector<G> graphs;
  void* ulo;  // scratch of the rebase: FP32 remainders of the largest configuration's links
  std::string err;
};

namespace {
std::string g_batch_err;

gfx_status bfail(gfx_batch* b, gfx_status s, const std::string& m) {
  if (b) b->err = m;
  g_batch_err = m;
  return s;
}

#define BCK(call)                                                                          \
  do {                                                                                     \
    cudaError_t e_ = (call);                                                               \
    if (e_ != cudaSuccess)                                                                 \
      return bfail(b, GFX_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

gfx_status balloc(gfx_batch* b, void** p, size_t bytes) {
  cudaError_t e = cudaMalloc(p, bytes);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return bfail(b, e == cudaErrorMemoryAllocation ? GFX_ERR_OOM : GFX_ERR_CUDA,
                 std::string("cudaMalloc: ") + cudaGetErrorString(e));
  }
  b->allocs.push_back(*p);
  return GFX_OK;
}

// last: the sweep before a check; FP32 one copy per thread then writes the check's odd
// partials in its odd half-sweep (or_batch_measure_kernel)
void enqueue_sweep(gfx_batch* b, int prec, int ndir, double omega, bool last = false) {
  const size_t sm = 0;
  for (int p = 0; p < 2; p++) {
    if (prec == 0 && !b->paired && last && p == 1) {
      if (ndir == 4)
        or_batch_measure_kernel<4><<<b->nitems, kBatchBlock, sm, b->stream>>>(b->desc, (float)omega);
      else
        or_batch_measure_kernel<3><<<b->nitems, kBatchBlock, sm, b->stream>>>(b->desc, (float)omega);
    } else if (prec == 3) {  // rebased FP32
      if (ndir == 4)
        or_batch_rebased_kernel<4><<<b->nitems, kBatchBlock, sm, b->stream>>>(b->desc, p, (float)omega);
      else
        or_batch_rebased_kernel<3><<<b->nitems, kBatchBlock, sm, b->stream>>>(b->desc, p, (float)omega);
    } else if (prec == 0 && b->paired) {
      if (ndir == 4)
        or_batch_pair_kernel<4><<<b->npitems, kBatchBlock, sm, b->stream>>>(b->desc, p, (float)omega);
      else
        or_batch_pair_kernel<3><<<b->npitems, kBatchBlock, sm, b->stream>>>(b->desc, p, (float)omega);
    } else if (prec == 0) {
      if (ndir == 4)
        or_batch_kernel<float, 4><<<b->nitems, kBatchBlock, sm, b->stream>>>(b->desc, p, (float)omega);
      else
        or_batch_kernel<float, 3><<<b->nitems, kBatchBlock, sm, b->stream>>>(b->desc, p, (float)omega);
    } else {
      if (ndir == 4)
        or_batch_kernel<double, 4><<<b->nitems, kBatchBlock, sm, b->stream>>>(b->desc, p, omega);
      else
        or_batch_kernel<double, 3><<<b->nitems, kBatchBlock, sm, b->stream>>>(b->desc, p, omega);
    }
  }
}

void enqueue_check(gfx_batch* b, int cprec, int gprec, int ndir, int advance,
                   unsigned long long handle, int use_handle) {
  if (cprec == 3) {
    if (ndir == 4) measure_batch_rebased_kernel<4><<<b->nmitems, kBatchBlock, 0, b->stream>>>(b->desc);
    else measure_batch_rebased_kernel<3><<<b->nmitems, kBatchBlock, 0, b->stream>>>(b->desc);
  } else if (cprec == 0) {
    const int fused = b->paired ? 0 : 1;
    bool all_fused = fused != 0;
    for (int c = 0; c < b->nconf; c++) all_fused &= b->desc.c[c].odd_only != 0;
    if (!all_fused) {
      if (ndir == 4)
        measure_batch_kernel<float, float, 4><<<b->nmitems, kBatchBlock, 0, b->stream>>>(b->desc, fused);
      else
        measure_batch_kernel<float, float, 3><<<b->nmitems, kBatchBlock, 0, b->stream>>>(b->desc, fused);
    }
  } else if (gprec == 0) {
    if (ndir == 4) measure_batch_kernel<double, float, 4><<<b->nmitems, kBatchBlock, 0, b->stream>>>(b->desc, 0);
    else measure_batch_kernel<double, float, 3><<<b->nmitems, kBatchBlock, 0, b->stream>>>(b->desc, 0);
  } else {
    if (ndir == 4) measure_batch_kernel<double, double, 4><<<b->nmitems, kBatchBlock, 0, b->stream>>>(b->desc, 0);
    else measure_batch_kernel<double, double, 3><<<b->nmitems, kBatchBlock, 0, b->stream>>>(b->desc, 0);
  }
  slice_batch_kernel<<<b->nsitems, 256, 0, b->stream>>>(b->desc, cprec == 0 && gprec == 0);
  check_batch_kernel<<<b->ncopies, 256, 0, b->stream>>>(b->desc, ndir, advance);
  continue_batch_kernel<<<1, 256, 0, b->stream>>>(b->desc, b->running,
                                                 (cudaGraphConditionalHandle)handle, use_handle);
}

gfx_status read_states(gfx_batch* b) {
  BCK(cudaMemcpyAsync(b->h_states, b->desc.states, sizeof(LoopState) * b->ncopies,
                      cudaMemcpyDeviceToHost, b->stream));
  BCK(cudaStreamSynchronize(b->stream));
  return GFX_OK;
}
gfx_status write_states(gfx_batch* b) {
  BCK(cudaMemcpyAsync(b->desc.states, b->h_states, sizeof(LoopState) * b->ncopies,
                      cudaMemcpyHostToDevice, b->stream));
  return GFX_OK;
}

gfx_status get_graph(gfx_batch* b, int prec, int ndir, int ck, double omega,
                     cudaGraphExec_t* out) {
  for (auto& g : b->graphs)
    if (g.prec == prec && g.ndir == ndir && g.ck == ck && g.omega == omega) {
      *out = g.exec;
      return GFX_OK;
    }
  cudaGraph_t graph;
  BCK(cudaGraphCreate(&graph, 0));
  cudaGraphConditionalHandle handle;
  BCK(cudaGraphConditionalHandleCreate(&handle, graph, 1, cudaGraphCondAssignDefault));
  cudaGraphNodeParams cp = {cudaGraphNodeTypeConditional};
  cp.conditional.handle = handle;
  cp.conditional.type = cudaGraphCondTypeWhile;
  cp.conditional.size = 1;
  cudaGraphNode_t node;
  BCK(cudaGraphAddNode(&node, graph, nullptr, nullptr, 0, &cp));
  cudaGraph_t body = cp.conditional.phGraph_out[0];
  BCK(cudaStreamBeginCaptureToGraph(b->stream, body, nullptr, nullptr, 0,
                                    cudaStreamCaptureModeThreadLocal));
  for (int k = 0; k < ck; k++) enqueue_sweep(b, prec, ndir, omega, k == ck - 1);
  enqueue_check(b, prec, prec, ndir, ck, (unsigned long long)handle, 1);
  cudaGraph_t cap;
  cudaError_t e = cudaStreamEndCapture(b->stream, &cap);
  if (e != cudaSuccess) {
    cudaGraphDestroy(graph);
    return bfail(b, GFX_ERR_CUDA, std::string("stream capture: ") + cudaGetErrorString(e));
  }
  cudaGraphExec_t ex;
  BCK(cudaGraphInstantiate(&ex, graph, 0));
  b->graphs.push_back({prec, ndir, ck, omega, graph, ex});
  *out = ex;
  return GFX_OK;
}

// run the device loop of one phase until no copy is running
gfx_status run_phase(gfx_batch* b, int prec, int ndir, int ck, double omega, int use_graph) {
  if (use_graph) {
    cudaGraphExec_t ex;
    gfx_status s = get_graph(b, prec, ndir, ck, omega, &ex);
    if (s) return s;
    BCK(cudaGraphLaunch(ex, b->stream));
    return read_states(b);
  }
  int running = 1;
  while (running > 0) {
    for (int k = 0; k < ck; k++) enqueue_sweep(b, prec, ndir, omega, k == ck - 1);
    enqueue_check(b, prec, prec, ndir, ck, 0, 0);
    BCK(cudaGetLastError());
    BCK(cudaMemcpyAsync(&running, b->running, sizeof(int), cudaMemcpyDeviceToHost, b->stream));
    BCK(cudaStreamSynchronize(b->stream));
  }
  return read_states(b);
}

// the rebased polish's fields, allocated on first use
gfx_status ensure_rebased(gfx_batch* b) {
  size_t ulo = 0;
  for (int c = 0; c < b->nconf; c++) {
    BConf& C = b->desc.c[c];
    C.urstride = (size_t)8 * 3 * C.L.vh;
    C.w0stride = rebased_w0_bytes(C.L) / 16;
    ulo = std::max(ulo, C.urstride * 16);
    gfx_status s;
    void* p;
    if (!C.Ur) {
      if ((s = balloc(b, &p, (size_t)C.ncopies * C.urstride * 16))) return s;
      C.Ur = p;
    }
    if (!C.W0) {
      if ((s = balloc(b, &p, (size_t)C.ncopies * C.w0stride * 16))) return s;
      C.W0 = p;
    }
  }
  if (!b->ulo) return balloc(b, &b->ulo, ulo);
  return GFX_OK;
}

// copy k of configuration c: a new base from its FP64 g (a = 0), or g = (1 + a) g_c
gfx_status rebase_copy(gfx_batch* b, int c, int k, int ndir) {
  const BConf& C = b->desc.c[c];
  launch_rebase(12, ndir, C.L, C.U64, (const double2*)C.G64 + (size_t)k * C.gstride64,
                (float4*)C.Ur + (size_t)k * C.urstride, b->ulo,
                (float4*)C.W0 + (size_t)k * C.w0stride, b->stream);
  BCK(cudaGetLastError());
  BCK(cudaMemsetAsync((float4*)C.G32 + (size_t)k * C.gstride32, 0, C.gstride32 * 16, b->stream));
  return GFX_OK;
}
void compose_copy(gfx_batch* b, int c, int k) {
  const BConf& C = b->desc.c[c];
  launch_compose_g(C.L, (double2*)C.G64 + (size_t)k * C.gstride64,
                   (const float4*)C.G32 + (size_t)k * C.gstride32, b->stream);
}
// copy index -> configuration
int conf_of_copy(const gfx_batch* b, int g) {
  int c = 0;
  while (c + 1 < b->nconf && g >= b->desc.c[c + 1].copy_base) c++;
  return c;
}
constexpr int kBatchRebaseSweeps = 1000;  // as the single-lattice polish
}  // namespace

extern "C" {

const char* gfx_batch_last_error(const gfx_batch* b) { return b ? b->err.c_str() : g_batch_err.c_str(); }

gfx_status gfx_batch_destroy(gfx_batch* b) {
  if (!b) return GFX_OK;
  cudaStreamSynchronize(b->stream);
  for (auto& g : b->graphs) {
    cudaGraphExecDestroy(g.exec);
    cudaGraphDestroy(g.graph);
  }
  for (void* p : b->allocs) cudaFree(p);
  if (b->h_states) cudaFreeHost(b->h_states);
  if (b->own_stream) cudaStreamDestroy(b->stream);
  delete b;
  return GFX_OK;
}

gfx_status gfx_batch_create(gfx_batch** out, int nconf, const int* dims, const int* ncopies,
                            int precision, void* stream) {
  gfx_batch* b = nullptr;
  if (!out || !dims || !ncopies) return bfail(nullptr, GFX_ERR_ARG, "gfx_batch_create: NULL argument");
  *out = nullptr;
  if (nconf < 1 || nconf > kMaxConf)
    return bfail(nullptr, GFX_ERR_ARG, "gfx_batch_create: 1..8 configurations");
  if (precision < GFX_PREC_DOUBLE || precision > GFX_PREC_MIXED)
    return bfail(nullptr, GFX_ERR_ARG, "gfx_batch_create: unknown precision");
  for (int c = 0; c < nconf; c++) {
    const int* d = dims + 4 * c;
    if (d[0] < 2 || d[1] < 2 || d[2] < 2 || d[3] < 2 || (d[0] | d[1] | d[2] | d[3]) & 1)
      return bfail(nullptr, GFX_ERR_BAD_VOLUME, "gfx_batch_create: extents must be even");
    if ((long long)d[0] * d[1] * d[2] * d[3] / 2 > (1ll << 30) || ncopies[c] < 1)
      return bfail(nullptr, GFX_ERR_ARG, "gfx_batch_create: volume or copy count");
  }
  b = new gfx_batch();
  b->nconf = nconf;
  b->precision = precision;
  b->running = nullptr;
  b->h_states = nullptr;
  b->ulo = nullptr;
  std::memset((void*)&b->desc, 0, sizeof(b->desc));
  if (stream) {
    b->stream = (cudaStream_t)stream;
    b->own_stream = false;
  } else {
    if (cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess) {
      delete b;
      return bfail(nullptr, GFX_ERR_CUDA, "cudaStreamCreate failed");
    }
    b->own_stream = true;
  }
  gfx_status s;
#define BTRY(x)          \
  do {                   \
    s = (x);             \
    if (s) {             \
      std::string m = b->err; \
      gfx_batch_destroy(b); \
      g_batch_err = m;   \
      return s;          \
    }                    \
  } while (0)
  int copy_base = 0, item = 0, mitem = 0, sitem = 0, slice = 0, pitem = 0;
  size_t part = 0;
  for (int c = 0; c < nconf; c++) {
    const int* d = dims + 4 * c;
    BConf& C = b->desc.c[c];
    C.L = make_lattice(d[0], d[1], d[2], d[3]);
    b->dims.push_back({d[0], d[1], d[2], d[3]});
    b->copies.push_back(ncopies[c]);
    C.ncopies = ncopies[c];
    C.copy_base = copy_base;
    C.nblk = (C.L.vh + kBatchBlock - 1) / kBatchBlock;
    C.item_base = item;
    C.npairs = (C.ncopies + 1) / 2;
    C.odd_only = 0;  // set per solve (gfx_batch_overrelax)
    C.pitem_base = pitem;
    C.nbx = (C.L.st + kBatchBlock - 1) / kBatchBlock;
    C.mitem_base = mitem;
    C.sitem_base = sitem;
    C.part_base = part;
    C.slice_base = slice;
    C.gstride32 = (size_t)2 * 3 * C.L.vh;
    C.gstride64 = (size_t)2 * 6 * C.L.vh;
    const size_t vh = C.L.vh;
    void* p;
    BTRY(balloc(b, &p, (size_t)8 * 6 * 16 * vh));
    C.U64 = p;
    BTRY(balloc(b, &p, (size_t)C.ncopies * C.gstride64 * 16));
    C.G64 = p;
    if (precision != GFX_PREC_DOUBLE) {
      BTRY(balloc(b, &p, (size_t)8 * 3 * 16 * vh));
      C.U32 = p;
      BTRY(balloc(b, &p, (size_t)8 * kPairPlanes * 16 * vh));
      C.U32P = p;
      // whole pairs: the pair layout of the FP32 sweeps fills 2 * npairs copy slots
      BTRY(balloc(b, &p, (size_t)2 * C.npairs * C.gstride32 * 16));
      C.G32 = p;
    }
    copy_base += C.ncopies;
    item += C.nblk * C.ncopies;
    pitem += C.nblk * C.npairs;
    mitem += C.ncopies * 2 * C.L.lt * C.nbx;
    sitem += C.ncopies * C.L.lt;
    slice += C.ncopies * C.L.lt;
    part += (size_t)C.ncopies * 2 * C.L.lt * C.nbx;
  }
  b->ncopies = copy_base;
  b->nitems = item;
  b->npitems = pitem;
  b->paired = 0;
  b->desc.paired = 0;
  b->nmitems = mitem;
  b->nsitems = sitem;
  b->desc.nconf = nconf;
  b->desc.ncopies = copy_base;
  void* p;
  BTRY(balloc(b, &p, sizeof(LoopState) * copy_base));
  b->desc.states = (LoopState*)p;
  BTRY(balloc(b, &p, sizeof(double) * 3 * part));
  b->desc.partials = (double*)p;
  BTRY(balloc(b, &p, sizeof(double) * 3 * slice));
  b->desc.slice_sums = (double*)p;
  BTRY(balloc(b, &p, sizeof(Reduced) * copy_base));
  b->desc.reduced = (Reduced*)p;
  BTRY(balloc(b, &p, sizeof(int)));
  b->running = (int*)p;
  if (cudaMallocHost((void**)&b->h_states, sizeof(LoopState) * copy_base) != cudaSuccess) {
    gfx_batch_destroy(b);
    return bfail(nullptr, GFX_ERR_OOM, "cudaMallocHost failed");
  }
  std::memset(b->h_states, 0, sizeof(LoopState) * copy_base);
#undef BTRY
  *out = b;
  return GFX_OK;
}

int gfx_batch_copies(const gfx_batch* b) { return b ? b->ncopies : 0; }

gfx_status gfx_batch_set_paired(gfx_batch* b, int paired) {
  if (!b) return bfail(nullptr, GFX_ERR_ARG, "NULL batch");
  paired = paired && b->precision != GFX_PREC_DOUBLE ? 1 : 0;
  if (paired == b->paired) return GFX_OK;
  BCK(cudaStreamSynchronize(b->stream));
  for (auto& g : b->graphs) {  // captured with the other sweep kernel
    cudaGraphExecDestroy(g.exec);
    cudaGraphDestroy(g.graph);
  }
  b->graphs.clear();
  b->paired = paired;
  b->desc.paired = paired;  // the FP32 g layout: each solve converts into it at its start
  return GFX_OK;
}

static gfx_status copy_index(gfx_batch* b, int conf, int copy) {
  if (!b || conf < 0 || conf >= b->nconf || copy < 0 || copy >= b->copies[conf])
    return bfail(b, GFX_ERR_ARG, "configuration or copy index out of range");
  return GFX_OK;
}

gfx_status gfx_batch_set_links(gfx_batch* b, int conf, const double* su3) {
  if (!b || !su3 || conf < 0 || conf >= b->nconf) return bfail(b, GFX_ERR_ARG, "bad argument");
  BConf& C = b->desc.c[conf];
  const size_t bytes = sizeof(double) * 18 * 4 * 2 * (size_t)C.L.vh;
  double* scratch;
  BCK(cudaMallocAsync((void**)&scratch, bytes, b->stream));
  BCK(cudaMemcpyAsync(scratch, su3, bytes, cudaMemcpyHostToDevice, b->stream));
  launch_pack_links(12, C.L, scratch, (void*)C.U64, b->stream);
  if (C.U32) {
    launch_convert_links_64_to_32(12, 12, C.L, C.U64, (void*)C.U32, b->stream);
    links_pair_kernel<<<dim3((C.L.vh + 127) / 128, 8), 128, 0, b->stream>>>(b->desc, conf);
  }
  BCK(cudaFreeAsync(scratch, b->stream));
  BCK(cudaGetLastError());
  BCK(cudaStreamSynchronize(b->stream));
  return GFX_OK;
}

gfx_status gfx_batch_set_trafo(gfx_batch* b, int conf, int copy, const double* su3) {
  gfx_status s = copy_index(b, conf, copy);
  if (s) return s;
  if (!su3) return bfail(b, GFX_ERR_ARG, "NULL trafo");
  BConf& C = b->desc.c[conf];
  const size_t bytes = sizeof(double) * 18 * 2 * (size_t)C.L.vh;
  double* scratch;
  BCK(cudaMallocAsync((void**)&scratch, bytes, b->stream));
  BCK(cudaMemcpyAsync(scratch, su3, bytes, cudaMemcpyHostToDevice, b->stream));
  launch_pack_g(1, C.L, scratch, (double2*)C.G64 + (size_t)copy * C.gstride64, b->stream);
  BCK(cudaFreeAsync(scratch, b->stream));
  BCK(cudaGetLastError());
  BCK(cudaStreamSynchronize(b->stream));
  return GFX_OK;
}

gfx_status gfx_batch_get_trafo(gfx_batch* b, int conf, int copy, double* su3) {
  gfx_status s = copy_index(b, conf, copy);
  if (s) return s;
  if (!su3) return bfail(b, GFX_ERR_ARG, "NULL trafo");
  BConf& C = b->desc.c[conf];
  const size_t bytes = sizeof(double) * 18 * 2 * (size_t)C.L.vh;
  double* scratch;
  BCK(cudaMallocAsync((void**)&scratch, bytes, b->stream));
  launch_unpack_g(1, C.L, (const double2*)C.G64 + (size_t)copy * C.gstride64, scratch, b->stream);
  BCK(cudaMemcpyAsync(su3, scratch, bytes, cudaMemcpyDeviceToHost, b->stream));
  BCK(cudaFreeAsync(scratch, b->stream));
  BCK(cudaStreamSynchronize(b->stream));
  return GFX_OK;
}

gfx_status gfx_batch_random_haar(gfx_batch* b, uint64_t seed) {
  if (!b) return bfail(nullptr, GFX_ERR_ARG, "NULL batch");
  for (int c = 0; c < b->nconf; c++) {
    BConf& C = b->desc.c[c];
    for (int k = 0; k < C.ncopies; k++)
      launch_haar_g(C.L, (double2*)C.G64 + (size_t)k * C.gstride64, seed + C.copy_base + k,
                    b->stream);
  }
  BCK(cudaGetLastError());
  BCK(cudaStreamSynchronize(b->stream));
  return GFX_OK;
}

gfx_status gfx_batch_random_haar_copy(gfx_batch* b, int conf, int copy, uint64_t seed) {
  gfx_status s = copy_index(b, conf, copy);
  if (s) return s;
  const BConf& C = b->desc.c[conf];
  launch_haar_g(C.L, (double2*)C.G64 + (size_t)copy * C.gstride64, seed, b->stream);
  BCK(cudaGetLastError());
  BCK(cudaStreamSynchronize(b->stream));
  return GFX_OK;
}

gfx_status gfx_batch_overrelax(gfx_batch* b, const gfx_or_params* pin, gfx_copy_result* res,
                               double* ms_out) {
  if (!b || !pin) return bfail(b, GFX_ERR_ARG, "gfx_batch_overrelax: NULL argument");
  gfx_or_params p = *pin;
  if (p.maxit < 1 || p.checkinterval < 1) return bfail(b, GFX_ERR_ARG, "maxit, checkinterval");
  if (p.checkinterval_double <= 0) p.checkinterval_double = p.checkinterval;
  const int ndir = p.gauge == GFX_GAUGE_COULOMB ? 3 : 4;
  const int prec0 = b->precision == GFX_PREC_DOUBLE ? 1 : 0;
  const bool handover = b->precision == GFX_PREC_MIXED;
  int maxvh = 0;
  for (int c = 0; c < b->nconf; c++) maxvh = std::max(maxvh, b->desc.c[c].L.vh);
  const dim3 cgrid((maxvh + 127) / 128, b->ncopies);
  for (int k = 0; k < b->ncopies; k++) {
    LoopState& H = b->h_states[k];
    std::memset(&H, 0, sizeof(H));
    H.ck = p.checkinterval;
    H.maxit = p.maxit;
    H.criterion = p.criterion;
    H.phase = handover ? 0 : 1;
    H.eps = p.eps;
    H.switch_eps = p.switch_eps;
    H.plateau_ratio = p.plateau_ratio > 0 ? std::pow(p.plateau_ratio, p.checkinterval) : 1e300;
  }
  // the FP32-phase checks measure what a single mixed solve of each lattice measures
  bool odd_changed = false;
  for (int c = 0; c < b->nconf; c++) {
    BConf& C = b->desc.c[c];
    const int odd = handover && !p.fp32_checks_all_sites && fused_check_ok(C.L, 12) ? 1 : 0;
    odd_changed |= odd != C.odd_only;
    C.odd_only = odd;
  }
  if (odd_changed) {  // graphs captured the descriptor by value
    BCK(cudaStreamSynchronize(b->stream));
    for (auto& g : b->graphs) {
      cudaGraphExecDestroy(g.exec);
      cudaGraphDestroy(g.graph);
    }
    b->graphs.clear();
  }
  gfx_status s = write_states(b);
  if (s) return s;
  EventPair ev;
  BCK(ev.create());
  cudaEvent_t e0 = ev.e0, e1 = ev.e1;
  BCK(cudaEventRecord(e0, b->stream));
  // FP32 sweeps start from the FP32 copy of g (g_64_to_32 per copy)
  if (prec0 == 0) convert_batch_kernel<<<cgrid, 128, 0, b->stream>>>(b->desc, 0, -1);
  // iteration 0: sweep, then the first check (advance 0), as overrelax_gauge
  enqueue_sweep(b, prec0, ndir, p.omega, true);
  enqueue_check(b, prec0, prec0, ndir, 0, 0, 0);
  BCK(cudaGetLastError());
  if ((s = read_states(b))) return s;
  auto any_running = [&]() {
    for (int k = 0; k < b->ncopies; k++)
      if (b->h_states[k].done == 0) return true;
    return false;
  };
  if (any_running() && (s = run_phase(b, prec0, ndir, p.checkinterval, p.omega, p.use_graph)))
    return s;
  std::vector<int> iter_switch(b->ncopies, -1);
  if (prec0 == 0) {
    // widen every copy's g to FP64 (reunitarized)
    convert_batch_kernel<<<cgrid, 128, 0, b->stream>>>(b->desc, 1, -1);
    BCK(cudaGetLastError());
  }
  if (handover) {
    // copies that left the FP32 phase are verified and polished: with FP64 sweeps, or
    // (polish = 2) with rebased FP32 sweeps confirmed in FP64, as gfx_overrelax does
    const bool rebased = p.polish == 2;
    const int pprec = rebased ? 3 : 1;
    if (rebased && (s = ensure_rebased(b))) return s;
    std::vector<char> polished(b->ncopies, 0);
    for (int k = 0; k < b->ncopies; k++) {
      LoopState& H = b->h_states[k];
      iter_switch[k] = H.iter;
      if (H.done == 2) {
        H.phase = 1;
        H.done = 0;
        H.prev = 0.0;
        H.ck = p.checkinterval_double;
        H.rebase_at = rebased ? H.iter + kBatchRebaseSweeps : 0;
        polished[k] = 1;
        if (rebased) {
          const int c = conf_of_copy(b, k);
          if ((s = rebase_copy(b, c, k - b->desc.c[c].copy_base, ndir))) return s;
        }
      }
    }
    if ((s = write_states(b))) return s;
    enqueue_check(b, pprec, pprec, ndir, 0, 0, 0);
    BCK(cudaGetLastError());
    if ((s = read_states(b))) return s;
    for (;;) {
      if (any_running() &&
          (s = run_phase(b, pprec, ndir, p.checkinterval_double, p.omega, p.use_graph)))
        return s;
      if (!rebased) break;
      // copies due for a new base (done = 5) get one and run on
      bool again = false;
      for (int k = 0; k < b->ncopies; k++) {
        LoopState& H = b->h_states[k];
        if (H.done != 5) continue;
        const int c = conf_of_copy(b, k), kc = k - b->desc.c[c].copy_base;
        compose_copy(b, c, kc);
        if ((s = rebase_copy(b, c, kc, ndir))) return s;
        H.done = 0;
        H.rebase_at = H.iter + kBatchRebaseSweeps;
        again = true;
      }
      if (!again) break;
      if ((s = write_states(b))) return s;
    }
    if (rebased) {
      // g = (1 + a) g_c in FP64 for every polished copy; an FP64 check confirms the
      // converged ones, and FP64 sweeps continue where it does not
      for (int k = 0; k < b->ncopies; k++) {
        if (!polished[k]) continue;
        const int c = conf_of_copy(b, k);
        compose_copy(b, c, k - b->desc.c[c].copy_base);
        LoopState& H = b->h_states[k];
        H.rebase_at = 0;
        if (H.done == 1) H.done = 0;
      }
      if ((s = write_states(b))) return s;
      enqueue_check(b, 1, 1, ndir, 0, 0, 0);
      BCK(cudaGetLastError());
      if ((s = read_states(b))) return s;
      if (any_running() &&
          (s = run_phase(b, 1, ndir, p.checkinterval_double, p.omega, p.use_graph)))
        return s;
    }
  }
  BCK(cudaEventRecord(e1, b->stream));
  BCK(cudaEventSynchronize(e1));
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  if (ms_out) *ms_out = ms;
  int all = 1;
  for (int c = 0; c < b->nconf; c++) {
    const BConf& C = b->desc.c[c];
    for (int k = 0; k < C.ncopies; k++) {
      const int g = C.copy_base + k;
      const LoopState& H = b->h_states[g];
      const bool conv = H.done == 1;
      all &= conv ? 1 : 0;
      if (!res) continue;
      gfx_copy_result& r = res[g];
      r.conf = c;
      r.copy = k;
      r.converged = conv ? 1 : 0;
      r.iterations = conv ? H.iter : -1;
      r.sweeps = H.iter + 1;
      if (b->precision == GFX_PREC_DOUBLE) r.sweeps_single = 0;
      else if (!handover) r.sweeps_single = r.sweeps;
      else r.sweeps_single = iter_switch[g] + 1;
      r.sweeps_double = r.sweeps - r.sweeps_single;
      r.F = H.last_F;
      r.dAdA = H.last_dAdA;
      r.maxdAdA = H.last_max;
      r.theta = H.last_theta;
      r.theta_slice_max = H.last_theta_slice_max;
    }
  }
  return all ? GFX_OK : GFX_ERR_NOT_CONVERGED;
}

gfx_status gfx_batch_best(gfx_batch* b, const gfx_copy_result* res, int conf, int* best_copy,
                          double* best_F) {
  if (!b || !res || conf < 0 || conf >= b->nconf) return bfail(b, GFX_ERR_ARG, "bad argument");
  const BConf& C = b->desc.c[conf];
  int best = -1;
  double bf = -1e300;
  for (int k = 0; k < C.ncopies; k++) {
    const gfx_copy_result& r = res[C.copy_base + k];
    if (r.converged && r.F > bf) {
      bf = r.F;
      best = k;
    }
  }
  if (best_copy) *best_copy = best;
  if (best_F) *best_F = bf;
  return best >= 0 ? GFX_OK : GFX_ERR_NOT_CONVERGED;
}

}  // extern "C"
