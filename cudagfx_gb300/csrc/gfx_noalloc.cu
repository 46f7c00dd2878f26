// gfx_noalloc.cu -- gfx_functional_noalloc: the gauge functional and theta of fields
// that the caller already holds on the device, computed without allocating memory.
//
// Some callers cannot allocate device memory once they are running: a host
// framework that owns every device byte through its own pool allocator, or a
// long-running service whose device footprint is fixed at start-up.  They keep
// their fields in device memory of their own and need the functional and theta
// without the library allocating reduction buffers.  This entry point uses a
// file-scope device array as its only scratch:
//   * capacity: at most kMaxSlices (1024) time slices; each (slice, parity) pair
//     is reduced by at most kBlocksPerSlice (16) blocks that stride over the slice,
//     so the array holds 2 * 1024 * 16 partial triples and 1024 slice triples
//     (about 0.8 MB, held on every device that loads the library until exit);
//   * the first call in a CUDA context looks up the array's device address with
//     cudaGetSymbolAddress (with that context current) and keeps it for that context;
//     make that first call before any stream capture.  A new context on the device
//     (after cudaDeviceReset, or another context made current) is recognised by its
//     context id and gets a fresh lookup, so a stale address is never used;
//   * every call on a device shares the array and leaves the last call's contents
//     in it.  Each call writes every slot it later reads, so nothing has to be
//     cleared between calls, but calls whose kernels overlap on the GPU (different
//     streams without ordering) race on the array.
#include <algorithm>
#include <cstdio>
#include <mutex>

#include "../../include/gfx.h"
#include "gfx_internal.h"

namespace gfx {
namespace {

constexpr int kMaxSlices = 1024;
constexpr int kBlocksPerSlice = 16;
constexpr int kBlock = 128;
constexpr int kPartialTriples = 2 * kMaxSlices * kBlocksPerSlice;
constexpr int kScratchDoubles = 3 * kPartialTriples + 3 * kMaxSlices;

static __device__ __align__(256) double g_noalloc_scratch[kScratchDoubles];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
// per device: the scratch array's address and the id of the context it belongs to
double* g_scratch_ptr[kMaxDevices] = {nullptr};
unsigned long long g_scratch_ctx[kMaxDevices] = {0};

// The id of the current CUDA context (cuCtxGetId, unique for the process lifetime),
// through the runtime's driver entry points so that the library needs no -lcuda.
// Returns 0 when it cannot be had; the caller then looks the symbol up every call.
typedef int (*CtxGetCurrentFn)(void**);
typedef int (*CtxGetIdFn)(void*, unsigned long long*);
unsigned long long current_context_id() {
  static CtxGetCurrentFn get_current = nullptr;
  static CtxGetIdFn get_id = nullptr;
  static bool looked_up = false;
  if (!looked_up) {
    looked_up = true;
    cudaDriverEntryPointQueryResult q;
    void* f = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) ==
            cudaSuccess && q == cudaDriverEntryPointSuccess)
      get_current = (CtxGetCurrentFn)f;
    f = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) ==
            cudaSuccess && q == cudaDriverEntryPointSuccess)
      get_id = (CtxGetIdFn)f;
  }
  void* ctx = nullptr;
  unsigned long long id = 0;
  if (!get_current || !get_id || get_current(&ctx) != 0 || !ctx || get_id(ctx, &id) != 0)
    return 0;
  return id;
}

// Same per-site quantities as the measurement kernel: X(x) = g(x) w(x),
// F contribution Re tr X, tr[Delta Delta^+] = sum |AH(X)_ij|^2; each block strides
// over its (slice, parity) range.
template <int NRU, int NDIR>
__global__ void __launch_bounds__(kBlock) measure_strided_kernel(Lattice L, const double2* U,
                                                                 const double2* G,
                                                                 double* partials) {
  const int parity = blockIdx.z, t = blockIdx.y;
  constexpr int NCU = Field<double, NRU>::NCHUNK;
  const size_t vh = (size_t)L.vh;
  const int q = 1 - parity;
  const double2* Gq = G + (size_t)q * 6 * vh;
  const double2* Gp = G + (size_t)parity * 6 * vh;
  double fsum = 0.0, dsum = 0.0, dmax = 0.0;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < L.st; k += gridDim.x * blockDim.x) {
    const int i = t * L.st + k;
    const Site c = site_of(L, i, parity);
    Mat3<double> star, a, b, g, X;
    mzero(star);
#pragma unroll
    for (int mu = 0; mu < NDIR; mu++) {
      Field<double, NRU>::load(U + (size_t)(parity * 4 + mu) * NCU * vh, vh, i, a);
      Field<double, 12>::load(Gq, vh, nb_fwd(L, c, mu), b);
      addmul_nd(star, a, b);
      const int jb = nb_bwd(L, c, mu);
      Field<double, NRU>::load(U + (size_t)(q * 4 + mu) * NCU * vh, vh, jb, a);
      Field<double, 12>::load(Gq, vh, jb, b);
      addmul_dd(star, a, b);
    }
    Field<double, 12>::load(Gp, vh, i, g);
    mul(X, g, star);
    fsum += X.e[0][0].re + X.e[1][1].re + X.e[2][2].re;
    const double tim = (X.e[0][0].im + X.e[1][1].im + X.e[2][2].im) * (1.0 / 3.0);
    double d = 0.0;
#pragma unroll
    for (int r = 0; r < 3; r++) d += (X.e[r][r].im - tim) * (X.e[r][r].im - tim);
    double off = 0.0;
#pragma unroll
    for (int r = 0; r < 3; r++)
#pragma unroll
      for (int s = r + 1; s < 3; s++) {
        const double re = (X.e[r][s].re - X.e[s][r].re) * 0.5;
        const double im = (X.e[r][s].im + X.e[s][r].im) * 0.5;
        off += re * re + im * im;
      }
    d += 2.0 * off;
    dsum += d;
    dmax = fmax(dmax, d);
  }
  __shared__ double sh[3][kBlock / 32];
  fsum = warp_sum(fsum);
  dsum = warp_sum(dsum);
  dmax = warp_max(dmax);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) {
    sh[0][w] = fsum;
    sh[1][w] = dsum;
    sh[2][w] = dmax;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double f = 0.0, s = 0.0, m = 0.0;
    for (int k = 0; k < kBlock / 32; k++) {
      f += sh[0][k];
      s += sh[1][k];
      m = fmax(m, sh[2][k]);
    }
    double* out = partials + 3 * ((size_t)(parity * L.lt + t) * gridDim.x + blockIdx.x);
    out[0] = f;
    out[1] = s;
    out[2] = m;
  }
}

}  // namespace
}  // namespace gfx

using namespace gfx;

extern "C" gfx_status gfx_functional_noalloc(const void* links_device, const void* trafo_device,
                                             int lx, int ly, int lz, int lt, int link_reals,
                                             int gauge, double* result_device, void* stream) {
  if (!links_device || !trafo_device || !result_device) return GFX_ERR_ARG;
  if (lx < 2 || ly < 2 || lz < 2 || lt < 2 || (lx | ly | lz | lt) & 1) return GFX_ERR_BAD_VOLUME;
  if ((long long)lx * ly * lz * lt / 2 > (1ll << 30)) return GFX_ERR_BAD_VOLUME;
  if (lt > kMaxSlices) {
    std::fprintf(stderr,
                 "gfx_functional_noalloc: time extent %d exceeds the %d time slices that the "
                 "fixed scratch array holds\n",
                 lt, kMaxSlices);
    return GFX_ERR_ARG;
  }
  if (link_reals != 12 && link_reals != 18) return GFX_ERR_ARG;
  if (gauge != GFX_GAUGE_LANDAU && gauge != GFX_GAUGE_COULOMB) return GFX_ERR_ARG;
  // an error left by the caller's earlier work is not this call's: report that one is
  // pending without clearing it (the caller still reads it with cudaGetLastError)
  if (cudaPeekAtLastError() != cudaSuccess) {
    std::fprintf(stderr, "gfx_functional_noalloc: an earlier CUDA error is pending: %s\n",
                 cudaGetErrorString(cudaPeekAtLastError()));
    return GFX_ERR_STATE;
  }
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return GFX_ERR_CUDA;
  double* scratch;
  {
    std::lock_guard<std::mutex> lock(g_mu);
    const unsigned long long ctx_id = current_context_id();
    if (!g_scratch_ptr[dev] || ctx_id == 0 || ctx_id != g_scratch_ctx[dev]) {
      void* p = nullptr;
      const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
      if (e != cudaSuccess || !p) {
        if (e != cudaSuccess) cudaGetLastError();  // this call's own failure
        g_scratch_ptr[dev] = nullptr;
        return GFX_ERR_CUDA;
      }
      g_scratch_ptr[dev] = (double*)p;
      g_scratch_ctx[dev] = ctx_id;
    }
    scratch = g_scratch_ptr[dev];
  }
  const Lattice L = make_lattice(lx, ly, lz, lt);
  const int nbx = std::min(kBlocksPerSlice, (L.st + kBlock - 1) / kBlock);
  const int ndir = gauge == GFX_GAUGE_COULOMB ? 3 : 4;
  double* partials = scratch;
  double* slice_sums = scratch + 3 * kPartialTriples;
  cudaStream_t s = (cudaStream_t)stream;
  dim3 grid(nbx, lt, 2);
  const double2* U = (const double2*)links_device;
  const double2* G = (const double2*)trafo_device;
  if (link_reals == 18) {
    if (ndir == 4) measure_strided_kernel<18, 4><<<grid, kBlock, 0, s>>>(L, U, G, partials);
    else measure_strided_kernel<18, 3><<<grid, kBlock, 0, s>>>(L, U, G, partials);
  } else {
    if (ndir == 4) measure_strided_kernel<12, 4><<<grid, kBlock, 0, s>>>(L, U, G, partials);
    else measure_strided_kernel<12, 3><<<grid, kBlock, 0, s>>>(L, U, G, partials);
  }
  if (cudaGetLastError() != cudaSuccess) return GFX_ERR_CUDA;
  // per-slice then global sums into the caller's result (gfx_functional_t layout)
  launch_reduce(L, ndir, partials, nbx, slice_sums, (Reduced*)result_device, nullptr, nullptr, 0,
                0, 0, s);
  return cudaGetLastError() == cudaSuccess ? GFX_OK : GFX_ERR_CUDA;
}
