// gfx_kernels.cu -- overrelaxation sweep, functional/theta measurement, reductions,
// plaquette, Polyakov loop and field-layout kernels for sm_103a.
#include <cstdio>

#include <algorithm>

#include "gfx_common.cuh"
#include "gfx_internal.h"

namespace gfx {

Lattice make_lattice(int lx, int ly, int lz, int lt) {
  Lattice L;
  L.lx = lx;
  L.ly = ly;
  L.lz = lz;
  L.lt = lt;
  L.lxh = lx / 2;
  L.vh = (int)((long long)lx * ly * lz * lt / 2);
  L.sy = L.lxh;
  L.sz = L.lxh * ly;
  L.st = L.lxh * ly * lz;
  auto mk = [](uint32_t d) {
    FastDiv f;
    f.d = d;
    uint32_t l = 0;
    while ((1ull << l) < d) l++;
    f.s = 31 + l;
    unsigned long long m = ((1ull << f.s) + d - 1) / d;
    f.m = (uint32_t)m;
    return f;
  };
  L.d_lxh = mk((uint32_t)L.lxh);
  L.d_ly = mk((uint32_t)ly);
  L.d_lz = mk((uint32_t)lz);
  return L;
}

// ---------------------------------------------------------------------------
// overrelaxation half-sweep (overrelax.cu:335-446), in place on parity `parity`
// ---------------------------------------------------------------------------
// MODE (launch_or_halfsweep's mode): 0 plain loads (modes 0 and 2); 1 each block first
// issues one L2 bulk prefetch per contiguous range it reads; 3 and 4 (FP32 12-real
// only) read and write g with the L2 eviction priority evict_last, 4 also reads the
// links as evict_first (or_site_update_hint).  rev != 0 runs the blocks in reverse
// index order: after a half-sweep in forward order, the next one then starts on the
// ranges the previous one touched last, which L2 may still hold.  The sites of one
// parity are independent, so the order does not change the result.
// WIDE = 0 caps an FP32 kernel at 64 registers (4 blocks of 256 per SM); WIDE = 1 leaves
// it its full register set (~124), with which the compiler keeps more loads in flight
// per warp (on GB300 7% faster on 32^4 at half the resident warps)
template <typename T, int NRU, int NDIR, int MODE, int WIDE = 0>
__global__ void __launch_bounds__(256, WIDE ? 1 : (sizeof(T) == 4 ? 4 : 2)) or_halfsweep_kernel(Lattice L,
                                                            const typename VecOf<T>::type* U,
                                                            typename VecOf<T>::type* G, int parity,
                                                            T omega, int rev) {
  constexpr int NCG = Field<T, 12>::NCHUNK;
  constexpr int NCU = Field<T, NRU>::NCHUNK;
  const int blk = rev ? (int)gridDim.x - 1 - (int)blockIdx.x : (int)blockIdx.x;
  if (MODE == 1) {
    const int i0 = blk * blockDim.x;
    prefetch_block<NCU, NCG, NDIR>(L, parity, i0, min((int)blockDim.x, L.vh - i0), U, G);
  }
  const int i = blk * blockDim.x + threadIdx.x;
  if (i >= L.vh) return;
  const Site c = site_of(L, i, parity);
  if constexpr (MODE >= 3 && sizeof(T) == 4 && NRU == 12)
    or_site_update_hint<NDIR, MODE == 4>(L, c, parity, (const float4*)U, (float4*)G, i, omega);
  else
    or_site_update<T, NRU, NDIR>(L, c, parity, U, G, i, omega);
}

void launch_or_halfsweep(int prec, int link_nr, int ndir, const Lattice& L, const void* U, void* G,
                         int parity, double omega, int block, int mode, cudaStream_t s,
                         int wide) {
  const dim3 grid((L.vh + block - 1) / block);
  if (prec == 0 && link_nr == 12 && wide) {
    const float4* u_ = (const float4*)U;
    float4* g_ = (float4*)G;
    const float w = (float)omega;
    if (mode == 1) {
      if (ndir == 4) or_halfsweep_kernel<float, 12, 4, 1, 1><<<grid, block, 0, s>>>(L, u_, g_, parity, w, 0);
      else or_halfsweep_kernel<float, 12, 3, 1, 1><<<grid, block, 0, s>>>(L, u_, g_, parity, w, 0);
    } else if (mode == 3) {
      if (ndir == 4) or_halfsweep_kernel<float, 12, 4, 3, 1><<<grid, block, 0, s>>>(L, u_, g_, parity, w, parity);
      else or_halfsweep_kernel<float, 12, 3, 3, 1><<<grid, block, 0, s>>>(L, u_, g_, parity, w, parity);
    } else if (mode == 4) {
      if (ndir == 4) or_halfsweep_kernel<float, 12, 4, 4, 1><<<grid, block, 0, s>>>(L, u_, g_, parity, w, parity);
      else or_halfsweep_kernel<float, 12, 3, 4, 1><<<grid, block, 0, s>>>(L, u_, g_, parity, w, parity);
    } else {
      const int rev = mode >= 2 ? parity : 0;
      if (ndir == 4) or_halfsweep_kernel<float, 12, 4, 0, 1><<<grid, block, 0, s>>>(L, u_, g_, parity, w, rev);
      else or_halfsweep_kernel<float, 12, 3, 0, 1><<<grid, block, 0, s>>>(L, u_, g_, parity, w, rev);
    }
    return;
  }
#define OR_LAUNCH(T, NR, ND)                                                                     \
  do {                                                                                           \
    const auto* u_ = (const typename VecOf<T>::type*)U;                                          \
    auto* g_ = (typename VecOf<T>::type*)G;                                                      \
    if (mode == 1)                                                                               \
      or_halfsweep_kernel<T, NR, ND, 1><<<grid, block, 0, s>>>(L, u_, g_, parity, (T)omega, 0);  \
    else                                                                                         \
      or_halfsweep_kernel<T, NR, ND, 0><<<grid, block, 0, s>>>(L, u_, g_, parity, (T)omega,      \
                                                               mode >= 2 ? parity : 0);          \
  } while (0)
  if (prec == 2) {  // double-float, 18-real links
    if (ndir == 4) OR_LAUNCH(dfl, 18, 4);
    else OR_LAUNCH(dfl, 18, 3);
  } else if (prec == 0 && link_nr == 8) {
    if (ndir == 4) OR_LAUNCH(float, 8, 4);
    else OR_LAUNCH(float, 8, 3);
  } else if (prec == 0 && mode >= 3) {
    const float4* u_ = (const float4*)U;
    float4* g_ = (float4*)G;
    const float w = (float)omega;
    if (mode == 3) {
      if (ndir == 4) or_halfsweep_kernel<float, 12, 4, 3><<<grid, block, 0, s>>>(L, u_, g_, parity, w, parity);
      else or_halfsweep_kernel<float, 12, 3, 3><<<grid, block, 0, s>>>(L, u_, g_, parity, w, parity);
    } else {
      if (ndir == 4) or_halfsweep_kernel<float, 12, 4, 4><<<grid, block, 0, s>>>(L, u_, g_, parity, w, parity);
      else or_halfsweep_kernel<float, 12, 3, 4><<<grid, block, 0, s>>>(L, u_, g_, parity, w, parity);
    }
  } else if (prec == 0) {
    if (ndir == 4) OR_LAUNCH(float, 12, 4);
    else OR_LAUNCH(float, 12, 3);
  } else if (link_nr == 18) {
    if (ndir == 4) OR_LAUNCH(double, 18, 4);
    else OR_LAUNCH(double, 18, 3);
  } else {
    if (ndir == 4) OR_LAUNCH(double, 12, 4);
    else OR_LAUNCH(double, 12, 3);
  }
#undef OR_LAUNCH
}

// ---------------------------------------------------------------------------
// functional and theta (overrelax.cu:451-605).
// With X(x) = g(x) w(x) = sum_mu U'_mu(x) + U'_mu(x-mu)^+  (U' = g U g^+):
//   sum_x Re tr X = 2 sum_{x,mu} Re tr U'_mu(x)          -> F
//   Delta(x) = sum_mu A_mu(x-mu) - A_mu(x) = -i AH(X)     -> tr[Delta Delta^+]
// where AH is the traceless anti-hermitian part; A = -i AH(U') is the reference's
// vector potential.  Each block covers part of one time slice of one parity and
// writes (sum F, sum dAdA, max dAdA).
// ---------------------------------------------------------------------------
template <typename TC, typename TSU, int NRU, typename TSG, int NDIR>
__global__ void __launch_bounds__(256) measure_kernel(Lattice L,
                                                       const typename VecOf<TSU>::type* U,
                                                       const typename VecOf<TSG>::type* G,
                                                       double* partials, int parity0) {
  // parity is the inner grid dimension: both parities of a slice run back to back, so
  // the links and g they share are read from L2 the second time (a grid of one parity
  // measures parity0 only)
  const int parity = parity0 + blockIdx.y, t = blockIdx.z;
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  constexpr bool F32 = sizeof(TC) == 4 && sizeof(TSG) == 4;
  double f = 0.0, d = 0.0;
  float f32 = 0.0f, d32 = 0.0f;
  if (k < L.st) {
    const int i = t * L.st + k;
    const Site c = site_of(L, i, parity);
    Mat3<TC> star, g;
    if constexpr (F32 && NRU == 12)
      compute_star_f32<NDIR>(L, c, parity, (const float4*)U, (const float4*)G, star);
    else
      compute_star<TC, TSU, NRU, TSG, 12, NDIR>(L, c, parity, U, G, star);
    constexpr int NCG = Field<TSG, 12>::NCHUNK;
    Load<TC, TSG, 12>::go(G + (size_t)parity * NCG * L.vh, (size_t)L.vh, i, g);
    if constexpr (F32) site_functional_f32(g, star, f32, d32);
    else site_functional(g, star, f, d);
  }
  const int nbx = gridDim.x;
  double* out = partials + 3 * ((size_t)(parity * L.lt + t) * nbx + blockIdx.x);
  if constexpr (F32) block_reduce3_f32(f32, d32, out);
  else block_reduce3(f, d, d, out);
}

// ---------------------------------------------------------------------------
// The last odd half-sweep before a check, fused with the check's odd-site partials
// (FP32, 12-real links).  The star w(x) of an odd site depends only on the links and
// the even g, which this half-sweep does not change, so X = g_new(x) w(x) -- the
// quantity the measurement kernel forms for that site after the sweep -- is one
// product away from the registers of the update.  Each block of kMeasBlock sites
// is exactly one measurement block (slice t, block bx; needs st % kMeasBlock == 0)
// and reduces in the measurement kernel's order, so the partials, and with them
// every check value, are bit-identical to the separate measurement; that kernel
// then runs over the even sites only.  This removes the measurement's second read
// of every link (each link has one even and one odd end).
// ---------------------------------------------------------------------------
template <int NDIR>
__global__ void __launch_bounds__(kMeasBlock, 6) or_halfsweep_measure_kernel(
    Lattice L, const float4* U, float4* G, float omega, int rev, int nbx, double* partials) {
  const int blk = rev ? (int)gridDim.x - 1 - (int)blockIdx.x : (int)blockIdx.x;
  const int i = blk * kMeasBlock + threadIdx.x;  // < vh: the grid covers vh exactly
  const int parity = 1;
  const size_t vh = (size_t)L.vh;
  const Site c = site_of(L, i, parity);
  float4* Gp = G + (size_t)parity * 3 * vh;
  Mat3<float> star, gold, gn;
  compute_star_f32<NDIR>(L, c, parity, U, G, star);
  Field<float, 12>::load(Gp, vh, i, gold);
  or_update_composed(gold, star, omega, gn);
  Field<float, 12>::store(Gp, vh, i, gn);
  row2_from_01(gn);  // as the measurement's load of the stored rows
  float f, d;
  site_functional_f32(gn, star, f, d);
  const int t = blk / nbx, bx = blk - t * nbx;
  block_reduce3_f32(f, d, partials + 3 * ((size_t)(parity * L.lt + t) * nbx + bx));
}

bool fused_check_ok(const Lattice& L, int link_nr32) {
  return link_nr32 == 12 && L.st % kMeasBlock == 0;
}

void launch_or_halfsweep_measure(int ndir, const Lattice& L, const void* U, void* G, double omega,
                                 int rev, double* partials, cudaStream_t s) {
  const int nbx = measure_blocks_x(L, kMeasBlock);
  const dim3 grid(L.vh / kMeasBlock);
  if (ndir == 4)
    or_halfsweep_measure_kernel<4><<<grid, kMeasBlock, 0, s>>>(
        L, (const float4*)U, (float4*)G, (float)omega, rev, nbx, partials);
  else
    or_halfsweep_measure_kernel<3><<<grid, kMeasBlock, 0, s>>>(
        L, (const float4*)U, (float4*)G, (float)omega, rev, nbx, partials);
}

// the FP32 measurement's blocks of one parity only
void launch_measure_parity(int ndir, const Lattice& L, const void* U, const void* G,
                           double* partials, int parity, cudaStream_t s) {
  const dim3 grid(measure_blocks_x(L, kMeasBlock), 1, L.lt);
  if (ndir == 4)
    measure_kernel<float, float, 12, float, 4><<<grid, kMeasBlock, 0, s>>>(
        L, (const float4*)U, (const float4*)G, partials, parity);
  else
    measure_kernel<float, float, 12, float, 3><<<grid, kMeasBlock, 0, s>>>(
        L, (const float4*)U, (const float4*)G, partials, parity);
}

int measure_blocks_x(const Lattice& L, int block) { return (L.st + block - 1) / block; }

void launch_measure(int cprec, int link_nr, int gprec, int ndir, const Lattice& L, const void* U,
                    const void* G, double* partials, int block, cudaStream_t s) {
  dim3 grid(measure_blocks_x(L, block), 2, L.lt);
#define MEAS(TC, TSU, NR, TSG, ND)                                                    \
  measure_kernel<TC, TSU, NR, TSG, ND><<<grid, block, 0, s>>>(                      \
      L, (const typename VecOf<TSU>::type*)U, (const typename VecOf<TSG>::type*)G, \
      partials, 0)
  if (cprec == 2) {  // double-float, 18-real links, double-float g
    if (ndir == 4) MEAS(dfl, dfl, 18, dfl, 4);
    else MEAS(dfl, dfl, 18, dfl, 3);
  } else if (cprec == 0 && link_nr == 8) {
    if (ndir == 4) MEAS(float, float, 8, float, 4);
    else MEAS(float, float, 8, float, 3);
  } else if (cprec == 0) {
    if (ndir == 4) MEAS(float, float, 12, float, 4);
    else MEAS(float, float, 12, float, 3);
  } else if (gprec == 0) {
    if (link_nr == 18) {
      if (ndir == 4) MEAS(double, double, 18, float, 4);
      else MEAS(double, double, 18, float, 3);
    } else {
      if (ndir == 4) MEAS(double, double, 12, float, 4);
      else MEAS(double, double, 12, float, 3);
    }
  } else {
    if (link_nr == 18) {
      if (ndir == 4) MEAS(double, double, 18, double, 4);
      else MEAS(double, double, 18, double, 3);
    } else {
      if (ndir == 4) MEAS(double, double, 12, double, 4);
      else MEAS(double, double, 12, double, 3);
    }
  }
#undef MEAS
}

// per-slice sums: block t reduces both parities' partials of slice t (fixed order).
// odd_only: the odd sites' partials alone, their F and dAdA sums doubled (the FP32-phase
// checks, gfx_internal.h)
__global__ void slice_reduce_kernel(const double* partials, int nbx, int lt, double* slice_sums,
                                    int odd_only) {
  const int t = blockIdx.x;
  double f = 0.0, d = 0.0, m = 0.0;
  const int j0 = odd_only ? nbx : 0;
  for (int j = j0 + threadIdx.x; j < 2 * nbx; j += blockDim.x) {
    const int p = j / nbx, bx = j % nbx;
    const double* q = partials + 3 * ((size_t)(p * lt + t) * nbx + bx);
    f += q[0];
    d += q[1];
    m = fmax(m, q[2]);
  }
  if (odd_only) {
    f *= 2.0;
    d *= 2.0;
  }
  block_reduce3(f, d, m, slice_sums + 3 * t);
}

__global__ void final_reduce_kernel(const double* slice_sums, int lt, double vol, double v3,
                                    int ndir, Reduced* out, LoopState* loop, CheckRecord* hist,
                                    int advance, cudaGraphConditionalHandle handle,
                                    int use_handle) {
  const int done = reduce_and_check(slice_sums, lt, vol, v3, ndir, out, loop, hist, advance);
  if (threadIdx.x == 0 && loop && use_handle)
    cudaGraphSetConditional(handle, done == 0 ? 1u : 0u);
}

void launch_reduce(const Lattice& L, int ndir, const double* partials, int nbx, double* slice_sums,
                   Reduced* out, LoopState* loop, CheckRecord* hist, int advance,
                   unsigned long long graph_handle, int use_handle, cudaStream_t s, int odd_only) {
  slice_reduce_kernel<<<L.lt, 256, 0, s>>>(partials, nbx, L.lt, slice_sums, odd_only);
  const double vol = 2.0 * (double)L.vh;
  const double v3 = (double)L.lx * L.ly * L.lz;
  final_reduce_kernel<<<1, 256, 0, s>>>(slice_sums, L.lt, vol, v3, ndir, out, loop, hist,
                                        advance, (cudaGraphConditionalHandle)graph_handle,
                                        use_handle);
}

// ---------------------------------------------------------------------------
// plaquette (overrelax.cu:34-138) and Polyakov loop
// ---------------------------------------------------------------------------
__device__ __forceinline__ void coords_of(const Lattice& L, int i, int parity, int& x, int& y,
                                          int& z, int& t) {
  Site c = site_of(L, i, parity);
  x = 2 * c.xh + c.s;
  y = c.y;
  z = c.z;
  t = c.t;
}
__device__ __forceinline__ int eo_of(const Lattice& L, int x, int y, int z, int t) {
  return (x >> 1) + L.lxh * (y + L.ly * (z + L.lz * t));
}
__device__ __forceinline__ void shift(const Lattice& L, int mu, int dir, int& x, int& y, int& z,
                                      int& t) {
  if (mu == 0) x = (x + dir + L.lx) % L.lx;
  else if (mu == 1) y = (y + dir + L.ly) % L.ly;
  else if (mu == 2) z = (z + dir + L.lz) % L.lz;
  else t = (t + dir + L.lt) % L.lt;
}

template <typename T, int NR>
__device__ __forceinline__ void load_link(const Lattice& L, const typename VecOf<T>::type* U,
                                          int x, int y, int z, int t, int mu, Mat3<double>& m) {
  constexpr int NC = Field<T, NR>::NCHUNK;
  const int p = (x + y + z + t) & 1;
  Mat3<T> a;
  Field<T, NR>::load(U + (size_t)(p * 4 + mu) * NC * L.vh, (size_t)L.vh, eo_of(L, x, y, z, t), a);
#pragma unroll
  for (int r = 0; r < 3; r++)
#pragma unroll
    for (int c = 0; c < 3; c++) m.e[r][c] = cmk<double>(a.e[r][c].re, a.e[r][c].im);
}

template <typename T, int NR>
__global__ void __launch_bounds__(256) plaquette_kernel(Lattice L, const typename VecOf<T>::type* U,
                                                         double* partials) {
  const int parity = blockIdx.y;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  double acc = 0.0;
  if (i < L.vh) {
    int x, y, z, t;
    coords_of(L, i, parity, x, y, z, t);
#pragma unroll 1
    for (int nu = 0; nu < 3; nu++)
#pragma unroll 1
      for (int mu = nu + 1; mu < 4; mu++) {
        Mat3<double> M1, M2, M3, M4, A, B;
        load_link<T, NR>(L, U, x, y, z, t, mu, M1);
        int x1 = x, y1 = y, z1 = z, t1 = t;
        shift(L, mu, 1, x1, y1, z1, t1);
        load_link<T, NR>(L, U, x1, y1, z1, t1, nu, M2);
        int x2 = x, y2 = y, z2 = z, t2 = t;
        shift(L, nu, 1, x2, y2, z2, t2);
        load_link<T, NR>(L, U, x2, y2, z2, t2, mu, M3);
        load_link<T, NR>(L, U, x, y, z, t, nu, M4);
        mul(A, M1, M2);  // U_mu(x) U_nu(x+mu)
        mul(B, M4, M3);  // U_nu(x) U_mu(x+nu)
        double tr = 0.0;
#pragma unroll
        for (int a = 0; a < 3; a++)
#pragma unroll
          for (int b = 0; b < 3; b++) tr += A.e[a][b].re * B.e[a][b].re + A.e[a][b].im * B.e[a][b].im;
        acc += tr / 3.0;
      }
  }
  block_reduce3(acc, 0.0, 0.0, partials + 3 * ((size_t)parity * gridDim.x + blockIdx.x));
}

__global__ void sum_partials_kernel(const double* partials, int n, double scale, double* out) {
  double f = 0.0;
  for (int j = threadIdx.x; j < n; j += blockDim.x) f += partials[3 * j];
  __shared__ double sh[32];
  f = warp_sum(f);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = f;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int k = 0; k < (int)(blockDim.x >> 5); k++) s += sh[k];
    *out = s * scale;
  }
}

void launch_plaquette(int link_nr_prec, const Lattice& L, const void* U, double* partials,
                      double* out, cudaStream_t s) {
  const int block = 128;
  dim3 grid((L.vh + block - 1) / block, 2);
  if (link_nr_prec == 0)
    plaquette_kernel<float, 12><<<grid, block, 0, s>>>(L, (const float4*)U, partials);
  else if (link_nr_prec == 18)
    plaquette_kernel<double, 18><<<grid, block, 0, s>>>(L, (const double2*)U, partials);
  else
    plaquette_kernel<double, 12><<<grid, block, 0, s>>>(L, (const double2*)U, partials);
  const double vol = 2.0 * (double)L.vh;
  sum_partials_kernel<<<1, 256, 0, s>>>(partials, 2 * grid.x, 1.0 / (6.0 * vol), out);
}

template <typename T, int NR>
__global__ void polyakov_kernel(Lattice L, const typename VecOf<T>::type* U, double* partials) {
  const int v3 = L.lx * L.ly * L.lz;
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  double re = 0.0, im = 0.0;
  if (k < v3) {
    const int x = k % L.lx, y = (k / L.lx) % L.ly, z = k / (L.lx * L.ly);
    Mat3<double> P, U3, tmp;
    mzero(P);
    P.e[0][0].re = P.e[1][1].re = P.e[2][2].re = 1.0;
    for (int t = 0; t < L.lt; t++) {
      load_link<T, NR>(L, U, x, y, z, t, 3, U3);
      mul(tmp, P, U3);
      P = tmp;
    }
    re = (P.e[0][0].re + P.e[1][1].re + P.e[2][2].re) / 3.0;
    im = (P.e[0][0].im + P.e[1][1].im + P.e[2][2].im) / 3.0;
  }
  block_reduce3(re, im, 0.0, partials + 3 * (size_t)blockIdx.x);
}

__global__ void sum_partials2_kernel(const double* partials, int n, double scale, double* out) {
  double a = 0.0, b = 0.0;
  for (int j = threadIdx.x; j < n; j += blockDim.x) {
    a += partials[3 * j];
    b += partials[3 * j + 1];
  }
  __shared__ double sh[2][32];
  a = warp_sum(a);
  b = warp_sum(b);
  if ((threadIdx.x & 31) == 0) {
    sh[0][threadIdx.x >> 5] = a;
    sh[1][threadIdx.x >> 5] = b;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double s0 = 0.0, s1 = 0.0;
    for (int k = 0; k < (int)(blockDim.x >> 5); k++) {
      s0 += sh[0][k];
      s1 += sh[1][k];
    }
    out[0] = s0 * scale;
    out[1] = s1 * scale;
  }
}

void launch_polyakov(int link_nr_prec, const Lattice& L, const void* U, double* partials,
                     double* out, cudaStream_t s) {
  const int v3 = L.lx * L.ly * L.lz;
  const int block = 128;
  const int nb = (v3 + block - 1) / block;
  if (link_nr_prec == 0)
    polyakov_kernel<float, 12><<<nb, block, 0, s>>>(L, (const float4*)U, partials);
  else if (link_nr_prec == 18)
    polyakov_kernel<double, 18><<<nb, block, 0, s>>>(L, (const double2*)U, partials);
  else
    polyakov_kernel<double, 12><<<nb, block, 0, s>>>(L, (const double2*)U, partials);
  sum_partials2_kernel<<<1, 256, 0, s>>>(partials, nb, 1.0 / (double)v3, out);
}

// ---------------------------------------------------------------------------
// layout conversion: host AoS (su3 = complex[3][3], lexicographic, link 4*pos+mu)
// <-> even/odd SoA planes
// ---------------------------------------------------------------------------
__device__ __forceinline__ long long lexi_of(const Lattice& L, int i, int parity) {
  int x, y, z, t;
  coords_of(L, i, parity, x, y, z, t);
  return x + (long long)L.lx * (y + (long long)L.ly * (z + (long long)L.lz * t));
}

template <typename T, int NR>
__global__ void pack_links_kernel(Lattice L, const double* aos, typename VecOf<T>::type* U) {
  const int parity = blockIdx.y;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= L.vh) return;
  constexpr int NC = Field<T, NR>::NCHUNK;
  const long long pos = lexi_of(L, i, parity);
  for (int mu = 0; mu < 4; mu++) {
    const double* src = aos + 18 * (4 * pos + mu);
    Mat3<T> m;
#pragma unroll
    for (int k = 0; k < 9; k++) m.e[k / 3][k % 3] = cmk<T>((T)src[2 * k], (T)src[2 * k + 1]);
    Field<T, NR>::store(U + (size_t)(parity * 4 + mu) * NC * L.vh, (size_t)L.vh, i, m);
  }
}

template <typename T, int NR>
__global__ void unpack_links_kernel(Lattice L, const typename VecOf<T>::type* U, double* aos) {
  const int parity = blockIdx.y;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= L.vh) return;
  constexpr int NC = Field<T, NR>::NCHUNK;
  const long long pos = lexi_of(L, i, parity);
  for (int mu = 0; mu < 4; mu++) {
    Mat3<T> m;
    Field<T, NR>::load(U + (size_t)(parity * 4 + mu) * NC * L.vh, (size_t)L.vh, i, m);
    double* dst = aos + 18 * (4 * pos + mu);
#pragma unroll
    for (int k = 0; k < 9; k++) {
      dst[2 * k] = (double)m.e[k / 3][k % 3].re;
      dst[2 * k + 1] = (double)m.e[k / 3][k % 3].im;
    }
  }
}

void launch_pack_links(int link_nr_prec, const Lattice& L, const double* aos, void* U,
                       cudaStream_t s) {
  dim3 grid((L.vh + 127) / 128, 2);
  if (link_nr_prec == 0) pack_links_kernel<float, 12><<<grid, 128, 0, s>>>(L, aos, (float4*)U);
  else if (link_nr_prec == 18) pack_links_kernel<double, 18><<<grid, 128, 0, s>>>(L, aos, (double2*)U);
  else pack_links_kernel<double, 12><<<grid, 128, 0, s>>>(L, aos, (double2*)U);
}
void launch_unpack_links(int link_nr_prec, const Lattice& L, const void* U, double* aos,
                         cudaStream_t s) {
  dim3 grid((L.vh + 127) / 128, 2);
  if (link_nr_prec == 0) unpack_links_kernel<float, 12><<<grid, 128, 0, s>>>(L, (const float4*)U, aos);
  else if (link_nr_prec == 18) unpack_links_kernel<double, 18><<<grid, 128, 0, s>>>(L, (const double2*)U, aos);
  else unpack_links_kernel<double, 12><<<grid, 128, 0, s>>>(L, (const double2*)U, aos);
}

template <typename T>
__global__ void pack_g_kernel(Lattice L, const double* aos, typename VecOf<T>::type* G) {
  const int parity = blockIdx.y;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= L.vh) return;
  constexpr int NC = Field<T, 12>::NCHUNK;
  const double* src = aos + 18 * lexi_of(L, i, parity);
  Mat3<T> m;
#pragma unroll
  for (int k = 0; k < 9; k++) m.e[k / 3][k % 3] = cmk<T>((T)src[2 * k], (T)src[2 * k + 1]);
  Field<T, 12>::store(G + (size_t)parity * NC * L.vh, (size_t)L.vh, i, m);
}

// rows 0,1 as stored; row 2 = conj(row0 x row1) as from2vtosu3_trafo (su3manip.c:303-359)
template <typename T>
__global__ void unpack_g_kernel(Lattice L, const typename VecOf<T>::type* G, double* aos) {
  const int parity = blockIdx.y;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= L.vh) return;
  constexpr int NC = Field<T, 12>::NCHUNK;
  Mat3<T> m;
  Field<T, 12>::load(G + (size_t)parity * NC * L.vh, (size_t)L.vh, i, m);
  Mat3<double> d;
#pragma unroll
  for (int r = 0; r < 2; r++)
#pragma unroll
    for (int c = 0; c < 3; c++) d.e[r][c] = cmk<double>(m.e[r][c].re, m.e[r][c].im);
  row2_from_01(d);
  double* dst = aos + 18 * lexi_of(L, i, parity);
#pragma unroll
  for (int k = 0; k < 9; k++) {
    dst[2 * k] = d.e[k / 3][k % 3].re;
    dst[2 * k + 1] = d.e[k / 3][k % 3].im;
  }
}

void launch_pack_g(int gprec, const Lattice& L, const double* aos, void* G, cudaStream_t s) {
  dim3 grid((L.vh + 127) / 128, 2);
  if (gprec == 0) pack_g_kernel<float><<<grid, 128, 0, s>>>(L, aos, (float4*)G);
  else pack_g_kernel<double><<<grid, 128, 0, s>>>(L, aos, (double2*)G);
}
void launch_unpack_g(int gprec, const Lattice& L, const void* G, double* aos, cudaStream_t s) {
  dim3 grid((L.vh + 127) / 128, 2);
  if (gprec == 0) unpack_g_kernel<float><<<grid, 128, 0, s>>>(L, (const float4*)G, aos);
  else unpack_g_kernel<double><<<grid, 128, 0, s>>>(L, (const double2*)G, aos);
}

// ---------------------------------------------------------------------------
// The same conversions by tiles, coalesced on both sides.  LX is even, so the
// lexicographic site pos has eo index pos >> 1 in its parity: a block takes the eo
// indices j0 .. j0 + kTileEo - 1 of both parities, which are exactly the 2 kTileEo
// consecutive sites 2 j0 .. of the host order.  That AoS range is moved with
// consecutive 16-byte accesses through shared memory -- from or to device memory, or
// page-locked host memory that the GPU reaches directly (the host copy and the
// layout change are then one pass) -- and each thread moves one matrix between the
// tile and the even/odd planes.  Needs a 16-byte aligned AoS pointer.
// ---------------------------------------------------------------------------
constexpr int kTileEo = 32;

// links (NMAT 4, link 4 pos + mu) or g (NMAT 1): AoS -> FP64 planes of NR reals, and
// with W32 the FP32 12-real copy (the rounding of rows 0, 1, as links_64_to_32_kernel)
template <int NMAT, int NR, bool W32>
__global__ void __launch_bounds__(128) pack_tile_kernel(Lattice L, const double2* __restrict__ aos,
                                                        double2* F64, float4* F32) {
  extern __shared__ double2 tile[];
  const int j0 = blockIdx.x * kTileEo;
  const int nj = min(kTileEo, L.vh - j0);
  const int n = 2 * nj * NMAT * 9;
  const double2* src = aos + (size_t)2 * j0 * NMAT * 9;
  for (int k = threadIdx.x; k < n; k += blockDim.x) tile[k] = src[k];
  __syncthreads();
  constexpr int NC = Field<double, NR>::NCHUNK;
  const size_t vh = (size_t)L.vh;
  for (int k = threadIdx.x; k < 2 * NMAT * nj; k += blockDim.x) {
    const int j = k % nj, pm = k / nj, parity = pm / NMAT, mu = pm - parity * NMAT;
    const Site c = site_of(L, j0 + j, parity);
    const double2* m = tile + ((2 * j + c.s) * NMAT + mu) * 9;
    Mat3<double> d;
#pragma unroll
    for (int e = 0; e < 9; e++) d.e[e / 3][e % 3] = cmk<double>(m[e].x, m[e].y);
    Field<double, NR>::store(F64 + (size_t)(parity * NMAT + mu) * NC * vh, vh, j0 + j, d);
    if (W32) {
      Mat3<float> f;
#pragma unroll
      for (int r = 0; r < 2; r++)
#pragma unroll
        for (int e = 0; e < 3; e++)
          f.e[r][e] = cmk<float>((float)d.e[r][e].re, (float)d.e[r][e].im);
      Field<float, 12>::store(F32 + (size_t)(parity * NMAT + mu) * 3 * vh, vh, j0 + j, f);
    }
  }
}

// FP64 12-real g planes -> AoS su3 (row 2 rebuilt, as unpack_g_kernel<double>)
__global__ void __launch_bounds__(128) unpack_g_tile_kernel(Lattice L, const double2* G,
                                                            double2* __restrict__ aos) {
  __shared__ double2 tile[2 * kTileEo * 9];
  const int j0 = blockIdx.x * kTileEo;
  const int nj = min(kTileEo, L.vh - j0);
  const size_t vh = (size_t)L.vh;
  for (int k = threadIdx.x; k < 2 * nj; k += blockDim.x) {
    const int j = k % nj, parity = k / nj;
    const Site c = site_of(L, j0 + j, parity);
    Mat3<double> m;
    Field<double, 12>::load(G + (size_t)parity * 6 * vh, vh, j0 + j, m);
    double2* o = tile + (2 * j + c.s) * 9;
#pragma unroll
    for (int e = 0; e < 9; e++) o[e] = make_double2(m.e[e / 3][e % 3].re, m.e[e / 3][e % 3].im);
  }
  __syncthreads();
  double2* dst = aos + (size_t)2 * j0 * 9;
  for (int k = threadIdx.x; k < 2 * nj * 9; k += blockDim.x) dst[k] = tile[k];
}

void launch_pack_links_tiled(int link_nr, const Lattice& L, const void* aos, void* U64, void* U32,
                             cudaStream_t s) {
  const int grid = (L.vh + kTileEo - 1) / kTileEo;
  const size_t sm = sizeof(double2) * 2 * kTileEo * 4 * 9;
  const double2* a = (const double2*)aos;
  if (link_nr == 18) {
    if (U32) pack_tile_kernel<4, 18, true><<<grid, 128, sm, s>>>(L, a, (double2*)U64, (float4*)U32);
    else pack_tile_kernel<4, 18, false><<<grid, 128, sm, s>>>(L, a, (double2*)U64, nullptr);
  } else {
    if (U32) pack_tile_kernel<4, 12, true><<<grid, 128, sm, s>>>(L, a, (double2*)U64, (float4*)U32);
    else pack_tile_kernel<4, 12, false><<<grid, 128, sm, s>>>(L, a, (double2*)U64, nullptr);
  }
}
void launch_pack_g_tiled(const Lattice& L, const void* aos, void* G64, cudaStream_t s) {
  const int grid = (L.vh + kTileEo - 1) / kTileEo;
  pack_tile_kernel<1, 12, false><<<grid, 128, sizeof(double2) * 2 * kTileEo * 9, s>>>(
      L, (const double2*)aos, (double2*)G64, nullptr);
}
void launch_unpack_g_tiled(const Lattice& L, const void* G64, void* aos, cudaStream_t s) {
  const int grid = (L.vh + kTileEo - 1) / kTileEo;
  unpack_g_tile_kernel<<<grid, 128, 0, s>>>(L, (const double2*)G64, (double2*)aos);
}

// FP32 copy of the links: 12 reals (rows 0, 1) or 8 (a2, a3, arg a1, arg c1, b1; the
// angles by atan2 in FP64 as su3to8 does, su3manip.c:234-253)
template <int NR, int NR32>
__global__ void links_64_to_32_kernel(Lattice L, const double2* U64, float4* U32) {
  const int blk = blockIdx.y;  // parity*4 + mu
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= L.vh) return;
  Mat3<double> m;
  Field<double, NR>::load(U64 + (size_t)blk * Field<double, NR>::NCHUNK * L.vh, (size_t)L.vh, i, m);
  Mat3<float> f;
#pragma unroll
  for (int r = 0; r < 3; r++)
#pragma unroll
    for (int c = 0; c < 3; c++) f.e[r][c] = cmk<float>((float)m.e[r][c].re, (float)m.e[r][c].im);
  if (NR32 == 8) {
    float4* o = U32 + (size_t)blk * 5 * L.vh;
    o[i] = make_float4((float)m.e[0][1].re, (float)m.e[0][1].im, (float)m.e[0][2].re,
                       (float)m.e[0][2].im);
    o[(size_t)L.vh + i] =
        make_float4((float)atan2(m.e[0][0].im, m.e[0][0].re), (float)atan2(m.e[2][0].im, m.e[2][0].re),
                    (float)m.e[1][0].re, (float)m.e[1][0].im);
    Field<float, 12>::store(o + 2 * (size_t)L.vh, (size_t)L.vh, i, f);  // the exact rows
    return;
  }
  Field<float, 12>::store(U32 + (size_t)blk * 3 * L.vh, (size_t)L.vh, i, f);
}

void launch_convert_links_64_to_32(int link_nr, int link_nr32, const Lattice& L, const void* U64,
                                   void* U32, cudaStream_t s) {
  dim3 grid((L.vh + 127) / 128, 8);
  const double2* u = (const double2*)U64;
  float4* o = (float4*)U32;
  if (link_nr == 18) {
    if (link_nr32 == 8) links_64_to_32_kernel<18, 8><<<grid, 128, 0, s>>>(L, u, o);
    else links_64_to_32_kernel<18, 12><<<grid, 128, 0, s>>>(L, u, o);
  } else {
    if (link_nr32 == 8) links_64_to_32_kernel<12, 8><<<grid, 128, 0, s>>>(L, u, o);
    else links_64_to_32_kernel<12, 12><<<grid, 128, 0, s>>>(L, u, o);
  }
}

// double-float copies: links as 18 reals (rows 0..2), g as 12; hi = fl(d), lo = fl(d - hi)
template <int NR>
__global__ void links_64_to_df_kernel(Lattice L, const double2* U64, float4* Udf) {
  const int blk = blockIdx.y;  // parity*4 + mu
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= L.vh) return;
  Mat3<double> m;
  Field<double, NR>::load(U64 + (size_t)blk * Field<double, NR>::NCHUNK * L.vh, (size_t)L.vh, i, m);
  float4* o = Udf + (size_t)blk * 9 * L.vh;
#pragma unroll
  for (int k = 0; k < 9; k++) {
    const dfl re(m.e[k / 3][k % 3].re), im(m.e[k / 3][k % 3].im);
    o[(size_t)k * L.vh + i] = make_float4(re.hi, re.lo, im.hi, im.lo);
  }
}

void launch_convert_links_64_to_df(int link_nr, const Lattice& L, const void* U64, void* Udf,
                                   cudaStream_t s) {
  dim3 grid((L.vh + 127) / 128, 8);
  if (link_nr == 18)
    links_64_to_df_kernel<18><<<grid, 128, 0, s>>>(L, (const double2*)U64, (float4*)Udf);
  else
    links_64_to_df_kernel<12><<<grid, 128, 0, s>>>(L, (const double2*)U64, (float4*)Udf);
}

// g: 12 reals per site, both parities; to_df = 1: G64 -> Gdf, 0: Gdf -> G64 (exact)
__global__ void g_df_kernel(Lattice L, double2* G64, float4* Gdf, int to_df) {
  const int parity = blockIdx.y;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= L.vh) return;
  double2* g = G64 + (size_t)parity * 6 * L.vh;
  float4* h = Gdf + (size_t)parity * 6 * L.vh;
#pragma unroll
  for (int k = 0; k < 6; k++) {
    const size_t o = (size_t)k * L.vh + i;
    if (to_df) {
      const double2 v = g[o];
      const dfl re(v.x), im(v.y);
      h[o] = make_float4(re.hi, re.lo, im.hi, im.lo);
    } else {
      const float4 v = h[o];
      g[o] = make_double2((double)v.x + (double)v.y, (double)v.z + (double)v.w);
    }
  }
}

void launch_convert_g_df(int to_df, const Lattice& L, void* G64, void* Gdf, cudaStream_t s) {
  dim3 grid((L.vh + 127) / 128, 2);
  g_df_kernel<<<grid, 128, 0, s>>>(L, (double2*)G64, (float4*)Gdf, to_df);
}

// g precision change; widening reunitarizes in FP64
__global__ void g_32_to_64_kernel(Lattice L, const float4* G32, double2* G64) {
  const int parity = blockIdx.y;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= L.vh) return;
  Mat3<double> m;
  Load<double, float, 12>::go(G32 + (size_t)parity * 3 * L.vh, (size_t)L.vh, i, m);
  Field<double, 12>::store(G64 + (size_t)parity * 6 * L.vh, (size_t)L.vh, i, m);
}
__global__ void g_64_to_32_kernel(Lattice L, const double2* G64, float4* G32) {
  const int parity = blockIdx.y;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= L.vh) return;
  Mat3<double> m;
  Field<double, 12>::load(G64 + (size_t)parity * 6 * L.vh, (size_t)L.vh, i, m);
  Mat3<float> f;
#pragma unroll
  for (int r = 0; r < 3; r++)
#pragma unroll
    for (int c = 0; c < 3; c++) f.e[r][c] = cmk<float>((float)m.e[r][c].re, (float)m.e[r][c].im);
  Field<float, 12>::store(G32 + (size_t)parity * 3 * L.vh, (size_t)L.vh, i, f);
}

void launch_convert_g(int from_prec, int to_prec, const Lattice& L, const void* Gin, void* Gout,
                      cudaStream_t s) {
  dim3 grid((L.vh + 127) / 128, 2);
  if (from_prec == 0 && to_prec == 1)
    g_32_to_64_kernel<<<grid, 128, 0, s>>>(L, (const float4*)Gin, (double2*)Gout);
  else if (from_prec == 1 && to_prec == 0)
    g_64_to_32_kernel<<<grid, 128, 0, s>>>(L, (const double2*)Gin, (float4*)Gout);
}

// U_mu(x) <- g(x) U_mu(x) g^+(x+mu), in place, FP64 (the host g_trafo of
// observables.c:17-47 moved to the device)
template <int NR>
__global__ void apply_trafo_kernel(Lattice L, double2* U, const double2* G) {
  const int parity = blockIdx.y;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= L.vh) return;
  constexpr int NC = Field<double, NR>::NCHUNK;
  const size_t vh = (size_t)L.vh;
  const Site c = site_of(L, i, parity);
  Mat3<double> g, gn, u, h, r;
  Field<double, 12>::load(G + (size_t)parity * 6 * vh, vh, i, g);
  for (int mu = 0; mu < 4; mu++) {
    double2* blk = U + (size_t)(parity * 4 + mu) * NC * vh;
    Field<double, NR>::load(blk, vh, i, u);
    Field<double, 12>::load(G + (size_t)(1 - parity) * 6 * vh, vh, nb_fwd(L, c, mu), gn);
    mul(h, g, u);
    mzero(r);
    addmul_nd(r, h, gn);
    Field<double, NR>::store(blk, vh, i, r);
  }
}

// Haar SU(3): rows 0,1 of a complex Gaussian matrix, Gram-Schmidt; the Gaussians come
// from splitmix64 streams keyed by (seed, lexicographic site) and Box-Muller in FP64
__device__ __forceinline__ unsigned long long splitmix64(unsigned long long& x) {
  unsigned long long z = (x += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

__global__ void haar_g_kernel(Lattice L, double2* G, unsigned long long seed) {
  const int parity = blockIdx.y;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= L.vh) return;
  const long long pos = lexi_of(L, i, parity);
  unsigned long long st = seed * 0xD1B54A32D192ED03ull + (unsigned long long)pos * 0x8CB92BA72F3D8DD7ull;
  Mat3<double> m;
#pragma unroll
  for (int k = 0; k < 6; k++) {
    const double u1 = ((double)(splitmix64(st) >> 11) + 0.5) * (1.0 / 9007199254740992.0);
    const double u2 = ((double)(splitmix64(st) >> 11) + 0.5) * (1.0 / 9007199254740992.0);
    const double r = sqrt(-2.0 * log(u1));
    double sp, cp;
    sincospi(2.0 * u2, &sp, &cp);
    m.e[k / 3][k % 3] = cmk(r * cp, r * sp);
  }
  normalize<double, false>(m);
  Field<double, 12>::store(G + (size_t)parity * 6 * L.vh, (size_t)L.vh, i, m);
}

void launch_haar_g(const Lattice& L, double2* G64, unsigned long long seed, cudaStream_t s) {
  dim3 grid((L.vh + 127) / 128, 2);
  haar_g_kernel<<<grid, 128, 0, s>>>(L, G64, seed);
}

void launch_apply_trafo(int link_nr, const Lattice& L, void* U64, const void* G64, cudaStream_t s) {
  dim3 grid((L.vh + 127) / 128, 2);
  if (link_nr == 18)
    apply_trafo_kernel<18><<<grid, 128, 0, s>>>(L, (double2*)U64, (const double2*)G64);
  else
    apply_trafo_kernel<12><<<grid, 128, 0, s>>>(L, (double2*)U64, (const double2*)G64);
}

}  // namespace gfx
