// gfx_rebased.cu -- FP32 overrelaxation sweeps with FP64 accuracy ("rebased" sweeps):
// the FP64 construction of a base, the sweep and check kernels, and their launchers.
// The method and the device code are described in gfx_rebased.cuh.
#include <algorithm>

#include "gfx_internal.h"
#include "gfx_rebased.cuh"

namespace gfx {

constexpr int kRebasedBlock = 128;

// ---------------------------------------------------------------------------
// base construction, in double-float on the FP32 units
// ---------------------------------------------------------------------------
// GB300 runs FP64 at 1/64 of its FP32 rate: the base built in FP64 took the FP64 pipe
// to 87-95% (3.1 ms on 32^4, 8% of a batched Gribov solve with a base per copy).  The
// FP64 links and g are split into double-float pairs on the integer units
// (gfx_narrow.h, bit for bit hi = (float)d, lo = (float)(d - hi)) and the products and
// sums run in double-float (~2^-46; the stored pairs hold ~2^-48).

// U'_mu(x) = g(x) U_mu(x) g(x+mu)^+ for mu = blockIdx.z: rows 0,1 as an FP32 value (Ur,
// the 12-real FP32 link layout) and the FP32 remainder (Ulo, the same layout)
template <int NR>
__global__ void __launch_bounds__(128) rebase_links_kernel(Lattice L, const double2* __restrict__ U,
                                                           const double2* __restrict__ G,
                                                           float4* __restrict__ Ur,
                                                           float4* __restrict__ Ulo) {
  const int parity = blockIdx.y, mu = blockIdx.z;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= L.vh) return;
  constexpr int NC = Field<double, NR>::NCHUNK;
  const size_t vh = (size_t)L.vh;
  const Site c = site_of(L, i, parity);
  Mat3<dfl> g, gn, u;
  load_narrow<6>(G + (size_t)parity * 6 * vh, vh, i, g);
  load_narrow<NC>(U + (size_t)(parity * 4 + mu) * NC * vh, vh, i, u);
  load_narrow<6>(G + (size_t)(1 - parity) * 6 * vh, vh, nb_fwd(L, c, mu), gn);
  float hi[12], lo[12];
#pragma unroll
  for (int a = 0; a < 2; a++) {
    cplx<dfl> h[3];
#pragma unroll
    for (int k = 0; k < 3; k++) h[k] = mul_entry(g, u, a, k);
#pragma unroll
    for (int j = 0; j < 3; j++) {
      cplx<dfl> x = cmulc(h[0], gn.e[j][0]);
      cmacc(x, h[1], gn.e[j][1]);
      cmacc(x, h[2], gn.e[j][2]);
      const int k = 2 * (3 * a + j);
      hi[k] = x.re.hi;
      hi[k + 1] = x.im.hi;
      lo[k] = x.re.lo;
      lo[k + 1] = x.im.lo;
    }
  }
  const size_t off = (size_t)(parity * 4 + mu) * 3 * vh + i;
#pragma unroll
  for (int p = 0; p < 3; p++) {
    Ur[off + p * vh] = make_float4(hi[4 * p], hi[4 * p + 1], hi[4 * p + 2], hi[4 * p + 3]);
    Ulo[off + p * vh] = make_float4(lo[4 * p], lo[4 * p + 1], lo[4 * p + 2], lo[4 * p + 3]);
  }
}

// rows 0,1 of a rebased link as double-float pairs hi + lo, row 2 = conj(row0 x row1)
__device__ __forceinline__ void load_rebased_df(const float4* __restrict__ hi,
                                                const float4* __restrict__ lo, size_t vh, int i,
                                                Mat3<dfl>& m) {
  float h[12], l[12];
#pragma unroll
  for (int p = 0; p < 3; p++) {
    const float4 a = hi[p * vh + i], b = lo[p * vh + i];
    h[4 * p] = a.x, h[4 * p + 1] = a.y, h[4 * p + 2] = a.z, h[4 * p + 3] = a.w;
    l[4 * p] = b.x, l[4 * p + 1] = b.y, l[4 * p + 2] = b.z, l[4 * p + 3] = b.w;
  }
#pragma unroll
  for (int r = 0; r < 2; r++)
#pragma unroll
    for (int c = 0; c < 3; c++) {
      const int k = 2 * (3 * r + c);
      m.e[r][c] = cmk<dfl>(dfl(h[k], l[k]), dfl(h[k + 1], l[k + 1]));
    }
  row2_from_01(m);
}

// w0(x) = sum_mu U'_mu(x) + U'_mu(x-mu)^+ in double-float, stored split (see kW0Planes)
template <int NDIR>
__global__ void __launch_bounds__(128) rebase_star_kernel(Lattice L, const float4* __restrict__ Ur,
                                                          const float4* __restrict__ Ulo,
                                                          float4* __restrict__ W0) {
  const int parity = blockIdx.y;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= L.vh) return;
  const size_t vh = (size_t)L.vh;
  const Site c = site_of(L, i, parity);
  const int q = 1 - parity;
  Mat3<dfl> w;
  mzero(w);
#pragma unroll
  for (int mu = 0; mu < NDIR; mu++) {
    Mat3<dfl> u;
    const size_t fo = (size_t)(parity * 4 + mu) * 3 * vh, bo = (size_t)(q * 4 + mu) * 3 * vh;
    load_rebased_df(Ur + fo, Ulo + fo, vh, i, u);
#pragma unroll
    for (int r = 0; r < 3; r++)
#pragma unroll
      for (int k = 0; k < 3; k++) w.e[r][k] = cadd(w.e[r][k], u.e[r][k]);
    load_rebased_df(Ur + bo, Ulo + bo, vh, nb_bwd(L, c, mu), u);
#pragma unroll
    for (int r = 0; r < 3; r++)
#pragma unroll
      for (int k = 0; k < 3; k++) w.e[r][k] = cadd(w.e[r][k], cconj(u.e[k][r]));
  }
  // hi: the FP32 star; the remainders (|lo| <= ulp(hi)/2) enter only through their
  // anti-hermitian part and trace
  float f[28];
  Mat3<float> lo;
#pragma unroll
  for (int r = 0; r < 3; r++)
#pragma unroll
    for (int k = 0; k < 3; k++) {
      const int j = 2 * (3 * r + k);
      f[j] = w.e[r][k].re.hi;
      f[j + 1] = w.e[r][k].im.hi;
      lo.e[r][k] = cmk<float>(w.e[r][k].re.lo, w.e[r][k].im.lo);
    }
  f[18] = lo.e[0][0].im;
  f[19] = lo.e[1][1].im;
  f[20] = lo.e[2][2].im;
  f[21] = 0.5f * (lo.e[0][1].re - lo.e[1][0].re);
  f[22] = 0.5f * (lo.e[0][1].im + lo.e[1][0].im);
  f[23] = 0.5f * (lo.e[0][2].re - lo.e[2][0].re);
  f[24] = 0.5f * (lo.e[0][2].im + lo.e[2][0].im);
  f[25] = 0.5f * (lo.e[1][2].re - lo.e[2][1].re);
  f[26] = 0.5f * (lo.e[1][2].im + lo.e[2][1].im);
  f[27] = lo.e[0][0].re + lo.e[1][1].re + lo.e[2][2].re;
  float4* out = W0 + (size_t)parity * kW0Planes * vh + i;
#pragma unroll
  for (int p = 0; p < kW0Planes; p++)
    out[p * vh] = make_float4(f[4 * p], f[4 * p + 1], f[4 * p + 2], f[4 * p + 3]);
}

// g <- normalize((1 + a) g) in FP64, rows 0,1
__global__ void __launch_bounds__(128) compose_g_kernel(Lattice L, double2* __restrict__ G,
                                                        const float4* __restrict__ A) {
  const int parity = blockIdx.y;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= L.vh) return;
  const size_t vh = (size_t)L.vh;
  Mat3<double> gc, gh, g;
  Field<double, 12>::load(G + (size_t)parity * 6 * vh, vh, i, gc);
  Mat3<float> a;
  load12_rows01(A + (size_t)parity * 3 * vh, vh, i, a);
#pragma unroll
  for (int r = 0; r < 2; r++)
#pragma unroll
    for (int k = 0; k < 3; k++)
      gh.e[r][k] = cmk<double>((double)a.e[r][k].re + (r == k ? 1.0 : 0.0), (double)a.e[r][k].im);
#pragma unroll
  for (int r = 0; r < 2; r++)
#pragma unroll
    for (int k = 0; k < 3; k++) g.e[r][k] = mul_entry(gh, gc, r, k);
  normalize<double, false>(g);
  Field<double, 12>::store(G + (size_t)parity * 6 * vh, vh, i, g);
}

// ---------------------------------------------------------------------------
// the FP32 sweep on the rebased fields (device code in gfx_rebased.cuh)
// ---------------------------------------------------------------------------
template <int NDIR>
__global__ void __launch_bounds__(kRebasedBlock, 4) or_rebased_kernel(Lattice L,
                                                                      const float4* __restrict__ Ur,
                                                                      const float4* __restrict__ W0,
                                                                      float4* __restrict__ A,
                                                                      int parity, float omega) {
  // parity 1 in reverse block order: it starts where parity 0 ended (L2 reuse)
  const int blk = parity ? (int)gridDim.x - 1 - (int)blockIdx.x : (int)blockIdx.x;
  const int i = blk * blockDim.x + threadIdx.x;
  if (i >= L.vh) return;
  rebased_site_update<NDIR>(L, site_of(L, i, parity), parity, Ur, W0, A, omega);
}

// functional and theta partials per block, as measure_kernel
template <int NDIR>
__global__ void __launch_bounds__(256) measure_rebased_kernel(Lattice L,
                                                              const float4* __restrict__ Ur,
                                                              const float4* __restrict__ W0,
                                                              const float4* __restrict__ A,
                                                              double* partials) {
  const int parity = blockIdx.y, t = blockIdx.z;  // parity inner, as measure_kernel
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  double f = 0.0, d = 0.0;
  if (k < L.st) {
    const int i = t * L.st + k;
    rebased_site_functional<NDIR>(L, site_of(L, i, parity), parity, Ur, W0, A, f, d);
  }
  const int nbx = gridDim.x;
  block_reduce3(f, d, d, partials + 3 * ((size_t)(parity * L.lt + t) * nbx + blockIdx.x));
}

// ---------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------
size_t rebased_w0_bytes(const Lattice& L) { return (size_t)2 * kW0Planes * 16 * (size_t)L.vh; }

void launch_rebase(int link_nr, int ndir, const Lattice& L, const void* U64, const void* G64,
                   void* Ur, void* Ulo, void* W0, cudaStream_t s) {
  const dim3 g1((L.vh + 127) / 128, 2, ndir);
  if (link_nr == 18)
    rebase_links_kernel<18><<<g1, 128, 0, s>>>(L, (const double2*)U64, (const double2*)G64,
                                                (float4*)Ur, (float4*)Ulo);
  else
    rebase_links_kernel<12><<<g1, 128, 0, s>>>(L, (const double2*)U64, (const double2*)G64,
                                                (float4*)Ur, (float4*)Ulo);
  const dim3 g2((L.vh + 127) / 128, 2);
  if (ndir == 4)
    rebase_star_kernel<4><<<g2, 128, 0, s>>>(L, (const float4*)Ur, (const float4*)Ulo, (float4*)W0);
  else
    rebase_star_kernel<3><<<g2, 128, 0, s>>>(L, (const float4*)Ur, (const float4*)Ulo, (float4*)W0);
}

void launch_compose_g(const Lattice& L, void* G64, const void* A, cudaStream_t s) {
  const dim3 g((L.vh + 127) / 128, 2);
  compose_g_kernel<<<g, 128, 0, s>>>(L, (double2*)G64, (const float4*)A);
}

void launch_or_rebased(int ndir, const Lattice& L, const void* Ur, const void* W0, void* A,
                       int parity, double omega, cudaStream_t s) {
  const dim3 g((L.vh + kRebasedBlock - 1) / kRebasedBlock);
  if (ndir == 4)
    or_rebased_kernel<4><<<g, kRebasedBlock, 0, s>>>(L, (const float4*)Ur, (const float4*)W0,
                                                      (float4*)A, parity, (float)omega);
  else
    or_rebased_kernel<3><<<g, kRebasedBlock, 0, s>>>(L, (const float4*)Ur, (const float4*)W0,
                                                      (float4*)A, parity, (float)omega);
}

void launch_measure_rebased(int ndir, const Lattice& L, const void* Ur, const void* W0,
                            const void* A, double* partials, int block, cudaStream_t s) {
  const dim3 g(measure_blocks_x(L, block), 2, L.lt);
  if (ndir == 4)
    measure_rebased_kernel<4><<<g, block, 0, s>>>(L, (const float4*)Ur, (const float4*)W0,
                                                  (const float4*)A, partials);
  else
    measure_rebased_kernel<3><<<g, block, 0, s>>>(L, (const float4*)Ur, (const float4*)W0,
                                                  (const float4*)A, partials);
}

}  // namespace gfx
