// gfx_internal.h -- host-side declarations shared by the library's translation units.
#pragma once

#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

#include "gfx_device.cuh"

namespace gfx {

// Host construction of the lattice descriptor.
Lattice make_lattice(int lx, int ly, int lz, int lt);

// A start/stop pair of CUDA events that is destroyed on every exit path.
struct EventPair {
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  EventPair() = default;
  EventPair(const EventPair&) = delete;
  EventPair& operator=(const EventPair&) = delete;
  cudaError_t create() {
    cudaError_t e = cudaEventCreate(&e0);
    return e != cudaSuccess ? e : cudaEventCreate(&e1);
  }
  ~EventPair() {
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
  }
};

// Per-check record kept on the device (one per functional evaluation).
struct CheckRecord {
  int iter;
  int phase;  // 0 = single-precision sweeps, 1 = double-precision sweeps
  double F, dAdA, maxdAdA, theta, theta_slice_max;
};

// Device-resident state of a convergence loop.
struct LoopState {
  int iter;       // iteration index of the last check
  int ck;         // sweeps between checks
  int maxit;      // iteration cap (exclusive, as in the reference loop)
  int done;       // 0 running, 1 converged, 2 switch precision, 3 stopped at cap,
                  // 4 below switch_eps: continue with ck_near sweeps between checks,
                  // 5 renew the base of the rebased FP32 sweeps
  int ck_near;    // sweeps between checks once the value is below switch_eps (0: ck)
  int criterion;  // GFX_CRIT_*
  int phase;
  int nhist, hist_cap;
  int rebase_at;  // > 0: done = 5 at the first check with iter >= rebase_at
  double eps;
  double switch_eps;     // phase 0 -> 1 when the monitored value drops below
  double plateau_ratio;  // phase 0 -> 1 when value_new > plateau_ratio * value_old (ck sweeps apart)
  double plateau_near;   // the same threshold for checks ck_near sweeps apart
  double prev;
  double last_F, last_dAdA, last_max, last_theta, last_theta_slice_max;
};

// Reduction results written by the final reduce kernel.
struct Reduced {
  double F, dAdA, maxdAdA, theta, theta_slice_max;
};

// ----- kernel launchers (gfx_kernels.cu) -----
// prec: 0 FP32, 1 FP64, 2 double-float (links 18 reals, g 12 reals, float pairs).
// link_nr arguments give the layout of the link field read: FP32 12 or 8 reals when
// prec == 0, FP64 12 or 18 reals when prec == 1
// mode: 0 plain loads, 1 L2 bulk prefetch per block, 2 plain loads with the blocks of
// parity 1 in reverse order
// wide: the FP32 12-real kernel with its full register set instead of 64 registers
void launch_or_halfsweep(int prec, int link_nr, int ndir, const Lattice& L, const void* U, void* G,
                         int parity, double omega, int block, int mode, cudaStream_t s,
                         int wide = 0);
// measure: compute precision (0 float, 1 double, 2 double-float fields), g storage (0
// float, 1 double, 2 double-float)
void launch_measure(int cprec, int link_nr, int gprec, int ndir, const Lattice& L, const void* U,
                    const void* G, double* partials, int block, cudaStream_t s);
int measure_blocks_x(const Lattice& L, int block);
// sites per measurement block (the grouping of the partial sums)
constexpr int kMeasBlock = 128;
// FP32 checks fused into the last odd half-sweep: possible for 12-real FP32 links when
// every time slice holds whole measurement blocks of each parity
bool fused_check_ok(const Lattice& L, int link_nr32);
// The FP32-phase checks of a mixed-precision solve measure the odd sites only, which
// the fused half-sweep has in registers.  Every link has exactly one odd end, so the
// sum of Re tr X(x) over the odd sites covers each link once: doubled, it is the
// all-site sum and F is exact.  tr[Delta Delta^+] summed over the odd sites and doubled
// estimates the all-site dAdA (and theta); max dAdA is the odd sites' maximum.  These
// checks only steer the FP32 phase (its plateau test and handover); convergence is
// always decided by a full FP64 measurement.
// the odd half-sweep that also writes the odd sites' partials (launch_measure's layout)
void launch_or_halfsweep_measure(int ndir, const Lattice& L, const void* U, void* G, double omega,
                                 int rev, double* partials, cudaStream_t s);
// launch_measure's FP32 blocks of one parity only
void launch_measure_parity(int ndir, const Lattice& L, const void* U, const void* G,
                           double* partials, int parity, cudaStream_t s);
// odd_only: sum the odd sites' partials alone, F and dAdA doubled (FP32-phase checks)
void launch_reduce(const Lattice& L, int ndir, const double* partials, int nbx, double* slice_sums,
                   Reduced* out, LoopState* loop, CheckRecord* hist, int advance,
                   unsigned long long graph_handle, int use_handle, cudaStream_t s,
                   int odd_only = 0);
void launch_plaquette(int link_nr_prec, const Lattice& L, const void* U, double* partials,
                      double* out, cudaStream_t s);
void launch_polyakov(int link_nr_prec, const Lattice& L, const void* U, double* partials,
                     double* out, cudaStream_t s);
void launch_pack_links(int link_nr_prec, const Lattice& L, const double* aos, void* U,
                       cudaStream_t s);
void launch_unpack_links(int link_nr_prec, const Lattice& L, const void* U, double* aos,
                         cudaStream_t s);
void launch_pack_g(int gprec, const Lattice& L, const double* aos, void* G, cudaStream_t s);
// the same by coalesced tiles; aos 16-byte aligned, in device memory or in page-locked
// host memory the device reaches (its device address).  Links: FP64 planes of link_nr
// reals and, when U32 is given, the FP32 12-real copy in the same pass
void launch_pack_links_tiled(int link_nr, const Lattice& L, const void* aos, void* U64, void* U32,
                             cudaStream_t s);
void launch_pack_g_tiled(const Lattice& L, const void* aos, void* G64, cudaStream_t s);
void launch_unpack_g_tiled(const Lattice& L, const void* G64, void* aos, cudaStream_t s);
void launch_unpack_g(int gprec, const Lattice& L, const void* G, double* aos, cudaStream_t s);
// double-float copies of the links (18 reals) and of g (12 reals; to_df = 0 back to FP64)
void launch_convert_links_64_to_df(int link_nr, const Lattice& L, const void* U64, void* Udf,
                                   cudaStream_t s);
void launch_convert_g_df(int to_df, const Lattice& L, void* G64, void* Gdf, cudaStream_t s);
// link_nr32: FP32 layout of the copy, 12 or 8 reals
void launch_convert_links_64_to_32(int link_nr, int link_nr32, const Lattice& L, const void* U64,
                                   void* U32, cudaStream_t s);
void launch_convert_g(int from_prec, int to_prec, const Lattice& L, const void* Gin, void* Gout,
                      cudaStream_t s);
void launch_apply_trafo(int link_nr, const Lattice& L, void* U64, const void* G64, cudaStream_t s);
// ----- rebased FP32 sweeps (gfx_rebased.cu): g = (1 + a) g_c, a in FP32 (G32 layout) -----
// base: Ur = rebased links (FP32 12-real layout), Ulo = their FP32 remainders (same
// size, scratch), W0 = the split star (rebased_w0_bytes); ndir directions
size_t rebased_w0_bytes(const Lattice& L);
void launch_rebase(int link_nr, int ndir, const Lattice& L, const void* U64, const void* G64,
                   void* Ur, void* Ulo, void* W0, cudaStream_t s);
// G64 <- normalize((1 + a) G64) in FP64
void launch_compose_g(const Lattice& L, void* G64, const void* A, cudaStream_t s);
void launch_or_rebased(int ndir, const Lattice& L, const void* Ur, const void* W0, void* A,
                       int parity, double omega, cudaStream_t s);
void launch_measure_rebased(int ndir, const Lattice& L, const void* Ur, const void* W0,
                            const void* A, double* partials, int block, cudaStream_t s);
// Haar-random FP64 g: the value at lexicographic site pos depends only on (seed, pos)
void launch_haar_g(const Lattice& L, double2* G64, unsigned long long seed, cudaStream_t s);

// ----- heatbath family (gfx_heatbath.cu) -----
void launch_sa_heatbath(int prec, int link_nr, const Lattice& L, const void* U, void* G,
                        int parity, double beta, const float* gauss, const float* unif,
                        int block, cudaStream_t s);
void launch_micro(int prec, int link_nr, int ndir, const Lattice& L, const void* U, void* G,
                  int parity, int block, cudaStream_t s);
void launch_link_heatbath(int link_nr, const Lattice& L, void* U, int parity, int nu,
                          double beta3, const float* gauss, const float* unif, int variant,
                          int block, cudaStream_t s);
// the same in FP32 arithmetic from the 12-real FP32 copy U32, updating U and U32
void launch_link_heatbath_f32(int link_nr, const Lattice& L, void* U, void* U32, int parity,
                              int nu, double beta3, const float* gauss, const float* unif,
                              int variant, cudaStream_t s);

// ----- Mersenne Twister bank (gfx_mt.cu) -----
struct MTBank {
  uint32_t* a;       // matrix_a[4096]
  uint32_t* b;       // mask_b[4096]
  uint32_t* c;       // mask_c[4096]
  uint32_t* seed;    // seed[4096]
  uint32_t* status;  // [19][4096]
};
constexpr int kMTCount = 4096;
constexpr int kMTN = 19;
void launch_mt_generate(const MTBank& bank, float* out, int nper, int initialized, int gauss,
                        cudaStream_t s);

}  // namespace gfx
