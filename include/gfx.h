/*
 * gfx.h -- C ABI of libgfx, the sm_103a (GB300) implementation of the cudagfx
 * gauge-fixing hot path.
 *
 * Two layers are exported:
 *   1. gfx_* : explicit-argument, context-handle functions returning gfx_status.
 *   2. the reference's own entry points (init_gaugefixing, overrelax_gauge,
 *      calc_functional, ...) with the reference's global variables, declared in
 *      gfx_legacy.h, so the reference's C host code links against libgfx unchanged.
 *
 * Conventions shared with the reference host code:
 *   - a site is pos = x + LX*(y + LY*(z + LZ*t)) (cudagaugefix.cu:79); directions
 *     mu = 0,1,2,3 = x,y,z,t;
 *   - host matrices are su3 = complex[3][3] of doubles, row-major, (re, im)
 *     interleaved: 18 doubles (global.h:26-33);
 *   - a gauge field is 4*V su3 with link (pos, mu) at index 4*pos+mu; a gauge
 *     transformation is V su3 with g(pos) at index pos.
 * All pointers are host pointers unless the name ends in _device.  No call keeps
 * a host pointer after it returns.
 */
#ifndef GFX_H
#define GFX_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GFX_ABI_VERSION 1

typedef enum {
  GFX_OK = 0,
  GFX_ERR_BAD_VOLUME = 1,    /* extents not even / volume not supported (reference: exit(100)) */
  GFX_ERR_OOM = 2,           /* device allocation failed (reference: exit(200)) */
  GFX_ERR_NOT_CONVERGED = 3, /* iteration cap reached (reference: overrelax_gauge returns -1) */
  GFX_ERR_IO = 4,            /* file missing, truncated or malformed (reference: exit(400)) */
  GFX_ERR_CUDA = 5,          /* a CUDA runtime call failed */
  GFX_ERR_ARG = 6,           /* invalid argument */
  GFX_ERR_STATE = 7          /* call out of order (e.g. update before init) */
} gfx_status;

typedef enum { GFX_PREC_DOUBLE = 0, GFX_PREC_SINGLE = 1, GFX_PREC_MIXED = 2 } gfx_precision;
typedef enum { GFX_GAUGE_LANDAU = 0, GFX_GAUGE_COULOMB = 1 } gfx_gauge;
typedef enum {
  GFX_CRIT_MAXDADA = 0,     /* max_x tr[Delta Delta^+] < eps (the reference criterion, overrelax.cu:794) */
  GFX_CRIT_THETA = 1,       /* theta = (1/3V) sum_x tr[Delta Delta^+] < eps */
  GFX_CRIT_THETA_SLICES = 2 /* max over time slices of theta_t < eps (Coulomb gauge) */
} gfx_criterion;

typedef struct gfx_ctx gfx_ctx;

/* calc_functional's results (overrelax.cu:610-671) plus theta */
typedef struct {
  double F;               /* (1/(ndir V)) sum_{x,mu} Re tr g(x) U_mu(x) g^+(x+mu) */
  double dAdA;            /* (1/V) sum_x tr[Delta Delta^+] */
  double maxdAdA;         /* max_x tr[Delta Delta^+] */
  double theta;           /* dAdA / 3 */
  double theta_slice_max; /* max_t (1/(3 V3)) sum_{x in slice t} tr[Delta Delta^+] */
} gfx_functional_t;

typedef struct {
  int maxit;              /* iteration cap (overrelax_gauge's maxit) */
  double eps;             /* convergence threshold on the criterion */
  int checkinterval;      /* sweeps between functional evaluations */
  double omega;           /* overrelaxation parameter (reference: 1.68, overrelax.cu:416) */
  int criterion;          /* gfx_criterion */
  int gauge;              /* gfx_gauge */
  double switch_eps;      /* mixed: below this the FP32 phase ends when the value stalls */
  double plateau_ratio;   /* mixed: per sweep; stalled = value_new > plateau_ratio^k * value_old
                             for checks k sweeps apart (default 0.998) */
  int checkinterval_double; /* sweeps between checks in the FP64 phase (0: checkinterval) */
  int use_graph;          /* 1: device-side loop in a CUDA graph (conditional while node) */
  int record_history;     /* keep every check (gfx_or_history) */
  int checkinterval_near; /* sweeps between checks once the value is below switch_eps
                             (0: checkinterval throughout, the reference schedule) */
  int polish;             /* mixed: 0 = FP64 sweeps after the handover; 1 = double-float
                             sweeps (pairs of floats, ~48 bits) on the FP32 units; 2 =
                             rebased FP32 sweeps: g = (1 + a) g_c with g_c fixed in FP64
                             and only the small a in FP32, which follow the FP64 sweeps
                             to ~1e-12 at FP32 cost.  The result of 1 and 2 is confirmed
                             by an FP64 measurement (FP64 sweeps continue if it is not).
                             GB300 runs FP32 64x faster than FP64. */
  int fp32_checks_all_sites; /* mixed: 0 (default) = the FP32-phase checks measure the odd
                                sites only when the check is fused into the last odd
                                half-sweep (F exact, dAdA and theta estimated as twice the
                                odd sites' sums); 1 = every site.  They only steer the FP32
                                phase; convergence is decided by an FP64 measurement. */
} gfx_or_params;

typedef struct {
  int iterations;     /* overrelax_gauge's return value: iteration of the converging check, or -1 */
  int sweeps;         /* sweeps performed */
  int sweeps_single;  /* of which in FP32 */
  int sweeps_double;  /* of which in FP64 */
  int converged;
  int checks;         /* functional evaluations */
  gfx_functional_t final_values; /* last evaluation (FP64 unless precision is SINGLE) */
  double ms;          /* device time of the whole call (CUDA events) */
  int sweeps_polish_df; /* of sweeps_double, those run in double-float (polish = 1) */
  int sweeps_polish_fp32; /* of sweeps_double, those run as rebased FP32 (polish = 2) */
} gfx_or_result;

typedef struct {
  int iter;
  int phase; /* 0: FP32 sweeps, 1: FP64 (or final) sweeps */
  double F, dAdA, maxdAdA, theta, theta_slice_max;
} gfx_check_record;

/* SAPARAM_LIST (global.h:51-57) plus the number of microcanonical sweeps per step */
typedef struct {
  double Tmin, Tmax, expo;
  int N;
  int checkint;
  int nmicro;
} gfx_sa_params;

typedef struct {
  int Nsweep;
  int checkint;
  double beta;
  int variant; /* GFX_HB_REFERENCE or GFX_HB_KENNEDY_PENDLETON */
  int precision; /* 0: FP64 arithmetic (the reference's); 1: FP32 staples and SU(2)
                    steps from the FP32 link copy, each new link reunitarized in
                    double-float (unitary to ~1e-14) and stored in FP64 and FP32
                    (SINGLE or MIXED contexts; the same distribution, on the FP32
                    units) */
} gfx_therm_params;

/* Link-heatbath variants.  REFERENCE reproduces the reference's update
 * (heatbath_thermalization.cu:493-550 with simulated_annealing.cu:5-142: one trial
 * with k = |w|^2, the same random numbers for all three subgroups, alpha = w on
 * rejection).  KENNEDY_PENDLETON samples the Wilson-action distribution at beta
 * (k = |w|, independent numbers per subgroup, no update on rejection). */
enum { GFX_HB_REFERENCE = 0, GFX_HB_KENNEDY_PENDLETON = 1 };

/* ---- library / context ---- */
int gfx_abi_version(void);
const char *gfx_status_string(int status);
/* last error message of this context (or the global one when ctx is NULL) */
const char *gfx_last_error(const gfx_ctx *ctx);

/* cudaSetDevice for C callers that do not link the CUDA runtime themselves
 * (the reference's main selects its card with -d, cudagaugefix.cu:628-661) */
gfx_status gfx_set_device(int device);

/* Create a context on the current device.  link_reals64 = 12 (two-row storage,
 * the reference layout) or 18 (full matrices) for the FP64 link copy.
 * stream = a cudaStream_t to run on, or NULL for a private stream. */
gfx_status gfx_create(gfx_ctx **out, int lx, int ly, int lz, int lt, int precision,
                      int link_reals64, void *stream);
gfx_status gfx_destroy(gfx_ctx *ctx);
gfx_status gfx_synchronize(gfx_ctx *ctx);
/* bytes of device memory held by the context */
size_t gfx_device_bytes(const gfx_ctx *ctx);
/* threads per block of the sweep kernels (0: library default / autotuned) */
gfx_status gfx_set_block(gfx_ctx *ctx, int block);

/* ---- launch tuning (no reference counterpart: the reference hard-codes 128
 *      threads per block, cudaglobal.h:8) ----
 * Settings of the overrelaxation half-sweep per precision, [0] = FP32 storage,
 * [1] = FP64.  block: threads per block (a multiple of 32 in [32, 256]).
 * staging: 0 = plain 128-bit loads; 1 = each block first issues one L2 bulk
 * prefetch (cp.async.bulk.prefetch.L2) per contiguous range it reads; 2 = plain
 * loads, and the odd half-sweep runs its blocks in reverse order, so that it starts
 * on the ranges the even half-sweep touched last (still in L2); 3 = as 2, with the
 * FP32 12-real sweep reading and writing g with the L2 eviction priority evict_last;
 * 4 = as 3, and its links read as evict_first (other sweeps: 3 and 4 act as 2).  A
 * new context starts with 2, and with 4 for its FP32 sweep when the FP32 g fits in
 * half the L2 but g and the links together do not fit in it.  All settings give bit-identical results.
 * link_reals64: FP64 link storage, 12 (two rows) or 18 (full).  link_reals32: the
 * FP32 copy the FP32 sweeps read, 12 or 8.  The 8-real form rebuilds rows 1, 2
 * dividing by |U_01|^2 + |U_02|^2; the few links where that is below 1e-2 are read
 * from exact rows kept beside it, so every link is accurate to FP32 rounding and
 * 32 bytes per link are read.  The FP64 links stay exact: the 8-real copy changes
 * FP32 sweeps at rounding level only; all other settings give bit-identical results.
 * checkinterval: sweeps per convergence check the tuner suggests for the FP32
 * phase (0 = no suggestion).  sweep_ms / check_ms: the tuner's timings of one full
 * sweep and of one check at the chosen settings (0 when set by hand). */
typedef struct {
  int block[2];
  int staging[2];
  int link_reals64;
  int link_reals32; /* FP32 link copy: 12, or 8 (the GF_8 parameters a2, a3, arg a1,
                       arg c1, b1, dev_su3.cu:428-728); 0 = keep */
  int checkinterval;
  double sweep_ms[2];
  double check_ms[2];
  int wide_regs; /* FP32 half-sweep kernel: 0 capped at 64 registers (32 warps per SM), 1
                    its full register set (~124; 16 warps per SM, more loads in flight per
                    warp); the results are bit-identical */
} gfx_tuning;

gfx_status gfx_get_tuning(const gfx_ctx *ctx, gfx_tuning *out);
/* Apply settings (block, staging, link_reals64; the timings are ignored).  A
 * change of link_reals64 re-packs the FP64 links on the device. */
gfx_status gfx_set_tuning(gfx_ctx *ctx, const gfx_tuning *t);
/* Time every candidate setting on this context's lattice and apply the fastest.
 * Candidates: block 64/128/192/256 x staging 0/1/2 (0-4 for FP32) for each precision the
 * context holds (x both register budgets for FP32), and both link layouts of each
 * precision.  The fields are left as they
 * were: the candidate sweeps run on g and it is restored afterwards.
 * expected_sweeps > 0 also sets checkinterval to the interval that minimises
 * check time plus the sweeps run past convergence, sqrt(2 n check_ms / sweep_ms),
 * clamped to [5, 100].  cache_path (or NULL): a text file of earlier results keyed
 * by device, lattice, precision mode and gauge; a hit applies the stored settings
 * without timing, a miss appends the new result. */
gfx_status gfx_autotune(gfx_ctx *ctx, int gauge, int expected_sweeps, const char *cache_path,
                        gfx_tuning *out);

/* ---- fields (init_gaugefixing / gfx_get_trafo of the reference's main, cudagaugefix.cu:204-374, 785-793) ---- */
gfx_status gfx_set_links(gfx_ctx *ctx, const double *su3_links);
gfx_status gfx_get_links(gfx_ctx *ctx, double *su3_links);
gfx_status gfx_set_trafo(gfx_ctx *ctx, const double *su3_trafo);
gfx_status gfx_get_trafo(gfx_ctx *ctx, double *su3_trafo);
/* g <- 1 */
gfx_status gfx_unit_trafo(gfx_ctx *ctx);

/* ---- gauge fixing ---- */
void gfx_or_params_default(gfx_or_params *p);
/* overrelax_gauge (overrelax.cu:677-823) */
gfx_status gfx_overrelax(gfx_ctx *ctx, const gfx_or_params *p, gfx_or_result *res);
/* copy up to cap check records of the last gfx_overrelax call; returns the count */
int gfx_or_history(const gfx_ctx *ctx, gfx_check_record *out, int cap);
/* nsweeps plain OR sweeps (even then odd) without checks; precision 0 = FP32, 1 = FP64,
 * 2 = double-float (the polish sweeps of gfx_or_params.polish = 1), 3 = rebased FP32 (the
 * polish sweeps of polish = 2; a base is taken from the current g unless the last call
 * left one for the same gauge and links) */
gfx_status gfx_or_sweeps(gfx_ctx *ctx, int nsweeps, double omega, int gauge, int precision);
/* one OR half-sweep of one parity */
gfx_status gfx_or_halfsweep(gfx_ctx *ctx, int parity, double omega, int gauge, int precision);
/* calc_functional (overrelax.cu:610-671); precision 0 = FP32 arithmetic, 1 = FP64,
 * 3 = rebased FP32 (the checks of polish = 2) */
gfx_status gfx_functional(gfx_ctx *ctx, int gauge, int precision, gfx_functional_t *out);
/* calc_plaquette (overrelax.cu:115-138) on the links */
gfx_status gfx_plaquette(gfx_ctx *ctx, double *plaq);
/* Polyakov loop (1/V3) sum_xvec tr prod_t U_t / 3 -> re_im[2] */
gfx_status gfx_polyakov(gfx_ctx *ctx, double *re_im);
/* U_mu(x) <- g(x) U_mu(x) g^+(x+mu) on the device, then g <- 1
 * (dev_apply_trafo overrelax.cu:273-331 / g_trafo observables.c:17-47) */
gfx_status gfx_apply_trafo(gfx_ctx *ctx);

/* No counterpart in the reference.  The functional and theta (gfx_functional_t layout,
 * written to result_device: 5 doubles in device memory) of fields the caller already
 * holds in device memory, for callers that cannot allocate device memory while they
 * run -- a framework that owns every device byte through its own pool, or a service
 * with a device footprint fixed at start-up.  Nothing is allocated: the reduction
 * scratch is a fixed file-scope device array (about 0.8 MB per device, held until the
 * process exits) with room for lt <= 1024 time slices; larger lt returns GFX_ERR_ARG.
 * links_device: FP64 links in the library's even/odd layout (link_reals 12 or 18
 * doubles per link, as a context stores them); trafo_device: FP64 12-real g in the
 * same layout; stream: a cudaStream_t or NULL.  The first call in a CUDA context looks
 * up the scratch array's address (make it before any stream capture); a new context on
 * the device (e.g. after cudaDeviceReset) is detected and gets a new lookup.  gauge must
 * be GFX_GAUGE_LANDAU or GFX_GAUGE_COULOMB (else GFX_ERR_ARG).  If a CUDA error from
 * earlier work is pending, the call returns GFX_ERR_STATE and leaves that error for the
 * caller.  All calls on a device share the array; calls that overlap on the GPU race.
 * Asynchronous on stream. */
gfx_status gfx_functional_noalloc(const void *links_device, const void *trafo_device, int lx,
                                  int ly, int lz, int lt, int link_reals, int gauge,
                                  double *result_device, void *stream);

/* device times (ms) of the last gfx_set_links, gfx_set_trafo and gfx_get_trafo: ms[2k]
 * the host<->device copy, ms[2k+1] the layout kernels; direct[k] = 1 when the GPU read
 * or wrote the caller's gfx_host_alloc buffer itself (no copy) */
gfx_status gfx_transfer_times(const gfx_ctx *ctx, double *ms, int *direct);
/* FP32 convergence checks fused into the last odd half-sweep before the check (1, the
 * default; used when the FP32 links hold 12 reals and each time slice holds whole
 * 128-site blocks of each parity) or a separate measurement (0); the check values are
 * bit-identical */
gfx_status gfx_set_fused_check(gfx_ctx *ctx, int fused);
/* device time (CUDA events on the context's stream) of nsweeps plain OR sweeps, run
 * as one CUDA graph (back to back, as in gfx_overrelax's device loop) */
gfx_status gfx_time_sweeps(gfx_ctx *ctx, int nsweeps, double omega, int gauge, int precision,
                           double *ms);
/* number of kernels this context has enqueued (graph bodies counted per execution) */
unsigned long long gfx_launch_count(const gfx_ctx *ctx);

/* ---- Mersenne Twister bank (MersenneTwister.cu / .h) ---- */
/* params: 4096 records {matrix_a, mask_b, mask_c, seed}, the MersenneTwister.dat layout */
gfx_status gfx_mt_load_params(gfx_ctx *ctx, const uint32_t *params);
gfx_status gfx_mt_load_file(gfx_ctx *ctx, const char *path);
/* seedMTGPU with srand(mtseed): seed_i = i-th rand() (MersenneTwister.cu:98-114) */
gfx_status gfx_mt_seed(gfx_ctx *ctx, unsigned int mtseed);
gfx_status gfx_mt_set_seeds(gfx_ctx *ctx, const uint32_t *seeds);
/* init_MT (MersenneTwister.cu:236-289) */
gfx_status gfx_mt_init(gfx_ctx *ctx, int n_gauss, int n_unif);
/* update_MT (MersenneTwister.cu:295-323) */
gfx_status gfx_mt_update(gfx_ctx *ctx);
/* read the current fields (sizes 4096*nper) and, optionally, the state [19][4096] and seeds[4096] */
gfx_status gfx_mt_read(gfx_ctx *ctx, float *gauss, float *unif, uint32_t *state, uint32_t *seeds);
gfx_status gfx_mt_sizes(const gfx_ctx *ctx, int *nper_gauss, int *nper_unif);

/* ---- simulated annealing (simulated_annealing.cu) ---- */
/* set_sa_temperature (simulated_annealing.cu:265-299) */
double gfx_sa_temperature(const gfx_sa_params *p, int i);
/* simannealing_gauge (simulated_annealing.cu:309-476), plus p->nmicro microcanonical
 * sweeps per heatbath step; needs an initialized MT bank */
gfx_status gfx_simanneal(gfx_ctx *ctx, const gfx_sa_params *p, gfx_functional_t *last);
/* steps first .. first+count-1 of the schedule (for callers that check in between) */
gfx_status gfx_simanneal_range(gfx_ctx *ctx, const gfx_sa_params *p, int first, int count);
/* single half-sweeps with the current random fields */
gfx_status gfx_sa_halfsweep(gfx_ctx *ctx, int parity, double beta, int precision);
gfx_status gfx_micro_halfsweep(gfx_ctx *ctx, int parity, int gauge, int precision);

/* ---- thermalization (heatbath_thermalization.cu) ---- */
/* thermalize_gauge (heatbath_thermalization.cu:568-841): Nsweep x 4 directions x 2 parities,
 * beta/3 per set_beta; plaquette every checkint sweeps into plaq (if non-NULL, capacity
 * Nsweep/checkint + 1).  The result stays on the device (gfx_get_links). */
gfx_status gfx_thermalize(gfx_ctx *ctx, const gfx_therm_params *p, double *plaq, int plaq_cap);
gfx_status gfx_link_heatbath_halfsweep(gfx_ctx *ctx, int parity, int nu, double beta,
                                       int variant);

/* ---- batched Gribov copies (no counterpart in the reference: its main fixes one
 * copy per run, cudagaugefix.cu:706-821) ---- */
typedef struct gfx_batch gfx_batch;

typedef struct {
  int conf, copy;
  int converged;
  int iterations;     /* as overrelax_gauge: converging check's iteration, or -1 */
  int sweeps, sweeps_single, sweeps_double;
  double F, dAdA, maxdAdA, theta, theta_slice_max;
} gfx_copy_result;

/* nconf configurations with extents dims[4*c..4*c+3] and ncopies[c] gauge copies each
 * (at most 8 configurations) */
gfx_status gfx_batch_create(gfx_batch **out, int nconf, const int *dims, const int *ncopies,
                            int precision, void *stream);
gfx_status gfx_batch_destroy(gfx_batch *b);
const char *gfx_batch_last_error(const gfx_batch *b);
int gfx_batch_copies(const gfx_batch *b);
/* FP32 sweeps with two copies of a configuration per thread in packed FP32 arithmetic
 * (1) or one copy per thread (0, the default: on GB300 the two-copy kernel issues 46%
 * fewer instructions but, at twice the registers, runs 9% slower); the results are
 * bit-identical */
gfx_status gfx_batch_set_paired(gfx_batch *b, int paired);
gfx_status gfx_batch_set_links(gfx_batch *b, int conf, const double *su3_links);
gfx_status gfx_batch_set_trafo(gfx_batch *b, int conf, int copy, const double *su3_trafo);
gfx_status gfx_batch_get_trafo(gfx_batch *b, int conf, int copy, double *su3_trafo);
/* Haar-random start for every copy: copy k of configuration c (global index
 * copy_base(c) + k) uses seed + global index (same generator as gfx_random_trafo_haar) */
gfx_status gfx_batch_random_haar(gfx_batch *b, uint64_t seed);
/* Haar-random start of one copy from its own seed (a replica that holds a share of a
 * larger set of copies seeds each copy by its index in the whole set) */
gfx_status gfx_batch_random_haar_copy(gfx_batch *b, int conf, int copy, uint64_t seed);
/* fix every copy (one device loop for the whole batch); results[gfx_batch_copies()].
 * Every copy follows exactly the trajectory of gfx_overrelax on a single context with
 * the same parameters, except that the batch uses checkinterval throughout
 * (checkinterval_near is ignored) and polish = 1 polishes with FP64 sweeps as
 * polish = 0 does (polish = 2, the rebased FP32 sweeps, is supported). */
gfx_status gfx_batch_overrelax(gfx_batch *b, const gfx_or_params *p, gfx_copy_result *results,
                               double *ms);
/* the converged copy of configuration conf with the largest functional */
gfx_status gfx_batch_best(gfx_batch *b, const gfx_copy_result *results, int conf,
                          int *best_copy, double *best_F);
/* Haar-random g on the device, g(site) from a counter-based stream of (seed, site) */
gfx_status gfx_random_trafo_haar(gfx_ctx *ctx, uint64_t seed);

/* ---- host-side helpers ---- */
/* page-locked host memory for the field copies (cudaMallocHost); NULL on failure */
/* Page-locked host memory.  Field arrays in it (gfx_set_links, gfx_set_trafo,
 * gfx_get_trafo) are read or written by the GPU directly, with no staging copy. */
void *gfx_host_alloc(size_t bytes);
void gfx_host_free(void *p);
/* glibc srand(seed)/rand() stream */
void gfx_glibc_rand(unsigned int seed, int n, int32_t *out);
/* random_init_trafo / random_init_gauge with Park-Miller PlantSeeds(seed) (su3manip.c:539-767) */
void gfx_random_init_reference(long seed, double *su3, long n);
/* Haar-distributed SU(3) matrices from a seeded counter-based generator */
void gfx_random_init_haar(uint64_t seed, double *su3, long n);
/* unit matrices */
void gfx_unit_init(double *su3, long n);

#ifdef __cplusplus
}
#endif
#endif
