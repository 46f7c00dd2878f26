#!/usr/bin/env python3
"""Benchmark: Landau gauge fixing of a 32^4 SU(3) lattice on one GB300.

One step = one complete gauge-fixing solve: the mixed-precision checkerboard
overrelaxation (FP32 12-real sweeps with FP64-accumulated checks, then polish
sweeps -- by default rebased FP32 sweeps, g = (1 + a) g_c with only the small a in
FP32) from the same random gauge start until theta = (1/3V) sum tr[DD^+] < 1e-12,
verified in FP64.  The links (beta = 6.0, heatbath-thermalized on the GPU
from a cold start) and the starting transformation are generated once before the
timed region.

  value : OR site updates per second over the K timed steps, inputs resident in HBM
  e2e   : the same metric through the public C ABI with host buffers -- H2D of
          the links and the start transformation from pinned memory, the solve,
          D2H of the gauge transformation -- every step
  time_to_theta_s : mixed vs all-FP64 solve of the same problem

`--impl reference` times the CPU restatement of the reference's OR update (the
reference has no CPU overrelaxation; its observables are host C) on all host
cores, on a bounded sample of sweeps of the same lattice.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "OR site-updates/s & time to θ<1e-12 (32^4 Landau), mixed vs FP64 on 1 GB300"
UNIT = "site-updates/s"
# algorithmic bytes of one OR site update, FP32 12-real storage: 8 links (96 reals)
# + g of this parity read and written (24) + g of the other parity read once (12)
BYTES_PER_UPDATE_FP32 = 132 * 4
BYTES_PER_UPDATE_FP64 = 132 * 8
FLOP_PER_UPDATE = 4766  # the reference's count (overrelax.cu:897)
# DRAM bytes per FP32 half-sweep launch at 32^4 (dram__bytes_read.sum +
# dram__bytes_write.sum) in the alternating sweep with warm L2, per staging mode, from
# the --cache-control none captures in profiles/or_halfsweep_fp32_32x4.md
NCU_TRAFFIC_FP32 = {((32, 32, 32, 32), 2): 198.4e6 + 27.2e6,
                    ((32, 32, 32, 32), 4): 185.3e6 + 6.7e6}


POLISH_NAMES = {0: "FP64", 1: "double-float (FP32 pairs), FP64-confirmed",
                2: "rebased FP32 (g = (1 + a) g_c, a in FP32), FP64-confirmed"}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gfx", choices=["gfx", "reference"])
    ap.add_argument("--dims", default="32,32,32,32")
    ap.add_argument("--therm", type=int, default=200, help="heatbath sweeps for the links")
    ap.add_argument("--beta", type=float, default=6.0)
    ap.add_argument("--eps", type=float, default=1e-12)
    ap.add_argument("--omega", type=float, default=1.7)
    ap.add_argument("--checkinterval", type=int, default=0,
                    help="sweeps per check (0: the autotuner's choice)")
    ap.add_argument("--switch-eps", type=float, default=1e-10)
    ap.add_argument("--checkinterval-double", type=int, default=2)
    ap.add_argument("--checkinterval-near", type=int, default=10,
                    help="sweeps per check once theta < switch-eps (0: off)")
    ap.add_argument("--no-fp64", action="store_true", help="skip the all-FP64 comparison")
    ap.add_argument("--no-tune", action="store_true", help="library default launch settings")
    ap.add_argument("--polish", type=int, default=2, choices=[0, 1, 2],
                    help="sweeps after the FP32 phase: 0 FP64, 1 double-float, 2 rebased FP32")
    ap.add_argument("--no-graph", action="store_true",
                    help="host-driven check loop instead of the CUDA-graph while loop (same "
                         "kernels; profilers list each launch)")
    ap.add_argument("--cpu-sweeps", type=int, default=0, help="CPU sample sweeps (0: auto)")
    ap.add_argument("--no-gribov", action="store_true",
                    help="skip the batched-Gribov-copies measurement")
    ap.add_argument("--gribov-copies", default="64,32",
                    help="copies of the 16^4 (beta 6.0) and 24^4 (beta 6.2) configurations")
    ap.add_argument("--gribov-paired", action="store_true",
                    help="batched FP32 sweeps with two copies per thread (packed FP32)")
    ap.add_argument("--batch-only", action="store_true",
                    help="Gribov copies: one warm-up and one timed batched solve, without the "
                         "other sweep kernel and the sequential arms (for profiler captures)")
    ap.add_argument("--config", choices=["c1", "c2", "c3", "c4", "c5"], default=None,
                    help="instead of the bench: one full workload, mixed against all-FP64 "
                         "(--no-fp64 skips that solve): c1 8^4 (also on the CPU oracle), c2 "
                         "16^3x32 SA then OR, c3 32^4 Coulomb, c4 the batched Gribov copies "
                         "alone, c5 48^3x96")
    ap.add_argument("--staging", type=int, default=2, choices=[0, 1, 2, 3, 4],
                    help="--kernels: OR half-sweep staging mode")
    ap.add_argument("--kernels", action="store_true",
                    help="no timing: a few launches of each hot kernel on the lattice, for "
                         "ncu captures")
    return ap.parse_args()


def split_copies(ncopies, rank, ws):
    """The Gribov copies rank `rank` of `ws` fixes: copies r, r + ws, r + 2 ws, ... of
    every configuration (indices within the configuration).  Copies are independent,
    so the replicas share no data during the solve."""
    return [list(range(rank, n, ws)) for n in ncopies]


def gather_best(dist, ws, local):
    """local[k] = (F, copy) of this rank's best converged copy of configuration k, or
    None; returns the best over all ranks (largest F, then the lower copy index)."""
    if dist is None or ws == 1:
        return list(local)
    every = [None] * ws
    dist.all_gather_object(every, list(local))
    best = []
    for k in range(len(local)):
        cand = [r[k] for r in every if r[k] is not None]
        best.append(max(cand, key=lambda fc: (fc[0], -fc[1])) if cand else None)
    return best


def sum_over_ranks(dist, x):
    if dist is None:
        return x
    import torch
    t = torch.tensor([float(x)], dtype=torch.float64, device=_coll_device())
    dist.all_reduce(t)
    return float(t.item())


def gribov_batch(args, gfx, mt_source, rank=0, ws=1, dist=None):
    """Batched Gribov copies: 64 copies of a 16^4 beta=6.0 configuration and 32 copies of
    a 24^4 beta=6.2 configuration, Haar-random starts (seed 2024 + copy), mixed OR
    omega=1.7 (FP32, then the --polish sweeps; double-float is not batched and falls
    back to FP64) to theta<1e-12, the largest-functional copy kept per configuration.
    Batched: one device loop for all copies.  Sequential: the same starts, one
    single-lattice solve per copy.  Both timed with CUDA events (solve only).  Under
    N ranks each rank fixes copies r, r + N, ... (split_copies); the times are the
    slowest rank's and the best copy is gathered over the ranks."""
    confs = [((16, 16, 16, 16), 6.0), ((24, 24, 24, 24), 6.2)]
    ncopies = [int(x) for x in args.gribov_copies.split(",")]
    mine = split_copies(ncopies, rank, ws)
    kw = dict(maxit=20000, eps=args.eps, checkinterval=args.checkinterval or 25, omega=args.omega,
              criterion=gfx.CRIT_THETA, switch_eps=args.switch_eps,
              checkinterval_double=args.checkinterval_double,
              polish=2 if args.polish == 2 else 0, use_graph=0 if args.no_graph else 1)
    links = []
    for k, (d, beta) in enumerate(confs):
        V = int(np.prod(d))
        c = gfx.Context(d)
        c.set_links(gfx.unit_init(4 * V))
        mt_source(c)
        c.mt_seed(100 + k)
        c.mt_init(2 * V, 8 * V)
        c.thermalize(beta, args.therm, variant=gfx.HB_KENNEDY_PENDLETON)
        links.append(c.get_links())
        c.close()
    base = [sum(ncopies[:k]) for k in range(len(confs))]
    held = [k for k in range(len(confs)) if mine[k]]
    b = gfx.Batch([confs[k][0] for k in held], [len(mine[k]) for k in held],
                  precision=gfx.PREC_MIXED)

    def starts():
        for bi, k in enumerate(held):
            for j, copy in enumerate(mine[k]):
                b.random_haar_copy(bi, j, 2024 + base[k] + copy)

    for bi, k in enumerate(held):
        b.set_links(bi, links[k])
    # the other FP32 sweep kernel first, for comparison: two copies per thread (packed
    # FP32) unless --gribov-paired makes that the measured one
    ms_b1 = None
    if not args.batch_only:
        b.set_paired(0 if args.gribov_paired else 1)
        starts()
        b.overrelax(**kw)  # warm-up (graph instantiation)
        starts()
        _, ms_b1 = b.overrelax(**kw)
    b.set_paired(1 if args.gribov_paired else 0)
    starts()
    b.overrelax(**kw)
    starts()
    res, ms_b = b.overrelax(**kw)
    local_best = [None] * len(confs)
    for bi, k in enumerate(held):
        j, f = b.best(bi)
        if j >= 0:
            local_best[k] = (f, mine[k][j])
    upd = sum(r["sweeps"] * int(np.prod(confs[held[r["conf"]]][0])) for r in res)
    b.close()
    if args.batch_only:
        ms_b, upd = max_over_ranks(dist, ms_b), sum_over_ranks(dist, upd)
        return {"workload": "%d x 16^4 (beta 6.0) + %d x 24^4 (beta 6.2) Gribov copies, Haar "
                            "starts, theta<%g, batched solve only" % (ncopies[0], ncopies[1], args.eps),
                "batched_s": ms_b / 1000.0, "batched_site_updates_per_s": upd / (ms_b / 1000.0),
                "converged": int(sum_over_ranks(dist, sum(r["converged"] for r in res)))}
    # sequential arms: the single-lattice solver per copy, (a) its device loop captured
    # in a CUDA graph (the strict comparison), (b) launched kernel by kernel with a host
    # check every checkinterval sweeps, the structure of the reference's overrelax_gauge
    ms_s, upd_s, ms_l = 0.0, 0, 0.0
    kw_l = dict(kw, use_graph=0)
    for k in held:
        d = confs[k][0]
        c = gfx.Context(d, precision=gfx.PREC_MIXED)
        c.set_links(links[k])
        c.random_trafo_haar(2024 + base[k] + mine[k][0])
        c.overrelax(**kw)  # warm-up
        for copy in mine[k]:
            c.random_trafo_haar(2024 + base[k] + copy)
            r = c.overrelax(**kw)
            ms_s += r.ms
            upd_s += r.sweeps * int(np.prod(d))
            c.random_trafo_haar(2024 + base[k] + copy)
            ms_l += c.overrelax(**kw_l).ms
        c.close()
    best = gather_best(dist, ws, local_best)
    ms_b, ms_s = max_over_ranks(dist, ms_b), max_over_ranks(dist, ms_s)
    ms_b1, ms_l = max_over_ranks(dist, ms_b1), max_over_ranks(dist, ms_l)
    upd, upd_s = sum_over_ranks(dist, upd), sum_over_ranks(dist, upd_s)
    conv = sum_over_ranks(dist, sum(r["converged"] for r in res))
    return {"workload": "%d x 16^4 (beta 6.0) + %d x 24^4 (beta 6.2) Gribov copies, Haar starts, "
                        "theta<%g" % (ncopies[0], ncopies[1], args.eps),
            "polish": POLISH_NAMES[kw["polish"]],
            "replicas": ws, "converged": int(conv), "copies": int(sum(ncopies)),
            "copies_per_thread": 2 if args.gribov_paired else 1,
            "batched_s": ms_b / 1000.0, "sequential_s": ms_s / 1000.0,
            "batched_other_kernel_s": ms_b1 / 1000.0,
            "batched_site_updates_per_s": upd / (ms_b / 1000.0),
            "sequential_site_updates_per_s": upd_s / (ms_s / 1000.0),
            "throughput_ratio": (upd / (ms_b / 1000.0)) / (upd_s / (ms_s / 1000.0)),
            "sequential_launched_s": ms_l / 1000.0,
            "throughput_ratio_vs_launched": (upd / (ms_b / 1000.0)) / (upd_s / (ms_l / 1000.0)),
            "best_copy": [{"copy": fc[1], "F": fc[0]} if fc else None for fc in best]}


def run_kernels(args, dims):
    """A short fixed workload for profiler captures: 3 FP32 OR sweeps, an FP32 and an
    FP64 functional, 31 sweeps of the FP32 convergence loop with a check every 10 (the
    fused check), 1 FP64 OR sweep, 3 rebased FP32 sweeps and their functional, one
    SA step with one microcanonical step, one link-heatbath sweep in FP64 and one in
    FP32 arithmetic, the plaquette and the Polyakov loop.  The OR sweeps use --staging
    (2, the odd half-sweep in reverse block order, unless given)."""
    import cudagfx_gb300 as gfx
    V = int(np.prod(dims))
    ctx = gfx.Context(dims, precision=gfx.PREC_MIXED)
    t = ctx.tuning()
    ctx.set_tuning(block=t["block"], staging=(args.staging, args.staging))
    ctx.set_links(gfx.random_init_haar(11, 4 * V))
    ctx.set_trafo(gfx.random_init_reference(351, V))
    ctx.or_sweeps(3, omega=args.omega, precision=0)
    ctx.functional(precision=0)
    ctx.functional(precision=1)
    # a few FP32 checks of the convergence loop, host-driven so that each launch is
    # visible to a profiler: the fused odd half-sweep and the even-site measurement
    ctx.overrelax(maxit=31, eps=1e-30, checkinterval=10, omega=args.omega,
                  criterion=gfx.CRIT_THETA, switch_eps=1e-40, use_graph=0)
    ctx.or_sweeps(1, omega=args.omega, precision=1)
    ctx.or_sweeps(3, omega=args.omega, precision=3)
    ctx.functional(precision=3)
    dat = mt_params_path()
    if dat:
        ctx.mt_load_file(dat)
    else:
        ctx.mt_load_params(synthetic_mt_params())
    ctx.mt_seed(42)
    ctx.mt_init(2 * V, 8 * V)
    ctx.simanneal(0.5, 0.5, 1, nmicro=1)
    ctx.thermalize(args.beta, 1, variant=gfx.HB_KENNEDY_PENDLETON)
    ctx.thermalize(args.beta, 1, variant=gfx.HB_KENNEDY_PENDLETON, precision=1)
    ctx.plaquette()
    ctx.polyakov()
    ctx.close()
    print("kernels ok")


# ---------------------------------------------------------------------------
class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.idx = gpu_index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.idx), "--query-gpu=" + self.FIELDS,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            p = [x.strip() for x in ln.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                mx.append(float(p[2]))
            except ValueError:
                continue
            for n, v in zip(names, p[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx),
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return d.get("hbm_gbs", 6800.0), "measured"
    return 6800.0, "fallback"


def mt_params_path():
    for p in (os.environ.get("GFX_MT_DAT"), os.path.join(os.getcwd(), "MersenneTwister.dat"),
              os.path.join(ROOT, "oracle", "_ref", "MersenneTwister.dat")):
        if p and os.path.exists(p):
            return p
    return None


def synthetic_mt_params(seed=4172):
    rng = np.random.default_rng(seed)
    p = rng.integers(0, 2 ** 32, size=(4096, 4), dtype=np.uint64).astype(np.uint32)
    p[:, 0] |= np.uint32(0x80000000)
    p[:, 3] = 0
    return p


# ---------------------------------------------------------------------------
class nvtx_range:
    """An NVTX range (named in profiler launch lists) when torch provides NVTX."""

    def __init__(self, name):
        self.name = name
        self.nvtx = None

    def __enter__(self):
        try:
            import torch
            self.nvtx = torch.cuda.nvtx
            self.nvtx.range_push(self.name)
        except Exception:  # noqa: BLE001  (no NVTX: the range is only a label)
            self.nvtx = None
        return self

    def __exit__(self, *exc):
        if self.nvtx is not None:
            self.nvtx.range_pop()
        return False


def dist_init(args):
    """torchrun ranks: NCCL between GPUs, gloo when no GPU is present (tests)."""
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    if ws <= 1:
        return 0, 1, 0, None
    import torch
    import torch.distributed as dist
    rank = int(os.environ["RANK"])
    local = int(os.environ.get("LOCAL_RANK", rank))
    if torch.cuda.is_available():
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    else:
        dist.init_process_group("gloo")
    return rank, ws, local, dist


def _coll_device():
    import torch
    return "cuda" if torch.cuda.is_available() else "cpu"


def barrier(dist):
    if dist is not None:
        import torch
        t = torch.zeros(1, device=_coll_device())
        dist.all_reduce(t)
        if t.is_cuda:
            torch.cuda.synchronize()


def max_over_ranks(dist, x):
    if dist is None:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64, device=_coll_device())
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_inputs(rank):
    """Each rank fixes its own configuration: heatbath seed and gauge-start seed."""
    return {"mt_seed": 42 + rank, "trafo_seed": 351 + rank}


def cpu_reference_rate(dims, links, g0, sweeps, omega):
    """The oracle's C port of the reference's OR update (overrelax.cu:149-446), built
    for speed (-O3, FMA contraction allowed), OpenMP over one parity on all host
    threads: `sweeps` sweeps of the given links from the start g0.  Returns site
    updates per second, the seconds and the thread count."""
    import oracle as orc
    o = orc.Oracle(fast=True)
    lat = o.lattice(dims)
    V = int(np.prod(dims))
    gf12 = o.to2v(links)
    g = np.ascontiguousarray(np.asarray(g0).reshape(-1, 18)[:, :12])
    o.or_halfsweep(lat, gf12, g, 0, omega)  # warm the threads
    t0 = time.perf_counter()
    o.or_sweeps(lat, gf12, g, sweeps, omega)
    dt = time.perf_counter() - t0
    return sweeps * V / dt, dt, os.cpu_count()


CPU_SWEEPS = 10  # per sample: a bounded share of the solve's ~4500 sweeps


def _have_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except ImportError:
        return False


def bench_inputs(gfx, dims, beta, therm, mt_seed, trafo_seed):
    """The solve's inputs: Kennedy-Pendleton heatbath links (cold start, `therm`
    sweeps, on the GPU) and the reference's random gauge start."""
    V = int(np.prod(dims))
    ctx = gfx.Context(dims, precision=gfx.PREC_MIXED)
    ctx.set_links(gfx.unit_init(4 * V))
    dat = mt_params_path()
    if dat:
        ctx.mt_load_file(dat)
    else:
        ctx.mt_load_params(synthetic_mt_params())
    ctx.mt_seed(mt_seed)
    ctx.mt_init(2 * V, 8 * V)
    t0 = time.perf_counter()
    ctx.thermalize(beta, therm, variant=gfx.HB_KENNEDY_PENDLETON)
    ctx.synchronize()
    therm_s = time.perf_counter() - t0
    plaq = ctx.plaquette()
    links = ctx.get_links()
    g0 = gfx.random_init_reference(trafo_seed, V)
    return ctx, links, g0, plaq, therm_s, dat


# ---------------------------------------------------------------------------
def run_reference(args, dims):
    """The reference arm: the CPU port of the reference's OR update on the bench's own
    inputs (the heatbath links and random start, made on the GPU before any timing),
    all host threads, CPU_SWEEPS sweeps per step."""
    rank, ws, local, dist = dist_init(args)
    if rank != 0:
        return
    from cudagfx_gb300 import build as b
    b.build()
    import cudagfx_gb300 as gfx
    seeds = replica_inputs(rank)
    V = int(np.prod(dims))
    if _have_gpu():
        ctx, links, g0, plaq, _, _ = bench_inputs(gfx, dims, args.beta, args.therm,
                                                  seeds["mt_seed"], seeds["trafo_seed"])
        ctx.close()
        link_kind = "the bench's beta=%g heatbath links" % args.beta
    else:
        # no GPU to make the heatbath links (a CPU-only check of this arm): Haar-random
        # links; the update's cost does not depend on the values
        links, plaq = gfx.random_init_haar(11, 4 * V), None
        g0 = gfx.random_init_reference(seeds["trafo_seed"], V)
        link_kind = "Haar-random links (no GPU for the heatbath)"
    sweeps = args.cpu_sweeps or CPU_SWEEPS
    for _ in range(max(0, min(args.warmup, 1))):
        cpu_reference_rate(dims, links, g0, 1, args.omega)
    rates, tot, cores = [], 0.0, os.cpu_count()
    for _ in range(args.steps):
        r, dt, cores = cpu_reference_rate(dims, links, g0, sweeps, args.omega)
        rates.append(r)
        tot += dt
    value = float(np.mean(rates))
    out = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000 * tot / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic", "impl": "reference",
        "config": {"workload": "%s Landau OR sweeps (omega=%g) of %s from the reference "
                               "random start, CPU port of the reference update, all host "
                               "threads" % ("x".join(map(str, dims)), args.omega, link_kind),
                   "lattice": list(dims), "sweeps_per_step": sweeps, "plaquette": plaq},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": "%d OR sweeps of %s per step (gcc -O3, FMA contraction), "
                                   "OpenMP over one parity" % (sweeps, "x".join(map(str, dims)))},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(out), flush=True)


def run_gfx(args, dims):
    rank, ws, local, dist = dist_init(args)
    from cudagfx_gb300 import build as b
    if rank == 0:
        b.build()
    barrier(dist)
    import cudagfx_gb300 as gfx

    V = int(np.prod(dims))
    # ---- inputs: heatbath links (beta, cold start), reference random gauge start
    seeds = replica_inputs(rank)
    ctx, links, g0, plaq, therm_s, dat = bench_inputs(gfx, dims, args.beta, args.therm,
                                                      seeds["mt_seed"], seeds["trafo_seed"])

    def mt_source(c):
        if dat:
            c.mt_load_file(dat)
        else:
            c.mt_load_params(synthetic_mt_params())

    def make_params(ck):
        return ctx.or_params(maxit=20000, eps=args.eps, checkinterval=ck, omega=args.omega,
                             criterion=gfx.CRIT_THETA, switch_eps=args.switch_eps,
                             checkinterval_double=args.checkinterval_double,
                             checkinterval_near=args.checkinterval_near,
                             polish=args.polish,
                             use_graph=0 if args.no_graph else 1)

    def solve(c, p):
        c.set_trafo(g0)
        r = c.overrelax(p)
        if not r.converged:
            raise RuntimeError("did not converge: %d sweeps" % r.sweeps)
        return r

    # ---- launch tuning (before any timing): the first warm-up solve gives the sweep
    # count the check interval is chosen for
    params = make_params(args.checkinterval or 25)
    r_w = solve(ctx, params)
    tune = None
    if not args.no_tune:
        tune = ctx.autotune(gfx.LANDAU, expected_sweeps=r_w.sweeps_single)
    if args.checkinterval == 0 and tune:
        params = make_params(tune["checkinterval"])
    for _ in range(args.warmup):
        solve(ctx, params)
    # ---- timed region: K solves, device time of each (CUDA events on the ctx stream)
    barrier(dist)
    launches0 = ctx.launch_count()
    with ClockSampler(local) as clk, nvtx_range("timed_solves"):
        results = [solve(ctx, params) for _ in range(args.steps)]
    launches = ctx.launch_count() - launches0
    ms_total = sum(r.ms for r in results)
    ms_total = max_over_ranks(dist, ms_total)
    updates = sum(r.sweeps for r in results) * V
    value = updates * ws / (ms_total / 1000.0)
    r_last = results[-1]
    clocks = clk.summary()

    # ---- e2e through the public API with pinned host buffers
    pin_links = gfx.pinned_empty(links.shape)
    pin_links[...] = links
    pin_g0 = gfx.pinned_empty(g0.shape)
    pin_g0[...] = g0
    pin_out = gfx.pinned_empty(g0.shape)
    e2e_t, e2e_upd, e2e_dev = 0.0, 0, 0.0
    parts = {"set_links": 0.0, "set_trafo": 0.0, "overrelax": 0.0, "get_trafo": 0.0}
    dev_parts = {k + s: 0.0 for k in ("set_links", "set_trafo", "get_trafo")
                 for s in ("_copy", "_layout")}
    io_direct = {}
    for _ in range(args.steps):
        ctx.synchronize()
        t0 = time.perf_counter()
        ctx.set_links(pin_links)
        t1 = time.perf_counter()
        ctx.set_trafo(pin_g0)
        t2 = time.perf_counter()
        r = ctx.overrelax(params)
        t3 = time.perf_counter()
        ctx.get_trafo_into(pin_out)
        t4 = time.perf_counter()
        e2e_t += t4 - t0
        e2e_upd += r.sweeps * V
        e2e_dev += r.ms / 1000.0
        io = ctx.transfer_times()
        for k, (cp, lay, direct) in io.items():
            dev_parts[k + "_copy"] += cp / 1000.0
            dev_parts[k + "_layout"] += lay / 1000.0
            io_direct[k] = direct
        # each call returns after its work on the device is done
        parts["set_links"] += t1 - t0
        parts["set_trafo"] += t2 - t1
        parts["overrelax"] += t3 - t2
        parts["get_trafo"] += t4 - t3
    e2e_t = max_over_ranks(dist, e2e_t)
    e2e_value = e2e_upd * ws / e2e_t

    # ---- kernel timing for the roofline (FP32 and FP64 half-sweeps)
    ctx.set_trafo(g0)
    nt = 20
    ms32 = ctx.time_sweeps(nt, args.omega, precision=0) / (2 * nt)
    ms64 = None
    t_fp64 = None
    sweeps64 = None
    tune64 = None
    if not args.no_fp64:
        c64 = gfx.Context(dims, precision=gfx.PREC_DOUBLE)
        c64.set_links(links)
        c64.set_trafo(g0)
        p64 = params
        if not args.no_tune:
            # the all-FP64 run gets its own tuning (FP64 link layout, check interval)
            tune64 = c64.autotune(gfx.LANDAU, expected_sweeps=r_last.sweeps)
            if args.checkinterval == 0:
                p64 = make_params(tune64["checkinterval"])
        ms64 = c64.time_sweeps(4, args.omega, precision=1) / 8
        r64 = solve(c64, p64)
        t_fp64 = r64.ms / 1000.0
        sweeps64 = r64.sweeps
        fv64 = r64.final_values
        c64.close()
    hbm, peak_kind = measured_peaks()
    t32_share = r_last.sweeps_single * 2 * ms32
    t64_share = r_last.sweeps_double * 2 * (ms64 if ms64 else 0.0)
    bytes32 = BYTES_PER_UPDATE_FP32 * V / 2
    ach32 = bytes32 / (ms32 / 1000.0) / 1e9
    staging32 = ctx.tuning()["staging"][0]
    roof = {"bound": "hbm", "kernel": "or_halfsweep_kernel<float,12,4>",
            "achieved": ach32, "peak": hbm, "unit": "GB/s", "frac": ach32 / hbm,
            "peak_source": peak_kind, "staging": staging32,
            "traffic": NCU_TRAFFIC_FP32.get((tuple(dims), staging32)), "ms_per_launch": ms32,
            "bytes_per_launch": bytes32,
            "time_share_in_solve": t32_share / max(r_last.ms, 1e-9)}
    if ms64:
        nr64 = tune64["link_reals64"] if tune64 else 12
        roof["fp64_kernel"] = {"kernel": "or_halfsweep_kernel<double,%d,4>" % nr64,
                               "ms_per_launch": ms64,
                               "gflops": FLOP_PER_UPDATE * V / 2 / (ms64 / 1000.0) / 1e9,
                               "time_share_in_solve": t64_share / max(r_last.ms, 1e-9)}

    cpu = None
    if rank == 0:
        cs = args.cpu_sweeps or CPU_SWEEPS
        rate, dt, cores = cpu_reference_rate(dims, links, g0, cs, args.omega)
        cpu = {"value": rate, "unit": UNIT, "cores": cores, "kind": "port",
               "sample": "%d OR sweeps of %s (%.1f s) on the bench's heatbath links from the "
                         "reference start, CPU port of the reference update (gcc -O3, FMA "
                         "contraction), OpenMP over one parity"
                         % (cs, "x".join(map(str, dims)), dt)}
    ctx.close()
    gribov = None if args.no_gribov else gribov_batch(args, gfx, mt_source, rank, ws, dist)
    if rank != 0:
        return
    h2d = pin_links.nbytes + pin_g0.nbytes
    out = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_total / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic",
        "config": {
            "workload": "%s Landau gauge fixing: beta=%g Kennedy-Pendleton heatbath links (%d "
                        "sweeps from cold, MT seed 42), reference random gauge start (RandSeed "
                        "351), mixed FP32->FP64 "
                        "OR omega=%g to theta<%g" % ("x".join(map(str, dims)), args.beta,
                                                     args.therm, args.omega, args.eps),
            "lattice": list(dims), "omega": args.omega, "eps": args.eps, "criterion": "theta",
            "checkinterval": params.checkinterval,
            "checkinterval_double": params.checkinterval_double,
            "checkinterval_near": params.checkinterval_near,
            "polish": POLISH_NAMES[args.polish],
            "tuning": tune, "tuning_fp64": tune64,
            "parallelism": "replicas" if ws > 1 else "1 GPU",
            "l2": "inputs larger than L2 (FP32 links %d MB, FP64 links %d MB)"
                  % (V * 4 * 48 // 2 ** 20, V * 4 * 96 // 2 ** 20),
            "mt_params": "reference file" if dat else "synthetic stand-in",
            "plaquette": plaq, "therm_s": therm_s},
        "sweeps_per_solve": {"total": r_last.sweeps, "fp32": r_last.sweeps_single,
                             "polish": r_last.sweeps_double,
                             "polish_double_float": r_last.sweeps_polish_df,
                             "polish_rebased_fp32": r_last.sweeps_polish_fp32},
        "time_to_theta_s": {"mixed": r_last.ms / 1000.0, "fp64": t_fp64,
                            "fp64_sweeps": sweeps64,
                            "speedup": (t_fp64 / (r_last.ms / 1000.0)) if t_fp64 else None,
                            # both measured in FP64 at the end of their solves
                            "theta_mixed": r_last.final_values.theta,
                            "maxdAdA_mixed": r_last.final_values.maxdAdA,  # the reference's criterion
                            "theta_fp64": fv64.theta if t_fp64 else None,
                            "F_mixed_minus_fp64": (r_last.final_values.F - fv64.F) if t_fp64
                            else None},
        "roofline": roof,
        "cpu_baseline": cpu,
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": pin_out.nbytes,
                # wall time per step, and the solve's device time within it
                "s_per_step": e2e_t / args.steps, "solve_device_s_per_step": e2e_dev / args.steps,
                # wall seconds per step of each public call (host-timed; every call
                # synchronizes before it returns); overrelax_host_s = its wall time
                # outside the device-timed solve
                "breakdown_s": dict({k: v / args.steps for k, v in parts.items()},
                                    overrelax_host_s=(parts["overrelax"] - e2e_dev) / args.steps),
                # CUDA-event times per step of the transfers' copies and layout kernels
                # (copy 0: the GPU reads / writes the page-locked host arrays directly)
                "device_breakdown_s": {k: v / args.steps for k, v in dev_parts.items()},
                "direct_host_access": io_direct},
        "clocks": clocks,
        "gpu_launches": int(launches),
        "gribov_batch": gribov,
    }
    print(json.dumps(out), flush=True)


def run_config_small(args):
    """c1  8^4 beta 6.0, links from the reference's heatbath (200 sweeps from cold, MT
        seed 1234), reference random gauge start (RandSeed 351), Landau OR omega 1.7
        to theta < 1e-12: mixed and all-FP64 on the GPU, and as the CPU baseline the
        oracle's FP64 port of the reference loop on the host cores (checks every 100
        sweeps);
    c2  16^3x32 beta 6.0 (500 KP heatbath sweeps, MT seed 7): SA 2000 steps T 1.45 ->
        0.01 (linear) with 3 microcanonical steps each on FP32 g, then OR omega 1.7 to
        theta < 1e-12, mixed against all-FP64 from the same annealed g."""
    import cudagfx_gb300 as gfx
    from cudagfx_gb300 import build as b
    b.build()
    c1 = args.config == "c1"
    dims = (8, 8, 8, 8) if c1 else (16, 16, 16, 32)
    V = int(np.prod(dims))
    out = {"config": args.config, "lattice": list(dims)}
    c = gfx.Context(dims, precision=gfx.PREC_MIXED)
    c.set_links(gfx.unit_init(4 * V))
    dat = mt_params_path()
    c.mt_load_file(dat) if dat else c.mt_load_params(synthetic_mt_params())
    c.mt_seed(1234 if c1 else 7)
    c.mt_init(2 * V, 8 * V)
    c.thermalize(6.0, 200 if c1 else 500,
                 variant=gfx.HB_REFERENCE if c1 else gfx.HB_KENNEDY_PENDLETON)
    out["plaquette"] = c.plaquette()
    links = c.get_links()
    c.set_trafo(gfx.random_init_reference(351, V))
    if not c1:
        c.synchronize()
        t0 = time.perf_counter()
        c.simanneal(0.01, 1.45, 2000, expo=-1.0, checkint=2000, nmicro=3)
        c.synchronize()
        out["simanneal_s"] = time.perf_counter() - t0
    g_start = c.get_trafo()
    kw = dict(maxit=20000, eps=1e-12, checkinterval=100 if c1 else 50, omega=1.7,
              criterion=gfx.CRIT_THETA)
    # one untimed solve first: the first launches of a process load the kernels
    c.overrelax(polish=2, **kw)
    c.set_trafo(g_start)
    r = c.overrelax(polish=2, **kw)
    f = c.functional()
    out["mixed"] = {"s": r.ms / 1000.0, "converged": r.converged, "sweeps_fp32": r.sweeps_single,
                    "sweeps_polish": r.sweeps_double, "theta": f.theta, "F": f.F}
    c.close()
    if not args.no_fp64:
        d = gfx.Context(dims, precision=gfx.PREC_DOUBLE)
        d.set_links(links)
        d.set_trafo(g_start)
        d.overrelax(**kw)
        d.set_trafo(g_start)
        r64 = d.overrelax(**kw)
        f64 = d.functional()
        out["fp64"] = {"s": r64.ms / 1000.0, "converged": r64.converged, "iterations": r64.iterations,
                       "sweeps": r64.sweeps, "theta": f64.theta, "F": f64.F}
        out["F_mixed_minus_fp64"] = f.F - f64.F
        d.close()
    if c1:
        import oracle as orc
        o = orc.Oracle()
        lat = o.lattice(dims)
        gf12, g12 = o.to2v(links), np.ascontiguousarray(np.asarray(g_start).reshape(-1, 18)[:, :12])
        t0 = time.perf_counter()
        it = 0
        o.or_sweeps(lat, gf12, g12, 1, 1.7)
        fo = o.functional(lat, gf12, g12)
        while fo["dAdA"] / 3.0 >= kw["eps"] and it < kw["maxit"]:
            o.or_sweeps(lat, gf12, g12, kw["checkinterval"], 1.7)
            it += kw["checkinterval"]
            fo = o.functional(lat, gf12, g12)
        # the CPU baseline of this workload: the oracle's port of the reference update
        out["cpu_baseline"] = {"kind": "port", "s": time.perf_counter() - t0, "iterations": it,
                               "theta": fo["dAdA"] / 3.0, "F": fo["F"],
                               "cores": os.cpu_count()}
    print(json.dumps(out))


def run_config(args):
    """The full C3 or C5 workload on one GPU, one JSON line:
    c3  32^4 beta 6.0 (200 FP64 KP heatbath sweeps from cold, MT seed 42), Coulomb
        gauge from the reference random start (RandSeed 351) to theta_t < 1e-15 per
        slice, mixed (rebased polish) against all-FP64, plaquette and Polyakov loop
        before and after fixing;
    c5  48^3x96 beta 6.2, FP64 18-real links: 1000 FP32-arithmetic KP heatbath sweeps
        from cold (MT seed 2024), SA 1000 steps T 1.0 -> 0.01 with 3 microcanonical
        steps each, then Landau OR omega 1.7 to theta < 1e-14, mixed (rebased polish)
        against all-FP64 from the same annealed g."""
    import cudagfx_gb300 as gfx
    from cudagfx_gb300 import build as b
    b.build()
    c5 = args.config == "c5"
    dims = (48, 48, 48, 96) if c5 else (32, 32, 32, 32)
    V = int(np.prod(dims))
    out = {"config": args.config, "lattice": list(dims)}

    def now(c):
        c.synchronize()
        return time.perf_counter()

    c = gfx.Context(dims, precision=gfx.PREC_MIXED, link_reals=18 if c5 else 12)
    c.set_links(gfx.unit_init(4 * V))
    dat = mt_params_path()
    c.mt_load_file(dat) if dat else c.mt_load_params(synthetic_mt_params())
    c.mt_seed(2024 if c5 else 42)
    c.mt_init(2 * V, 8 * V)
    t0 = now(c)
    c.thermalize(6.2 if c5 else 6.0, 1000 if c5 else 200, variant=gfx.HB_KENNEDY_PENDLETON,
                 precision=1 if c5 else 0)
    out["thermalize_s"] = now(c) - t0
    plaq0, poly0 = c.plaquette(), c.polyakov()
    out["plaquette"] = plaq0
    c.set_trafo(gfx.random_init_reference(351, V))
    if c5:
        t0 = now(c)
        c.simanneal(0.01, 1.0, 1000, expo=-1.0, checkint=1000, nmicro=3)
        out["simanneal_s"] = now(c) - t0
        kw = dict(maxit=20000, eps=1e-14, checkinterval=100, omega=1.7,
                  criterion=gfx.CRIT_THETA, checkinterval_near=10)
        gauge = gfx.LANDAU
    else:
        kw = dict(maxit=20000, eps=1e-15, checkinterval=50, omega=1.7, gauge=gfx.COULOMB,
                  criterion=gfx.CRIT_THETA_SLICES)
        gauge = gfx.COULOMB
    g_start = c.get_trafo()
    r = c.overrelax(polish=2, **kw)
    f = c.functional(gauge=gauge)
    out["mixed"] = {"s": r.ms / 1000.0, "converged": r.converged, "sweeps_fp32": r.sweeps_single,
                    "sweeps_polish": r.sweeps_double, "theta": f.theta,
                    "theta_slice_max": f.theta_slice_max, "F": f.F}
    g_mixed = c.get_trafo()
    links = c.get_links() if not args.no_fp64 else None
    c.apply_trafo()
    out["plaquette_rel_change"] = abs(c.plaquette() - plaq0) / plaq0
    out["polyakov_abs_change"] = abs(c.polyakov() - poly0)
    c.close()
    if not args.no_fp64:
        d = gfx.Context(dims, precision=gfx.PREC_DOUBLE, link_reals=18 if c5 else 12)
        d.set_links(links)
        d.set_trafo(g_start)
        r64 = d.overrelax(**kw)
        f64 = d.functional(gauge=gauge)
        out["fp64"] = {"s": r64.ms / 1000.0, "converged": r64.converged, "sweeps": r64.sweeps,
                       "theta": f64.theta, "theta_slice_max": f64.theta_slice_max, "F": f64.F}
        out["speedup"] = r64.ms / r.ms
        out["F_mixed_minus_fp64"] = f.F - f64.F
        out["max_abs_g_diff"] = float(np.max(np.abs(g_mixed - d.get_trafo())))
        d.close()
    print(json.dumps(out))


def run_config_c4(args):
    """c4  the batched Gribov copies alone (gribov_batch), one JSON line"""
    from cudagfx_gb300 import build as b
    b.build()
    import cudagfx_gb300 as gfx
    dat = mt_params_path()

    def mt_source(c):
        if dat:
            c.mt_load_file(dat)
        else:
            c.mt_load_params(synthetic_mt_params())

    print(json.dumps(gribov_batch(args, gfx, mt_source)))


def main():
    args = parse()
    dims = tuple(int(x) for x in args.dims.split(","))
    if args.config in ("c1", "c2"):
        run_config_small(args)
    elif args.config == "c4":
        run_config_c4(args)
    elif args.config:
        run_config(args)
    elif args.kernels:
        run_kernels(args, dims)
    elif args.impl == "reference":
        run_reference(args, dims)
    else:
        run_gfx(args, dims)


if __name__ == "__main__":
    main()
