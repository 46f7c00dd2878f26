"""Generate tests/golden/reference_fixtures.npz by running the reference's own CUDA code.

Run on a machine with a GPU after `python oracle/ref_gpu.py` has prepared and built
oracle/_ref/libref_gpu.so from the reference checkout:

    python tests/golden/make_reference_fixtures.py <out.npz>

Scenarios (inputs are regenerated by the tests from the seeds below; the link arrays'
SHA-256 is stored to detect any drift of the generator):
  A  4^4: the reference's random start (RandSeed 351), OR half-sweeps even, odd, then
     10 more sweeps -> g after each; functional and plaquette.
  B  8^4: overrelax_gauge(3000, 1e-10, 10) -> converging iteration, FUNC, DADA, maxDADA.
  C  twister bank: init_MT(V/2, 2V) for 8^4 with srand(1234), then 2 update_MT ->
     SHA-256 and the first 512 values of each field, the field sizes.
  D  4^4: init_MT(V/2, 2V) with srand(7), SA half-sweep even at beta 1/1.45, update_MT,
     odd at beta 1/0.3 -> g after each; the fields used.
  E  4^4: simannealing_gauge(Tmin 0.01, Tmax 1.45, expo -1, N 20, checkint 5) from the
     scenario-A start with srand(7) -> FUNC, DADA, maxDADA.

With --workloads it writes tests/golden/reference_workloads.npz instead: the
8^4 gauge-fixing workload and the annealing statistics on realistic links.  The
links come from this repository's own heatbath (libgfx, built on the same
machine), and the fixture stores their SHA-256 so the tests can check that they
regenerate the same links:
  C1  8^4, beta 6.0, 200 heatbath sweeps from a cold start, MT seed 1234, twister
      fields 2V gauss + 8V uniform, the reference's heatbath update (C1R) and the
      Kennedy-Pendleton update (C1K); the reference's random start (RandSeed 351).
      For each: (a) the reference's kernels at omega 1.7 with a theta = DADA/3 < 1e-12
      stop, checked every 10 sweeps (the loop of overrelax_gauge with theta as the
      criterion) -> converging iteration, FUNC, DADA, maxDADA; (b) the reference's
      own overrelax_gauge(5000, 1e-10, 10) at its omega 1.68 (maxdAdA criterion).
  SA  8^4 C1K links, the reference's random start, 16 twister seeds (3001..3016):
      init_MT(V/2, 2V), simannealing_gauge(Tmin 0.01, Tmax 1.45, expo -1, N 300,
      checkint 300) -> FUNC, DADA, maxDADA per seed.
"""
import ctypes as c
import hashlib
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests"))

from golden_inputs import links_for  # noqa: E402

_dp = c.POINTER(c.c_double)
_fp = c.POINTER(c.c_float)


def _p(a, t=c.c_double):
    return a.ctypes.data_as(c.POINTER(t))


def sha(a):
    return np.frombuffer(hashlib.sha256(np.ascontiguousarray(a).tobytes()).digest(),
                         dtype=np.uint8)


def main(out):
    from oracle import ref_gpu
    ref_gpu.prepare()
    lib = c.CDLL(ref_gpu.build())
    lib.ref_calc_plaquette.restype = c.c_double
    lib.ref_calc_functional.restype = c.c_double
    lib.ref_overrelax.restype = c.c_int
    lib.ref_random_init_trafo.argtypes = [c.c_long, c.c_int, _dp]
    lib.ref_sa_halfsweep.argtypes = [c.c_int, c.c_double]
    lib.ref_overrelax.argtypes = [c.c_int, c.c_double, c.c_int]
    lib.ref_init_mt.argtypes = [c.c_char_p, c.c_uint, c.c_int, c.c_int]
    lib.ref_simanneal.argtypes = [c.c_double, c.c_double, c.c_double, c.c_int, c.c_int]
    datdir = os.fsencode(ref_gpu.REF_DIR)
    fx = {}

    def start(dims, link_seed, trafo_seed=351):
        V = int(np.prod(dims))
        u = links_for(dims, link_seed)
        g = np.empty((V, 18))
        lib.ref_random_init_trafo(trafo_seed, V, _p(g))
        assert lib.ref_setup(*dims, _p(u), _p(g)) == 0
        return u, g

    def trafo(V):
        g = np.empty((V, 18))
        lib.ref_get_trafo(_p(g))
        return g[:, :12].copy()

    # A
    dims = (4, 4, 4, 4)
    u, g0 = start(dims, 101)
    fx["A_links_sha"] = sha(u)
    fx["A_g0"] = g0[:, :12].copy()
    lib.ref_or_halfsweep(0)
    fx["A_g_even"] = trafo(256)
    lib.ref_or_halfsweep(1)
    fx["A_g_sweep1"] = trafo(256)
    for _ in range(10):
        lib.ref_or_halfsweep(0)
        lib.ref_or_halfsweep(1)
    fx["A_g_sweep11"] = trafo(256)
    f3 = np.zeros(3)
    lib.ref_calc_functional(_p(f3))
    fx["A_functional"] = f3.copy()
    fx["A_plaquette"] = np.array([lib.ref_calc_plaquette()])
    lib.ref_finalize()

    # B
    dims = (8, 8, 8, 8)
    u, g0 = start(dims, 202)
    fx["B_links_sha"] = sha(u)
    it = lib.ref_overrelax(3000, 1e-10, 10)
    lib.ref_calc_functional(_p(f3))
    fx["B_result"] = np.array([it, f3[0], f3[1], f3[2]])
    lib.ref_finalize()

    # C
    u, g0 = start(dims, 202)
    V = 4096
    assert lib.ref_init_mt(datdir, 1234, V // 2, 2 * V) == 0
    ng, nu = c.c_int(), c.c_int()
    lib.ref_mt_sizes(c.byref(ng), c.byref(nu))
    fx["C_nper"] = np.array([ng.value, nu.value])
    for step in range(3):
        gs = np.empty(4096 * ng.value, dtype=np.float32)
        us = np.empty(4096 * nu.value, dtype=np.float32)
        lib.ref_read_rng(_p(gs, c.c_float), _p(us, c.c_float))
        fx["C_gauss_sha_%d" % step] = sha(gs)
        fx["C_unif_sha_%d" % step] = sha(us)
        fx["C_gauss_head_%d" % step] = gs[:512].copy()
        fx["C_unif_head_%d" % step] = us[:512].copy()
        lib.ref_update_mt()
    lib.ref_finalize()

    # D
    dims = (4, 4, 4, 4)
    u, g0 = start(dims, 101)
    assert lib.ref_init_mt(datdir, 7, 128, 512) == 0
    lib.ref_mt_sizes(c.byref(ng), c.byref(nu))
    for k, (parity, beta) in enumerate(((0, 1.0 / 1.45), (1, 1.0 / 0.3))):
        gs = np.empty(4096 * ng.value, dtype=np.float32)
        us = np.empty(4096 * nu.value, dtype=np.float32)
        lib.ref_read_rng(_p(gs, c.c_float), _p(us, c.c_float))
        fx["D_gauss_%d" % k] = gs[:128].copy()
        fx["D_unif_%d" % k] = us[:512].copy()
        lib.ref_sa_halfsweep(parity, beta)
        fx["D_g_%d" % k] = trafo(256)
        lib.ref_update_mt()
    lib.ref_finalize()

    # E
    u, g0 = start(dims, 101)
    assert lib.ref_init_mt(datdir, 7, 128, 512) == 0
    lib.ref_simanneal(0.01, 1.45, -1.0, 20, 5)
    lib.ref_calc_functional(_p(f3))
    fx["E_functional"] = f3.copy()
    lib.ref_finalize()

    np.savez_compressed(out, **fx)
    print("wrote", out, sorted(fx))


C1_DIMS = (8, 8, 8, 8)
C1_OMEGA, C1_EPS, C1_CK = 1.7, 1e-12, 10
SA_SEEDS = list(range(3001, 3017))
SA_PARAMS = dict(Tmin=0.01, Tmax=1.45, expo=-1.0, N=300, checkint=300)


def c1_links(gfx, variant, mt_dat):
    """The C1 links from this repository's heatbath: 8^4, beta 6.0, 200 sweeps from a
    cold start, MT seed 1234, fields 2V gauss + 8V uniform."""
    V = int(np.prod(C1_DIMS))
    c = gfx.Context(C1_DIMS)
    c.set_links(gfx.unit_init(4 * V))
    c.mt_load_file(mt_dat)
    c.mt_seed(1234)
    c.mt_init(2 * V, 8 * V)
    c.thermalize(6.0, 200, variant=variant)
    u = np.ascontiguousarray(c.get_links())
    c.close()
    return u


def workloads(out):
    import cudagfx_gb300 as gfx
    from oracle import ref_gpu
    ref_gpu.prepare()
    lib = c.CDLL(ref_gpu.build())
    lib.ref_calc_functional.restype = c.c_double
    lib.ref_overrelax.restype = c.c_int
    lib.ref_overrelax.argtypes = [c.c_int, c.c_double, c.c_int]
    lib.ref_random_init_trafo.argtypes = [c.c_long, c.c_int, _dp]
    lib.ref_init_mt.argtypes = [c.c_char_p, c.c_uint, c.c_int, c.c_int]
    lib.ref_simanneal.argtypes = [c.c_double, c.c_double, c.c_double, c.c_int, c.c_int]
    lib.ref_set_omega.argtypes = [c.c_double]
    datdir = os.fsencode(ref_gpu.REF_DIR)
    mt_dat = os.path.join(ref_gpu.REF_DIR, "MersenneTwister.dat")
    V = int(np.prod(C1_DIMS))
    fx = {}

    def setup(u):
        g = np.empty((V, 18))
        lib.ref_random_init_trafo(351, V, _p(g))
        assert lib.ref_setup(*C1_DIMS, _p(u), _p(g)) == 0

    f3 = np.zeros(3)
    for tag, variant in (("C1R", gfx.HB_REFERENCE), ("C1K", gfx.HB_KENNEDY_PENDLETON)):
        u = c1_links(gfx, variant, mt_dat)
        fx[tag + "_links_sha"] = sha(u)
        # (a) omega 1.7, theta < 1e-12, as overrelax_gauge's loop (overrelax.cu:710-805)
        setup(u)
        assert lib.ref_set_omega(C1_OMEGA) == 0
        it = -1
        for i in range(20000):
            lib.ref_or_halfsweep(0)
            lib.ref_or_halfsweep(1)
            if i % C1_CK == 0:
                lib.ref_calc_functional(_p(f3))
                if f3[1] / 3.0 < C1_EPS:
                    it = i
                    break
        fx[tag + "_theta"] = np.array([it, f3[0], f3[1], f3[2]])
        assert lib.ref_set_omega(1.68) == 0
        lib.ref_finalize()
        # (b) the reference's own loop at its own omega and criterion
        setup(u)
        it = lib.ref_overrelax(5000, 1e-10, 10)
        lib.ref_calc_functional(_p(f3))
        fx[tag + "_stock"] = np.array([it, f3[0], f3[1], f3[2]])
        lib.ref_finalize()
        if tag == "C1K":
            sa = []
            for seed in SA_SEEDS:
                setup(u)
                assert lib.ref_init_mt(datdir, seed, V // 2, 2 * V) == 0
                lib.ref_simanneal(SA_PARAMS["Tmin"], SA_PARAMS["Tmax"], SA_PARAMS["expo"],
                                  SA_PARAMS["N"], SA_PARAMS["checkint"])
                lib.ref_calc_functional(_p(f3))
                sa.append(f3.copy())
                lib.ref_finalize()
            fx["SA_seeds"] = np.array(SA_SEEDS)
            fx["SA_results"] = np.array(sa)
    np.savez_compressed(out, **fx)
    print("wrote", out, {k: v for k, v in fx.items() if not k.endswith("sha")})


if __name__ == "__main__":
    here = os.path.dirname(__file__)
    args = [a for a in sys.argv[1:] if a != "--workloads"]
    if "--workloads" in sys.argv:
        workloads(args[0] if args else os.path.join(here, "reference_workloads.npz"))
    else:
        main(args[0] if args else os.path.join(here, "reference_fixtures.npz"))
