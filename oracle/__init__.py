"""ctypes front end of the CPU oracle (test infrastructure only).

``Oracle``: the restatement in gfx_oracle.c (liboracle.so).
``RefHost``: the reference's own host C files built into _ref/libref_host.so
(observables.c, su3manip.c, rngs.c, complex.c), when the reference checkout was
present at build time.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use this.
"""
import ctypes as c
import os

import numpy as np

from . import build as _build

HERE = os.path.dirname(os.path.abspath(__file__))
DAT_PATH = _build.REF_DAT

_dp = c.POINTER(c.c_double)
_fp = c.POINTER(c.c_float)
_ip = c.POINTER(c.c_int)
_u32p = c.POINTER(c.c_uint32)
_i32p = c.POINTER(c.c_int32)


class OrcLattice(c.Structure):
    _fields_ = [("lx", c.c_int), ("ly", c.c_int), ("lz", c.c_int), ("lt", c.c_int),
                ("vol", c.c_long), ("nn", _ip), ("eo_even", _ip), ("eo_odd", _ip)]


class OrcMT(c.Structure):
    _fields_ = [("matrix_a", c.c_uint32 * 4096), ("mask_b", c.c_uint32 * 4096),
                ("mask_c", c.c_uint32 * 4096), ("seed", c.c_uint32 * 4096),
                ("status", c.c_uint32 * (4096 * 19))]


class OrcPM(c.Structure):
    _fields_ = [("seed", c.c_long * 256), ("stream", c.c_int)]


def _p(a, t=c.c_double):
    return a.ctypes.data_as(c.POINTER(t))


class Oracle:
    """CPU restatement of the reference's hot path on 12-real ('2v') fields.

    fast=True loads the speed build of the same source (-O3, FMA contraction allowed),
    which bench.py times as the CPU baseline; its results differ from the checker's in
    the last bits, so tests use the default build."""

    def __init__(self, fast=False):
        self.lib = c.CDLL(_build.build_fast() if fast else _build.build_oracle())
        L = self.lib
        L.orc_plaquette.restype = c.c_double
        L.orc_gauge_functional18.restype = c.c_double
        L.orc_dAdA18.restype = c.c_double
        L.orc_mean_plaq18.restype = c.c_double
        L.orc_pm_random.restype = c.c_double
        L.orc_mt_nper.restype = c.c_int
        L.orc_overrelax_halfsweep.argtypes = [c.POINTER(OrcLattice), _dp, _dp, c.c_int,
                                              c.c_double, c.c_int]
        L.orc_heatbath_halfsweep.argtypes = [c.POINTER(OrcLattice), _dp, _dp, c.c_int, _fp,
                                             _fp, c.c_double]
        L.orc_link_heatbath_halfsweep.argtypes = [c.POINTER(OrcLattice), _dp, c.c_int, c.c_int,
                                                  _fp, _fp, c.c_double]
        L.orc_link_heatbath_halfsweep_kp.argtypes = L.orc_link_heatbath_halfsweep.argtypes
        L.orc_micro_halfsweep.argtypes = [c.POINTER(OrcLattice), _dp, _dp, c.c_int, c.c_int]

    # ---- lattice
    def lattice(self, dims):
        lx, ly, lz, lt = dims
        vol = lx * ly * lz * lt
        nn = np.empty(8 * vol, dtype=np.int32)
        ev = np.empty(vol // 2, dtype=np.int32)
        od = np.empty(vol // 2, dtype=np.int32)
        self.lib.orc_initnn(lx, ly, lz, lt, _p(nn, c.c_int))
        self.lib.orc_initnn_eo(lx, ly, lz, lt, _p(ev, c.c_int), _p(od, c.c_int))
        lat = OrcLattice(lx, ly, lz, lt, vol, _p(nn, c.c_int), _p(ev, c.c_int), _p(od, c.c_int))
        lat._keep = (nn, ev, od)
        return lat

    # ---- layout
    @staticmethod
    def to2v(su3):
        a = np.ascontiguousarray(su3, dtype=np.float64).reshape(-1, 18)
        return np.ascontiguousarray(a[:, :12])

    def from2v(self, v12):
        v = np.ascontiguousarray(v12, dtype=np.float64).reshape(-1, 12)
        out = np.empty((v.shape[0], 18))
        self.lib.orc_2v_to_su3(_p(v), _p(out), c.c_long(v.shape[0]))
        return out

    # ---- sweeps / observables (in place on the 2v arrays)
    def or_halfsweep(self, lat, gf12, g12, parity, omega=1.68, ndir=4):
        self.lib.orc_overrelax_halfsweep(c.byref(lat), _p(gf12), _p(g12), parity, omega, ndir)

    def or_sweeps(self, lat, gf12, g12, n, omega=1.68, ndir=4):
        for _ in range(n):
            self.or_halfsweep(lat, gf12, g12, 0, omega, ndir)
            self.or_halfsweep(lat, gf12, g12, 1, omega, ndir)

    def functional(self, lat, gf12, g12, ndir=4):
        out = np.zeros(3)
        self.lib.orc_functional(c.byref(lat), _p(gf12), _p(g12), ndir, _p(out))
        return {"F": out[0], "dAdA": out[1], "maxdAdA": out[2], "theta": out[1] / 3.0}

    def theta_slices(self, lat, gf12, g12, ndir=3):
        out = np.zeros(lat.lt)
        self.lib.orc_theta_slices(c.byref(lat), _p(gf12), _p(g12), ndir, _p(out))
        return out

    def plaquette(self, lat, gf12):
        return self.lib.orc_plaquette(c.byref(lat), _p(gf12))

    def polyakov(self, lat, gf12):
        out = np.zeros(2)
        self.lib.orc_polyakov(c.byref(lat), _p(gf12), _p(out))
        return complex(out[0], out[1])

    def heatbath_halfsweep(self, lat, gf12, g12, parity, gauss, unif, beta):
        self.lib.orc_heatbath_halfsweep(c.byref(lat), _p(gf12), _p(g12), parity,
                                        _p(gauss, c.c_float), _p(unif, c.c_float), beta)

    def micro_halfsweep(self, lat, gf12, g12, parity, ndir=4):
        self.lib.orc_micro_halfsweep(c.byref(lat), _p(gf12), _p(g12), parity, ndir)

    def link_heatbath_halfsweep(self, lat, gf12, parity, nu, gauss, unif, beta, variant=0):
        """variant 0: the reference's update; 1: Kennedy-Pendleton (Wilson action)"""
        f = self.lib.orc_link_heatbath_halfsweep_kp if variant else \
            self.lib.orc_link_heatbath_halfsweep
        f(c.byref(lat), _p(gf12), parity, nu, _p(gauss, c.c_float), _p(unif, c.c_float),
          beta / 3.0)

    def thermalize(self, lat, gf12, m, fields, nper_g, nper_u, beta, nsweep, variant=1):
        """nsweep sweeps of the link heatbath in the order of gfx_thermalize (nu = 0..3,
        parity 0, 1, a twister update after each half-sweep).  m is a twister bank and
        fields its current (gauss, unif) pair, from mt_init_fields.  Returns the
        plaquette after each sweep and the last fields."""
        plaq = []
        gauss, unif = fields
        for _ in range(nsweep):
            for nu in range(4):
                for par in range(2):
                    self.link_heatbath_halfsweep(lat, gf12, par, nu, gauss, unif, beta, variant)
                    gauss, unif = self.mt_update_fields(m, nper_g, nper_u)
            plaq.append(self.plaquette(lat, gf12))
        return np.array(plaq), (gauss, unif)

    # ---- twister bank
    def mt_new(self, params, seeds=None):
        m = OrcMT()
        p = np.asarray(params, dtype=np.uint32).reshape(4096, 4)
        np.ctypeslib.as_array(m.matrix_a)[:] = p[:, 0]
        np.ctypeslib.as_array(m.mask_b)[:] = p[:, 1]
        np.ctypeslib.as_array(m.mask_c)[:] = p[:, 2]
        np.ctypeslib.as_array(m.seed)[:] = p[:, 3] if seeds is None else seeds
        return m

    def mt_nper(self, n):
        return self.lib.orc_mt_nper(n)

    def mt_generate(self, m, nper, initialized):
        out = np.empty(4096 * nper, dtype=np.float32)
        self.lib.orc_mt_generate(c.byref(m), _p(out, c.c_float), nper, initialized)
        return out

    def boxmuller(self, d, nper):
        self.lib.orc_boxmuller(_p(d, c.c_float), nper)

    def mt_init_fields(self, m, nper_g, nper_u):
        g = np.empty(4096 * nper_g, dtype=np.float32)
        u = np.empty(4096 * nper_u, dtype=np.float32)
        self.lib.orc_mt_init_fields(c.byref(m), _p(g, c.c_float), nper_g, _p(u, c.c_float), nper_u)
        return g, u

    def mt_update_fields(self, m, nper_g, nper_u):
        g = np.empty(4096 * nper_g, dtype=np.float32)
        u = np.empty(4096 * nper_u, dtype=np.float32)
        self.lib.orc_mt_update_fields(c.byref(m), _p(g, c.c_float), nper_g, _p(u, c.c_float),
                                      nper_u)
        return g, u

    def mt_generic(self, state, n, m, umask, lmask, a, u, s, b, t, cc, l, nout):
        st = np.ascontiguousarray(state, dtype=np.uint32).copy()
        out = np.empty(nout, dtype=np.uint32)
        self.lib.orc_mt_generic(_p(st, c.c_uint32), n, m, c.c_uint32(umask), c.c_uint32(lmask),
                                c.c_uint32(a), u, s, c.c_uint32(b), t, c.c_uint32(cc), l,
                                _p(out, c.c_uint32), nout)
        return out

    def glibc_rand(self, seed, n):
        out = np.empty(n, dtype=np.int32)
        self.lib.orc_glibc_rand(c.c_uint(seed), n, _p(out, c.c_int32))
        return out

    # ---- Park-Miller and initial fields
    def pm_new(self, seed):
        pm = OrcPM()
        self.lib.orc_pm_plant(c.byref(pm), c.c_long(seed))
        return pm

    def pm_random(self, pm):
        return self.lib.orc_pm_random(c.byref(pm))

    def random_init(self, pm, n):
        out = np.empty((n, 18))
        self.lib.orc_random_init_su3_field(c.byref(pm), _p(out), c.c_long(n))
        return out

    # ---- host observables on 18-real fields
    def g_trafo18(self, lat, u18, g18):
        u = np.ascontiguousarray(u18, dtype=np.float64).copy()
        self.lib.orc_g_trafo18(c.byref(lat), _p(u), _p(np.ascontiguousarray(g18)))
        return u

    def gauge_functional18(self, lat, u18):
        return self.lib.orc_gauge_functional18(c.byref(lat), _p(np.ascontiguousarray(u18)))

    def dAdA18(self, lat, u18):
        mx = c.c_double(0)
        v = self.lib.orc_dAdA18(c.byref(lat), _p(np.ascontiguousarray(u18)), c.byref(mx))
        return v, mx.value

    def mean_plaq18(self, lat, u18):
        return self.lib.orc_mean_plaq18(c.byref(lat), _p(np.ascontiguousarray(u18)))


def load_mt_params(path=None):
    """The reference's twister parameters as a (4096, 4) uint32 array, or None."""
    path = path or DAT_PATH
    if not os.path.exists(path):
        return None
    return np.fromfile(path, dtype="<u4").reshape(4096, 4)


def synthetic_mt_params(seed=4172):
    """A deterministic stand-in parameter set (matrix_a with the top bit set, random
    tempering masks) for runs where the reference's parameter file is absent.  Not
    the reference's parameters; bit-exactness against the oracle holds for any set."""
    rng = np.random.default_rng(seed)
    p = rng.integers(0, 2 ** 32, size=(4096, 4), dtype=np.uint64).astype(np.uint32)
    p[:, 0] |= np.uint32(0x80000000)
    p[:, 3] = 0
    return p


class RefHost:
    """The reference's own host C code (observables.c, su3manip.c, rngs.c)."""

    def __init__(self):
        path = _build.build_reference_host()
        if not path or not os.path.exists(path):
            raise FileNotFoundError("reference host library not built (reference checkout absent)")
        self.lib = c.CDLL(path)
        L = self.lib
        for f in ("gauge_functional", "dAdA", "mean_plaq", "Random"):
            getattr(L, f).restype = c.c_double
        L.PlantSeeds.argtypes = [c.c_long]
        L.PutSeed.argtypes = [c.c_long]
        L.GetSeed.argtypes = [c.POINTER(c.c_long)]

    def set_lattice(self, dims, nn):
        lx, ly, lz, lt = dims
        for name, v in (("LX", lx), ("LY", ly), ("LZ", lz), ("T", lt),
                        ("VOLUME", lx * ly * lz * lt)):
            c.c_int.in_dll(self.lib, name).value = v
        self._nn = np.ascontiguousarray(nn, dtype=np.int32)
        c.c_void_p.in_dll(self.lib, "nn").value = self._nn.ctypes.data

    def gauge_functional(self, u18):
        return self.lib.gauge_functional(_p(np.ascontiguousarray(u18)))

    def dAdA(self, u18):
        v = self.lib.dAdA(_p(np.ascontiguousarray(u18)))
        return v, c.c_double.in_dll(self.lib, "maxDADA").value

    def mean_plaq(self, u18):
        return self.lib.mean_plaq(_p(np.ascontiguousarray(u18)))

    def g_trafo(self, u18, g18):
        u = np.ascontiguousarray(u18, dtype=np.float64).copy()
        self.lib.g_trafo(_p(u), _p(np.ascontiguousarray(g18)))
        return u

    def random_init_trafo(self, seed, n):
        """PlantSeeds(seed) then random_init_trafo on n = VOLUME matrices."""
        self.lib.PlantSeeds(seed)
        out = np.empty((n, 18))
        self.lib.random_init_trafo(_p(out))
        return out

    def random_init_gauge(self, seed, n):
        self.lib.PlantSeeds(seed)
        out = np.empty((n, 18))
        self.lib.random_init_gauge(_p(out))
        return out

    def su3to2v(self, su3, n):
        out = np.empty((n, 12))
        self.lib.su3to2v(_p(np.ascontiguousarray(su3)), _p(out))
        return out

    def from2vtosu3_trafo(self, v12, n):
        out = np.empty((n, 18))
        self.lib.from2vtosu3_trafo(_p(out), _p(np.ascontiguousarray(v12)))
        return out

    def test_random_state(self):
        """TestRandom's checks: state after 10000 draws from seed 1, and stream 1
        after PlantSeeds(1)."""
        L = self.lib
        L.SelectStream(0)
        L.PutSeed(1)
        for _ in range(10000):
            L.Random()
        x = c.c_long()
        L.GetSeed(c.byref(x))
        s0 = x.value
        L.SelectStream(1)
        L.PlantSeeds(1)
        L.GetSeed(c.byref(x))
        s1 = x.value
        L.SelectStream(0)
        return s0, s1
