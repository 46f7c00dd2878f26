"""cudagfx_gb300 -- Python host mirror of the cudagfx gauge-fixing interface on GB300.

Everything here calls libgfx.so (the sm_103a CUDA library, C ABI in include/gfx.h)
through ctypes.  There is no CPU fallback: importing the package builds the
library when it is missing or stale (``cudagfx_gb300.build.build()``) and raises
when that fails.

Two layers, as in the C ABI:
  * ``Context``: one lattice on the GPU with explicit-argument methods
    (set_links, overrelax, functional, plaquette, polyakov, simanneal, thermalize,
    the twister bank ...);
  * reference-named functions (``init_gaugefixing``, ``overrelax_gauge``,
    ``calc_functional``, ``calc_plaquette``, ``simannealing_gauge``,
    ``thermalize_gauge``, ``init_MT``, ``update_MT``) acting on the library's
    process-wide context and the reference's globals (``globals_()``).

Host arrays are numpy float64 arrays of shape (n, 3, 3, 2) or any shape with
18 doubles per SU(3) matrix, ordered as the reference's su3 (complex[3][3]).
"""
import ctypes
import os

import numpy as np

__all__ = ["lib", "Context", "GfxError", "ORParams", "ORResult", "Functional", "SAParams",
           "ThermParams", "PREC_DOUBLE", "PREC_SINGLE", "PREC_MIXED", "LANDAU", "COULOMB",
           "CRIT_MAXDADA", "CRIT_THETA", "CRIT_THETA_SLICES", "glibc_rand",
           "random_init_reference", "random_init_haar", "unit_init", "library_path"]

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "libgfx.so")

PREC_DOUBLE, PREC_SINGLE, PREC_MIXED = 0, 1, 2
LANDAU, COULOMB = 0, 1
CRIT_MAXDADA, CRIT_THETA, CRIT_THETA_SLICES = 0, 1, 2
HB_REFERENCE, HB_KENNEDY_PENDLETON = 0, 1
STATUS = {0: "GFX_OK", 1: "GFX_ERR_BAD_VOLUME", 2: "GFX_ERR_OOM", 3: "GFX_ERR_NOT_CONVERGED",
          4: "GFX_ERR_IO", 5: "GFX_ERR_CUDA", 6: "GFX_ERR_ARG", 7: "GFX_ERR_STATE"}


def library_path():
    return _LIB_PATH


# compile the library when it is missing or older than its sources (nvcc, sm_103a;
# an mtime check when it is current).  No fallback: without the library, no import.
try:
    from . import build as _build
    _build.build()
except Exception as e:  # noqa: BLE001
    if not os.path.exists(_LIB_PATH):
        raise ImportError("cudagfx_gb300: %s is missing and could not be built: %s"
                          % (_LIB_PATH, e)) from e
if not os.path.exists(_LIB_PATH):
    raise ImportError("cudagfx_gb300: %s is missing" % _LIB_PATH)

# RTLD_LOCAL: libgfx defines the reference's globals (LX, VOLUME, FUNC, ...); keep them
# out of the global namespace so other libraries in the process keep their own.
lib = ctypes.CDLL(_LIB_PATH, mode=ctypes.RTLD_LOCAL)

_c = ctypes
_dp = _c.POINTER(_c.c_double)
_fp = _c.POINTER(_c.c_float)
_u32p = _c.POINTER(_c.c_uint32)
_i32p = _c.POINTER(_c.c_int32)


class Functional(_c.Structure):
    _fields_ = [("F", _c.c_double), ("dAdA", _c.c_double), ("maxdAdA", _c.c_double),
                ("theta", _c.c_double), ("theta_slice_max", _c.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class ORParams(_c.Structure):
    _fields_ = [("maxit", _c.c_int), ("eps", _c.c_double), ("checkinterval", _c.c_int),
                ("omega", _c.c_double), ("criterion", _c.c_int), ("gauge", _c.c_int),
                ("switch_eps", _c.c_double), ("plateau_ratio", _c.c_double),
                ("checkinterval_double", _c.c_int), ("use_graph", _c.c_int),
                ("record_history", _c.c_int), ("checkinterval_near", _c.c_int),
                ("polish", _c.c_int), ("fp32_checks_all_sites", _c.c_int)]


class ORResult(_c.Structure):
    _fields_ = [("iterations", _c.c_int), ("sweeps", _c.c_int), ("sweeps_single", _c.c_int),
                ("sweeps_double", _c.c_int), ("converged", _c.c_int), ("checks", _c.c_int),
                ("final_values", Functional), ("ms", _c.c_double),
                ("sweeps_polish_df", _c.c_int), ("sweeps_polish_fp32", _c.c_int)]


class CheckRecord(_c.Structure):
    _fields_ = [("iter", _c.c_int), ("phase", _c.c_int), ("F", _c.c_double),
                ("dAdA", _c.c_double), ("maxdAdA", _c.c_double), ("theta", _c.c_double),
                ("theta_slice_max", _c.c_double)]


class SAParams(_c.Structure):
    _fields_ = [("Tmin", _c.c_double), ("Tmax", _c.c_double), ("expo", _c.c_double),
                ("N", _c.c_int), ("checkint", _c.c_int), ("nmicro", _c.c_int)]


class ThermParams(_c.Structure):
    _fields_ = [("Nsweep", _c.c_int), ("checkint", _c.c_int), ("beta", _c.c_double),
                ("variant", _c.c_int), ("precision", _c.c_int)]


class Tuning(_c.Structure):
    _fields_ = [("block", _c.c_int * 2), ("staging", _c.c_int * 2), ("link_reals64", _c.c_int),
                ("link_reals32", _c.c_int), ("checkinterval", _c.c_int),
                ("sweep_ms", _c.c_double * 2), ("check_ms", _c.c_double * 2),
                ("wide_regs", _c.c_int)]

    def as_dict(self):
        return {"block": list(self.block), "staging": list(self.staging),
                "link_reals64": self.link_reals64, "link_reals32": self.link_reals32,
                "checkinterval": self.checkinterval,
                "sweep_ms": list(self.sweep_ms), "check_ms": list(self.check_ms),
                "wide_regs": self.wide_regs}


def _sig(name, res, args):
    f = getattr(lib, name)
    f.restype = res
    f.argtypes = args
    return f


_V = _c.c_void_p
_I = _c.c_int
_D = _c.c_double
_sig("gfx_abi_version", _I, [])
_sig("gfx_status_string", _c.c_char_p, [_I])
_sig("gfx_last_error", _c.c_char_p, [_V])
_sig("gfx_create", _I, [_c.POINTER(_V), _I, _I, _I, _I, _I, _I, _V])
_sig("gfx_destroy", _I, [_V])
_sig("gfx_synchronize", _I, [_V])
_sig("gfx_device_bytes", _c.c_size_t, [_V])
_sig("gfx_set_block", _I, [_V, _I])
_sig("gfx_get_tuning", _I, [_V, _c.POINTER(Tuning)])
_sig("gfx_set_tuning", _I, [_V, _c.POINTER(Tuning)])
_sig("gfx_autotune", _I, [_V, _I, _I, _c.c_char_p, _c.POINTER(Tuning)])
for _n in ("gfx_set_links", "gfx_get_links", "gfx_set_trafo", "gfx_get_trafo"):
    _sig(_n, _I, [_V, _dp])
_sig("gfx_unit_trafo", _I, [_V])
_sig("gfx_or_params_default", None, [_c.POINTER(ORParams)])
_sig("gfx_overrelax", _I, [_V, _c.POINTER(ORParams), _c.POINTER(ORResult)])
_sig("gfx_or_history", _I, [_V, _c.POINTER(CheckRecord), _I])
_sig("gfx_or_sweeps", _I, [_V, _I, _D, _I, _I])
_sig("gfx_or_halfsweep", _I, [_V, _I, _D, _I, _I])
_sig("gfx_functional", _I, [_V, _I, _I, _c.POINTER(Functional)])
_sig("gfx_plaquette", _I, [_V, _dp])
_sig("gfx_polyakov", _I, [_V, _dp])
_sig("gfx_apply_trafo", _I, [_V])
_sig("gfx_mt_load_params", _I, [_V, _u32p])
_sig("gfx_mt_load_file", _I, [_V, _c.c_char_p])
_sig("gfx_mt_seed", _I, [_V, _c.c_uint])
_sig("gfx_mt_set_seeds", _I, [_V, _u32p])
_sig("gfx_mt_init", _I, [_V, _I, _I])
_sig("gfx_mt_update", _I, [_V])
_sig("gfx_mt_read", _I, [_V, _fp, _fp, _u32p, _u32p])
_sig("gfx_mt_sizes", _I, [_V, _c.POINTER(_I), _c.POINTER(_I)])
_sig("gfx_sa_temperature", _D, [_c.POINTER(SAParams), _I])
_sig("gfx_simanneal", _I, [_V, _c.POINTER(SAParams), _c.POINTER(Functional)])
_sig("gfx_simanneal_range", _I, [_V, _c.POINTER(SAParams), _I, _I])
_sig("gfx_sa_halfsweep", _I, [_V, _I, _D, _I])
_sig("gfx_micro_halfsweep", _I, [_V, _I, _I, _I])
_sig("gfx_thermalize", _I, [_V, _c.POINTER(ThermParams), _dp, _I])
_sig("gfx_link_heatbath_halfsweep", _I, [_V, _I, _I, _D, _I])
_sig("gfx_time_sweeps", _I, [_V, _I, _D, _I, _I, _dp])
_sig("gfx_launch_count", _c.c_ulonglong, [_V])
_sig("gfx_glibc_rand", None, [_c.c_uint, _I, _i32p])
_sig("gfx_random_init_reference", None, [_c.c_long, _dp, _c.c_long])
_sig("gfx_random_init_haar", None, [_c.c_uint64, _dp, _c.c_long])
_sig("gfx_unit_init", None, [_dp, _c.c_long])


class GfxError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__("%s: %s" % (STATUS.get(status, status), msg))
        self.status = status


def _ptr(a, ctype=_c.c_double):
    return a.ctypes.data_as(_c.POINTER(ctype))


def _f64(a, n):
    a = np.ascontiguousarray(a, dtype=np.float64)
    if a.size != 18 * n:
        raise ValueError("expected %d SU(3) matrices (%d doubles), got %d doubles"
                         % (n, 18 * n, a.size))
    return a


_sig("gfx_host_alloc", _V, [_c.c_size_t])
_sig("gfx_host_free", None, [_V])


class _Pinned:
    def __init__(self, nbytes):
        self.ptr = lib.gfx_host_alloc(nbytes)
        if not self.ptr:
            raise MemoryError("cudaMallocHost(%d) failed" % nbytes)

    def __del__(self):
        if self.ptr:
            lib.gfx_host_free(self.ptr)
            self.ptr = None


def pinned_empty(shape, dtype=np.float64):
    """numpy array in page-locked host memory (freed with the array)."""
    dtype = np.dtype(dtype)
    n = int(np.prod(shape)) * dtype.itemsize
    keep = _Pinned(max(n, 1))
    buf = (_c.c_char * n).from_address(keep.ptr)
    buf._owner = keep  # the array's base chain keeps buf, buf keeps the allocation
    return np.frombuffer(buf, dtype=dtype).reshape(shape)


def glibc_rand(seed, n):
    out = np.empty(n, dtype=np.int32)
    lib.gfx_glibc_rand(seed, n, _ptr(out, _c.c_int32))
    return out


def random_init_reference(seed, n):
    """random_init_trafo / random_init_gauge after PlantSeeds(seed) (n matrices)."""
    out = np.empty((n, 3, 3, 2))
    lib.gfx_random_init_reference(seed, _ptr(out), n)
    return out


def random_init_haar(seed, n):
    out = np.empty((n, 3, 3, 2))
    lib.gfx_random_init_haar(seed, _ptr(out), n)
    return out


def unit_init(n):
    out = np.empty((n, 3, 3, 2))
    lib.gfx_unit_init(_ptr(out), n)
    return out


class Context:
    """One lattice on the current CUDA device (gfx_create)."""

    def __init__(self, dims, precision=PREC_DOUBLE, link_reals=12, stream=None):
        lx, ly, lz, lt = dims
        h = _V()
        s = lib.gfx_create(_c.byref(h), lx, ly, lz, lt, precision, link_reals,
                           _V(stream) if stream else None)
        if s != 0:
            raise GfxError(s, lib.gfx_last_error(None).decode())
        self._h = h
        self.dims = (lx, ly, lz, lt)
        self.volume = lx * ly * lz * lt
        self.precision = precision

    def _check(self, s, ok=(0,)):
        if s not in ok:
            raise GfxError(s, lib.gfx_last_error(self._h).decode())
        return s

    def close(self):
        if self._h:
            lib.gfx_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    @property
    def handle(self):
        return self._h

    def device_bytes(self):
        return lib.gfx_device_bytes(self._h)

    def set_block(self, b):
        self._check(lib.gfx_set_block(self._h, b))

    def tuning(self):
        t = Tuning()
        self._check(lib.gfx_get_tuning(self._h, _c.byref(t)))
        return t.as_dict()

    def set_tuning(self, block=(128, 128), staging=(0, 0), link_reals64=0, checkinterval=0,
                   link_reals32=0, wide_regs=1):
        """staging per precision: 0 plain loads, 1 an L2 bulk prefetch per block first,
        2 plain loads with the odd half-sweep's blocks in reverse order, 3 as 2 with the
        FP32 g kept in L2 (evict_last), 4 as 3 with the FP32 links evict_first.  wide_regs: the
        FP32 half-sweep kernel with its full register set (1) or 64 registers (0)."""
        t = Tuning()
        t.wide_regs = wide_regs
        t.block[0], t.block[1] = block
        t.staging[0], t.staging[1] = staging
        t.link_reals64 = link_reals64
        t.link_reals32 = link_reals32
        t.checkinterval = checkinterval
        self._check(lib.gfx_set_tuning(self._h, _c.byref(t)))

    def autotune(self, gauge=LANDAU, expected_sweeps=0, cache_path=None):
        """Time the candidate launch settings on this lattice and keep the fastest
        (gfx_autotune); returns the chosen settings and their timings."""
        t = Tuning()
        self._check(lib.gfx_autotune(self._h, gauge, expected_sweeps,
                                     cache_path.encode() if cache_path else None, _c.byref(t)))
        return t.as_dict()

    def synchronize(self):
        self._check(lib.gfx_synchronize(self._h))

    # ---- fields
    def set_links(self, u):
        u = _f64(u, 4 * self.volume)
        self._check(lib.gfx_set_links(self._h, _ptr(u)))

    def get_links(self):
        out = np.empty((4 * self.volume, 3, 3, 2))
        self._check(lib.gfx_get_links(self._h, _ptr(out)))
        return out

    def set_trafo(self, g):
        g = _f64(g, self.volume)
        self._check(lib.gfx_set_trafo(self._h, _ptr(g)))

    def get_trafo(self):
        out = np.empty((self.volume, 3, 3, 2))
        self._check(lib.gfx_get_trafo(self._h, _ptr(out)))
        return out

    def get_trafo_into(self, out):
        if out.dtype != np.float64 or out.size != 18 * self.volume or not out.flags.c_contiguous:
            raise ValueError("out must be a C-contiguous float64 array of V su3 matrices")
        self._check(lib.gfx_get_trafo(self._h, _ptr(out)))
        return out

    def unit_trafo(self):
        self._check(lib.gfx_unit_trafo(self._h))

    def random_trafo_haar(self, seed):
        self._check(lib.gfx_random_trafo_haar(self._h, seed))

    # ---- gauge fixing
    @staticmethod
    def or_params(**kw):
        p = ORParams()
        lib.gfx_or_params_default(_c.byref(p))
        for k, v in kw.items():
            if not hasattr(p, k):
                raise AttributeError(k)
            setattr(p, k, v)
        return p

    def overrelax(self, params=None, **kw):
        p = params if params is not None else self.or_params(**kw)
        r = ORResult()
        self._check(lib.gfx_overrelax(self._h, _c.byref(p), _c.byref(r)), ok=(0, 3))
        return r

    def history(self):
        n = lib.gfx_or_history(self._h, None, 0)
        arr = (CheckRecord * max(n, 1))()
        lib.gfx_or_history(self._h, arr, n)
        return [{k: getattr(arr[i], k) for k, _ in CheckRecord._fields_} for i in range(n)]

    def or_sweeps(self, n, omega=1.68, gauge=LANDAU, precision=1):
        self._check(lib.gfx_or_sweeps(self._h, n, omega, gauge, precision))

    def time_sweeps(self, n, omega=1.68, gauge=LANDAU, precision=1):
        ms = np.zeros(1)
        self._check(lib.gfx_time_sweeps(self._h, n, omega, gauge, precision, _ptr(ms)))
        return float(ms[0])

    def transfer_times(self):
        """device ms of the last set_links / set_trafo / get_trafo: {name: (copy, layout,
        direct)}; direct = the GPU used the gfx_host_alloc buffer itself"""
        ms, d = np.zeros(6), (_I * 3)()
        self._check(lib.gfx_transfer_times(self._h, _ptr(ms), d))
        return {n: (float(ms[2 * k]), float(ms[2 * k + 1]), bool(d[k]))
                for k, n in enumerate(("set_links", "set_trafo", "get_trafo"))}

    def set_fused_check(self, fused):
        self._check(lib.gfx_set_fused_check(self._h, 1 if fused else 0))

    def launch_count(self):
        return lib.gfx_launch_count(self._h)

    def or_halfsweep(self, parity, omega=1.68, gauge=LANDAU, precision=1):
        self._check(lib.gfx_or_halfsweep(self._h, parity, omega, gauge, precision))

    def functional(self, gauge=LANDAU, precision=1):
        f = Functional()
        self._check(lib.gfx_functional(self._h, gauge, precision, _c.byref(f)))
        return f

    def plaquette(self):
        v = np.zeros(1)
        self._check(lib.gfx_plaquette(self._h, _ptr(v)))
        return float(v[0])

    def polyakov(self):
        v = np.zeros(2)
        self._check(lib.gfx_polyakov(self._h, _ptr(v)))
        return complex(v[0], v[1])

    def apply_trafo(self):
        self._check(lib.gfx_apply_trafo(self._h))

    # ---- twister bank
    def mt_load_params(self, params):
        p = np.ascontiguousarray(params, dtype=np.uint32).reshape(-1)
        if p.size != 4 * 4096:
            raise ValueError("twister parameters: 4096 x {matrix_a, mask_b, mask_c, seed}")
        self._check(lib.gfx_mt_load_params(self._h, _ptr(p, _c.c_uint32)))

    def mt_load_file(self, path):
        self._check(lib.gfx_mt_load_file(self._h, os.fsencode(path)))

    def mt_seed(self, seed):
        self._check(lib.gfx_mt_seed(self._h, seed))

    def mt_set_seeds(self, seeds):
        s = np.ascontiguousarray(seeds, dtype=np.uint32)
        self._check(lib.gfx_mt_set_seeds(self._h, _ptr(s, _c.c_uint32)))

    def mt_init(self, n_gauss, n_unif):
        self._check(lib.gfx_mt_init(self._h, n_gauss, n_unif))

    def mt_update(self):
        self._check(lib.gfx_mt_update(self._h))

    def mt_sizes(self):
        a, b = _I(), _I()
        lib.gfx_mt_sizes(self._h, _c.byref(a), _c.byref(b))
        return a.value, b.value

    def mt_read(self):
        ng, nu = self.mt_sizes()
        g = np.empty(4096 * ng, dtype=np.float32)
        u = np.empty(4096 * nu, dtype=np.float32)
        st = np.empty(19 * 4096, dtype=np.uint32)
        sd = np.empty(4096, dtype=np.uint32)
        self._check(lib.gfx_mt_read(self._h, _ptr(g, _c.c_float), _ptr(u, _c.c_float),
                                    _ptr(st, _c.c_uint32), _ptr(sd, _c.c_uint32)))
        return g, u, st.reshape(19, 4096), sd

    # ---- simulated annealing / thermalization
    def simanneal(self, Tmin, Tmax, N, expo=-1.0, checkint=100, nmicro=0):
        p = SAParams(Tmin, Tmax, expo, N, checkint, nmicro)
        f = Functional()
        self._check(lib.gfx_simanneal(self._h, _c.byref(p), _c.byref(f)))
        return f

    def sa_halfsweep(self, parity, beta, precision=1):
        self._check(lib.gfx_sa_halfsweep(self._h, parity, beta, precision))

    def micro_halfsweep(self, parity, gauge=LANDAU, precision=1):
        self._check(lib.gfx_micro_halfsweep(self._h, parity, gauge, precision))

    def thermalize(self, beta, nsweep, checkint=0, variant=HB_REFERENCE, precision=0):
        """precision 0: FP64 heatbath (the reference's arithmetic); 1: FP32 staples and
        SU(2) steps, reunitarized in double-float and stored in FP64 and FP32 (SINGLE or
        MIXED contexts)."""
        p = ThermParams(nsweep, checkint, beta, variant, precision)
        cap = (nsweep + checkint - 1) // checkint if checkint > 0 else 0
        plaq = np.zeros(max(cap, 1))
        self._check(lib.gfx_thermalize(self._h, _c.byref(p), _ptr(plaq), cap))
        return plaq[:cap]

    def link_heatbath_halfsweep(self, parity, nu, beta, variant=HB_REFERENCE):
        self._check(lib.gfx_link_heatbath_halfsweep(self._h, parity, nu, beta, variant))

    # ---- files (include/gfx_io.h)
    def load_links_ildg(self, path):
        info = IldgInfo()
        self._check(lib.gfx_load_links_ildg(self._h, os.fsencode(path), _c.byref(info)))
        return info.as_dict()

    def write_links_ildg(self, path, precision=64, beta=0.0):
        self._check(lib.gfx_write_links_ildg(self._h, os.fsencode(path), precision, beta))

    def write_fixed_ildg(self, path, precision=64, beta=0.0):
        """The gauge-fixed field g U g^+ as an ILDG file; the context is unchanged."""
        self._check(lib.gfx_write_fixed_ildg(self._h, os.fsencode(path), precision, beta))

    def checkpoint_save(self, path):
        self._check(lib.gfx_checkpoint_save(self._h, os.fsencode(path)))

    def checkpoint_load(self, path):
        self._check(lib.gfx_checkpoint_load(self._h, os.fsencode(path)))


class CopyResult(_c.Structure):
    _fields_ = [("conf", _c.c_int), ("copy", _c.c_int), ("converged", _c.c_int),
                ("iterations", _c.c_int), ("sweeps", _c.c_int), ("sweeps_single", _c.c_int),
                ("sweeps_double", _c.c_int), ("F", _c.c_double), ("dAdA", _c.c_double),
                ("maxdAdA", _c.c_double), ("theta", _c.c_double),
                ("theta_slice_max", _c.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


_sig("gfx_batch_create", _I, [_c.POINTER(_V), _I, _c.POINTER(_I), _c.POINTER(_I), _I, _V])
_sig("gfx_batch_destroy", _I, [_V])
_sig("gfx_batch_last_error", _c.c_char_p, [_V])
_sig("gfx_batch_copies", _I, [_V])
_sig("gfx_batch_set_links", _I, [_V, _I, _dp])
_sig("gfx_batch_set_trafo", _I, [_V, _I, _I, _dp])
_sig("gfx_batch_get_trafo", _I, [_V, _I, _I, _dp])
_sig("gfx_batch_random_haar", _I, [_V, _c.c_uint64])
_sig("gfx_batch_random_haar_copy", _I, [_V, _I, _I, _c.c_uint64])
_sig("gfx_batch_set_paired", _I, [_V, _I])
_sig("gfx_set_fused_check", _I, [_V, _I])
_sig("gfx_transfer_times", _I, [_V, _dp, _c.POINTER(_I)])
_sig("gfx_batch_overrelax", _I, [_V, _c.POINTER(ORParams), _c.POINTER(CopyResult), _dp])
_sig("gfx_batch_best", _I, [_V, _c.POINTER(CopyResult), _I, _c.POINTER(_I), _dp])
_sig("gfx_random_trafo_haar", _I, [_V, _c.c_uint64])


class Batch:
    """Gauge copies of several configurations fixed together (gfx_batch_*)."""

    def __init__(self, dims_list, ncopies, precision=PREC_MIXED, stream=None):
        n = len(dims_list)
        d = (_I * (4 * n))(*[x for dims in dims_list for x in dims])
        c = (_I * n)(*ncopies)
        h = _V()
        s = lib.gfx_batch_create(_c.byref(h), n, d, c, precision,
                                 _V(stream) if stream else None)
        if s != 0:
            raise GfxError(s, lib.gfx_batch_last_error(None).decode())
        self._h = h
        self.dims = [tuple(x) for x in dims_list]
        self.ncopies = list(ncopies)
        self.total = lib.gfx_batch_copies(h)

    def _check(self, s, ok=(0,)):
        if s not in ok:
            raise GfxError(s, lib.gfx_batch_last_error(self._h).decode())
        return s

    def close(self):
        if self._h:
            lib.gfx_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_links(self, conf, u):
        v = int(np.prod(self.dims[conf]))
        self._check(lib.gfx_batch_set_links(self._h, conf, _ptr(_f64(u, 4 * v))))

    def set_trafo(self, conf, copy, g):
        v = int(np.prod(self.dims[conf]))
        self._check(lib.gfx_batch_set_trafo(self._h, conf, copy, _ptr(_f64(g, v))))

    def get_trafo(self, conf, copy):
        out = np.empty((int(np.prod(self.dims[conf])), 3, 3, 2))
        self._check(lib.gfx_batch_get_trafo(self._h, conf, copy, _ptr(out)))
        return out

    def random_haar(self, seed):
        self._check(lib.gfx_batch_random_haar(self._h, seed))

    def set_paired(self, paired):
        self._check(lib.gfx_batch_set_paired(self._h, 1 if paired else 0))

    def random_haar_copy(self, conf, copy, seed):
        self._check(lib.gfx_batch_random_haar_copy(self._h, conf, copy, seed))

    def overrelax(self, params=None, **kw):
        p = params if params is not None else Context.or_params(**kw)
        res = (CopyResult * self.total)()
        ms = np.zeros(1)
        self._check(lib.gfx_batch_overrelax(self._h, _c.byref(p), res, _ptr(ms)), ok=(0, 3))
        self.last_results = res
        return [r.as_dict() for r in res], float(ms[0])

    def best(self, conf):
        k, f = _I(), np.zeros(1)
        self._check(lib.gfx_batch_best(self._h, self.last_results, conf, _c.byref(k), _ptr(f)),
                    ok=(0, 3))
        return k.value, float(f[0])


def sa_temperature(Tmin, Tmax, N, expo, i):
    p = SAParams(Tmin, Tmax, expo, N, 1, 0)
    return lib.gfx_sa_temperature(_c.byref(p), i)


from . import legacy  # noqa: E402,F401  (reference-named entry points)


# ---------------------------------------------------------------------------
# gauge-field files (include/gfx_io.h): ILDG, BQCD, POSIX cksum
# ---------------------------------------------------------------------------
class IldgInfo(_c.Structure):
    _fields_ = [("dims", _I * 4), ("precision", _I), ("plaquette", _c.c_double),
                ("beta", _c.c_double), ("data_bytes", _c.c_uint64)]

    def as_dict(self):
        return {"dims": tuple(self.dims), "precision": self.precision,
                "plaquette": self.plaquette, "beta": self.beta, "data_bytes": self.data_bytes}


class SliceCksum(_c.Structure):
    _fields_ = [("file", _c.c_char * 80), ("sum", _c.c_uint64), ("bytes", _c.c_uint64)]


class BqcdInfo(_c.Structure):
    _fields_ = [("run", _I), ("dims", _I * 4), ("beta", _c.c_double), ("plaquette", _c.c_double)]


class CksumState(_c.Structure):
    _fields_ = [("crc", _c.c_uint32), ("bytes", _c.c_uint64)]


_sig("gfx_ildg_read_info", _I, [_c.c_char_p, _c.POINTER(IldgInfo)])
_sig("gfx_ildg_read", _I, [_c.c_char_p, _c.POINTER(_I), _dp, _c.POINTER(IldgInfo)])
_sig("gfx_ildg_write", _I, [_c.c_char_p, _c.POINTER(_I), _dp, _I, _D, _D])
_sig("gfx_cksum_init", None, [_c.POINTER(CksumState)])
_sig("gfx_cksum_add", None, [_c.POINTER(CksumState), _V, _c.c_size_t])
_sig("gfx_cksum_get", _c.c_uint32, [_c.POINTER(CksumState)])
_sig("gfx_bqcd_write", _I, [_c.c_char_p, _c.POINTER(_I), _dp, _D, _D, _I,
                            _c.POINTER(SliceCksum)])
_sig("gfx_bqcd_read", _I, [_c.c_char_p, _c.POINTER(_I), _dp, _c.POINTER(SliceCksum)])
_sig("gfx_bqcd_read_trafo", _I, [_c.c_char_p, _c.POINTER(_I), _dp, _c.POINTER(SliceCksum)])
_sig("gfx_bqcd_write_trafo", _I, [_c.c_char_p, _c.POINTER(_I), _dp, _c.POINTER(SliceCksum)])
_sig("gfx_bqcd_read_info", _I, [_c.c_char_p, _c.POINTER(BqcdInfo), _c.POINTER(SliceCksum), _I,
                                _c.POINTER(_I)])
_sig("gfx_load_links_ildg", _I, [_V, _c.c_char_p, _c.POINTER(IldgInfo)])
_sig("gfx_write_links_ildg", _I, [_V, _c.c_char_p, _I, _D])
_sig("gfx_write_fixed_ildg", _I, [_V, _c.c_char_p, _I, _D])
_sig("gfx_checkpoint_save", _I, [_V, _c.c_char_p])
_sig("gfx_checkpoint_load", _I, [_V, _c.c_char_p])


def _io_check(s):
    if s != 0:
        raise GfxError(s, lib.gfx_last_error(None).decode())


def _dims4(dims):
    return (_I * 4)(*[int(x) for x in dims])


def _cks_list(arr, n):
    return [{"file": arr[k].file.decode(), "sum": arr[k].sum, "bytes": arr[k].bytes}
            for k in range(n)]


def ildg_read_info(path):
    info = IldgInfo()
    _io_check(lib.gfx_ildg_read_info(os.fsencode(path), _c.byref(info)))
    return info.as_dict()


def ildg_read(path, dims):
    """links (4V, 3, 3, 2) and the file's metadata"""
    V = int(np.prod(dims))
    out = np.empty((4 * V, 3, 3, 2))
    info = IldgInfo()
    _io_check(lib.gfx_ildg_read(os.fsencode(path), _dims4(dims), _ptr(out), _c.byref(info)))
    return out, info.as_dict()


def ildg_write(path, dims, links, precision=64, plaquette=0.0, beta=0.0):
    V = int(np.prod(dims))
    a = _f64(links, 4 * V)
    _io_check(lib.gfx_ildg_write(os.fsencode(path), _dims4(dims), _ptr(a), precision,
                                 plaquette, beta))


def cksum(data):
    """POSIX cksum of a bytes-like object: (crc, byte count)"""
    b = bytes(data)
    st = CksumState()
    lib.gfx_cksum_init(_c.byref(st))
    buf = _c.create_string_buffer(b, len(b))
    lib.gfx_cksum_add(_c.byref(st), _c.cast(buf, _V), len(b))
    return int(lib.gfx_cksum_get(_c.byref(st))), int(st.bytes)


def bqcd_write(basename, dims, links, plaquette=0.0, beta=0.0, ensemble=0):
    V = int(np.prod(dims))
    a = _f64(links, 4 * V)
    cks = (SliceCksum * dims[3])()
    _io_check(lib.gfx_bqcd_write(os.fsencode(basename), _dims4(dims), _ptr(a), plaquette, beta,
                                 ensemble, cks))
    return _cks_list(cks, dims[3])


def bqcd_read(basename, dims):
    V = int(np.prod(dims))
    out = np.empty((4 * V, 3, 3, 2))
    cks = (SliceCksum * dims[3])()
    _io_check(lib.gfx_bqcd_read(os.fsencode(basename), _dims4(dims), _ptr(out), cks))
    return out, _cks_list(cks, dims[3])


def bqcd_write_trafo(basename, dims, trafo):
    V = int(np.prod(dims))
    a = _f64(trafo, V)
    cks = (SliceCksum * dims[3])()
    _io_check(lib.gfx_bqcd_write_trafo(os.fsencode(basename), _dims4(dims), _ptr(a), cks))
    return _cks_list(cks, dims[3])


def bqcd_read_trafo(basename, dims):
    V = int(np.prod(dims))
    out = np.empty((V, 3, 3, 2))
    cks = (SliceCksum * dims[3])()
    _io_check(lib.gfx_bqcd_read_trafo(os.fsencode(basename), _dims4(dims), _ptr(out), cks))
    return out, _cks_list(cks, dims[3])


def bqcd_read_info(path, cap=4096):
    info = BqcdInfo()
    cks = (SliceCksum * cap)()
    n = _I()
    _io_check(lib.gfx_bqcd_read_info(os.fsencode(path), _c.byref(info), cks, cap, _c.byref(n)))
    return ({"run": info.run, "dims": tuple(info.dims), "beta": info.beta,
             "plaquette": info.plaquette}, _cks_list(cks, n.value))
