"""Reference-named entry points of libgfx (include/gfx_legacy.h) for Python callers.

These act on the library's process-wide context and the reference's globals
(T, LX, LY, LZ, VOLUME, FUNC, DADA, maxDADA, PLAQ, orx*, saparam, thermparam),
exactly as the reference's main uses them (cudagaugefix.cu:599-828).
"""
import ctypes as _c

import numpy as np

from . import lib

_dp = _c.POINTER(_c.c_double)


class SAParamList(_c.Structure):
    """SAPARAM_LIST (global.h:51-57)"""
    _fields_ = [("Tmin", _c.c_double), ("Tmax", _c.c_double), ("expo", _c.c_double),
                ("N", _c.c_int), ("checkint", _c.c_int)]


class ThermParamList(_c.Structure):
    """THERMPARAM_LIST (global.h:61-67)"""
    _fields_ = [("Nsweep", _c.c_int), ("Nsave", _c.c_int), ("beta", _c.c_double),
                ("checkint", _c.c_int), ("startcond", _c.c_int)]


_INTS = ["T", "L", "LX", "LY", "LZ", "VOLUME", "randseed", "orxmaxit", "orxcheckinterval",
         "saflag", "orxflag", "thermflag"]
_DOUBLES = ["PLAQ", "FUNC", "DADA", "maxDADA", "orxeps"]


def gvar(name):
    """ctypes view of one of the reference's globals inside libgfx."""
    if name in _INTS:
        return _c.c_int.in_dll(lib, name)
    if name in _DOUBLES:
        return _c.c_double.in_dll(lib, name)
    if name == "saparam":
        return SAParamList.in_dll(lib, name)
    if name == "thermparam":
        return ThermParamList.in_dll(lib, name)
    raise KeyError(name)


def set_lattice(lx, ly, lz, lt):
    """What read_input does with T and L (read_input.l:276-279), for any extents."""
    gvar("LX").value, gvar("LY").value, gvar("LZ").value, gvar("T").value = lx, ly, lz, lt
    gvar("L").value = lx
    gvar("VOLUME").value = lx * ly * lz * lt


def _sig(name, res, args):
    f = getattr(lib, name)
    f.restype = res
    f.argtypes = args
    return f


_sig("init_gaugefixing", None, [_dp, _dp])
_sig("finalize_gaugefixing", None, [])
_sig("init_thermalization", None, [_dp])
_sig("finalize_thermalization", None, [])
_sig("overrelax_gauge", _c.c_int, [_c.c_int, _c.c_double, _c.c_int])
_sig("calc_functional", _c.c_double, [_c.c_void_p, _c.c_void_p])
_sig("calc_plaquette", _c.c_double, [_c.c_void_p, _c.c_int])
_sig("simannealing_gauge", None, [])
_sig("thermalize_gauge", None, [])
_sig("init_MT", None, [_c.c_int, _c.c_int])
_sig("update_MT", None, [])
_sig("finalize_MT", None, [])
_sig("benchmark", None, [])
_sig("gfx_legacy_get_trafo", _c.c_int, [_dp])
_sig("gfx_legacy_get_gauge", _c.c_int, [_dp])
_sig("gfx_legacy_set_precision", None, [_c.c_int])
_sig("gfx_legacy_set_omega", None, [_c.c_double])
_sig("gfx_legacy_set_mtseed", None, [_c.c_uint])
_sig("gfx_legacy_set_nmicro", None, [_c.c_int])
_sig("gfx_legacy_context", _c.c_void_p, [])


def _arr(a, n):
    a = np.ascontiguousarray(a, dtype=np.float64)
    assert a.size == 18 * n
    return a


def init_gaugefixing(gf, trafo):
    v = gvar("VOLUME").value
    lib.init_gaugefixing(_arr(gf, 4 * v).ctypes.data_as(_dp), _arr(trafo, v).ctypes.data_as(_dp))


def finalize_gaugefixing():
    lib.finalize_gaugefixing()


def init_thermalization(gf):
    v = gvar("VOLUME").value
    lib.init_thermalization(_arr(gf, 4 * v).ctypes.data_as(_dp))


def finalize_thermalization():
    lib.finalize_thermalization()


def overrelax_gauge(maxit, eps, checkinterval):
    return lib.overrelax_gauge(maxit, eps, checkinterval)


def calc_functional():
    return lib.calc_functional(None, None)


def calc_plaquette(outputyn=0):
    return lib.calc_plaquette(None, outputyn)


def simannealing_gauge():
    lib.simannealing_gauge()


def thermalize_gauge():
    lib.thermalize_gauge()


def init_MT(n_gauss, n_unif):
    lib.init_MT(n_gauss, n_unif)


def update_MT():
    lib.update_MT()


def finalize_MT():
    lib.finalize_MT()


def get_trafo():
    out = np.empty((gvar("VOLUME").value, 3, 3, 2))
    s = lib.gfx_legacy_get_trafo(out.ctypes.data_as(_dp))
    if s != 0:
        raise RuntimeError("gfx_legacy_get_trafo: status %d" % s)
    return out


def get_gauge():
    out = np.empty((4 * gvar("VOLUME").value, 3, 3, 2))
    s = lib.gfx_legacy_get_gauge(out.ctypes.data_as(_dp))
    if s != 0:
        raise RuntimeError("gfx_legacy_get_gauge: status %d" % s)
    return out


set_precision = lib.gfx_legacy_set_precision
set_omega = lib.gfx_legacy_set_omega
set_mtseed = lib.gfx_legacy_set_mtseed
set_nmicro = lib.gfx_legacy_set_nmicro
