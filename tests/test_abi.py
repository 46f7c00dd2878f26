"""The C-ABI library loads without a GPU and exports every function and global that
include/*.h declares; host-side helpers agree with the oracle.  CPU only."""
import ctypes
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared(header):
    src = open(os.path.join(ROOT, "include", header)).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    funcs = set(re.findall(r"\b([A-Za-z_]\w*)\s*\([^;{]*\)\s*;", src))
    funcs -= {"if", "while", "for", "return", "sizeof"}
    globs = set()
    for line in src.splitlines():
        m = re.match(r"\s*extern\s+[\w\s\*]+?\s+([\w\s,\*]+);", line)
        if m and "(" not in line:
            for name in m.group(1).split(","):
                globs.add(name.strip().lstrip("*").strip())
    return funcs, globs


@pytest.mark.parametrize("header", ["gfx.h", "gfx_legacy.h", "gfx_io.h", "lime.h"])
def test_every_declared_symbol_is_exported(gfx, header):
    funcs, globs = _declared(header)
    assert len(funcs) > 10 if header == "gfx.h" else len(funcs) > 8
    lib = ctypes.CDLL(gfx.library_path())
    missing = [n for n in sorted(funcs | globs) if not hasattr(lib, n)]
    assert not missing, missing


def test_abi_version_and_status_strings(gfx):
    assert gfx.lib.gfx_abi_version() == 1
    assert gfx.lib.gfx_status_string(3).decode().startswith("gauge condition")


def test_glibc_seed_stream_matches_oracle(gfx, oracle):
    for seed in (1, 42, 351, 2 ** 31 + 7):
        assert np.array_equal(gfx.glibc_rand(seed, 4096), oracle.glibc_rand(seed, 4096))


def test_reference_random_init_matches_reference(gfx, oracle, refhost):
    lat = oracle.lattice((4, 4, 4, 8))
    refhost.set_lattice((4, 4, 4, 8), lat._keep[0])
    got = gfx.random_init_reference(351, 512).reshape(512, 18)
    assert np.array_equal(got, refhost.random_init_trafo(351, 512))


def test_haar_init_is_su3_and_seeded(gfx):
    a = gfx.random_init_haar(7, 2000)
    b = gfx.random_init_haar(7, 2000)
    assert np.array_equal(a, b)
    m = a[..., 0] + 1j * a[..., 1]
    eye = np.eye(3)
    assert np.max(np.abs(m @ np.conj(np.swapaxes(m, 1, 2)) - eye)) < 1e-14
    assert np.max(np.abs(np.linalg.det(m) - 1.0)) < 1e-14
    # Haar moments: E[tr U] = 0, E[|tr U|^2] = 1
    tr = np.trace(m, axis1=1, axis2=2)
    assert abs(tr.mean()) < 0.1
    assert abs(np.mean(np.abs(tr) ** 2) - 1.0) < 0.15


def test_context_creation_errors_without_device(gfx):
    # bad extents are rejected before any device call
    with pytest.raises(gfx.GfxError) as e:
        gfx.Context((3, 4, 4, 4))
    assert e.value.status == 1


def test_sa_temperature_matches_reference_formulas(gfx):
    # set_sa_temperature (simulated_annealing.cu:265-299)
    from cudagfx_gb300 import sa_temperature
    Tmin, Tmax, N = 1e-4, 0.5, 5000
    for i in (0, 1, 17, 4999):
        assert sa_temperature(Tmin, Tmax, N, -1.0, i) == pytest.approx(
            (Tmin - Tmax) / (N - 1) * i + Tmax, rel=1e-15)
        assert sa_temperature(Tmin, Tmax, N, 0.0, i) == pytest.approx(
            (Tmin / Tmax) ** (i / (N - 1)) * Tmax, rel=1e-15)
        a = (Tmin ** -2.0 - Tmax ** -2.0) / (N - 1)
        assert sa_temperature(Tmin, Tmax, N, 2.0, i) == pytest.approx(
            (a * i + Tmax ** -2.0) ** (-1 / 2.0), rel=1e-14)


def test_legacy_host_tables_match_reference_layout(gfx, oracle):
    # the tables init_gaugefixing fills for the reference's host code (initnn and
    # initnn_eo, cudagaugefix.cu:72-196): compared with the oracle's restatement
    import ctypes
    lib = gfx.lib
    dims = (4, 6, 2, 8)
    for name, v in zip(("LX", "LY", "LZ", "T"), dims):
        ctypes.c_int.in_dll(lib, name).value = v
    V = int(np.prod(dims))
    assert lib.gfx_legacy_init_tables() == 0

    def table(name, n):
        p = ctypes.c_void_p.in_dll(lib, name).value
        return np.ctypeslib.as_array((ctypes.c_int * n).from_address(p)).copy()

    onn, oev, ood = oracle.lattice(dims)._keep
    nn = table("nn", 8 * V)
    assert np.array_equal(nn, onn)
    even, odd = table("eoidx_even", V // 2), table("eoidx_odd", V // 2)
    assert np.array_equal(even, oev) and np.array_equal(odd, ood)
    assert np.array_equal(table("ind", V), np.arange(V))
    l2e = table("lexic2eo", V)
    assert np.array_equal(l2e[even], np.arange(V // 2)) and np.array_equal(l2e[odd], np.arange(V // 2))
    nn_eo, nn_oe = table("nn_eo", 4 * V).reshape(-1, 8), table("nn_oe", 4 * V).reshape(-1, 8)
    assert np.array_equal(nn_eo, l2e[nn.reshape(-1, 8)[even]])
    assert np.array_equal(nn_oe, l2e[nn.reshape(-1, 8)[odd]])
