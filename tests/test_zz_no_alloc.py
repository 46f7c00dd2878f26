"""gfx_functional_noalloc: the functional and theta of device-resident fields computed
without any device allocation (for callers whose device memory is owned by their own
pool or fixed at start-up).  The caller's fields live in memory the test allocates
with torch; the result must match the context entry point gfx_functional on the same
fields, for two calls in a row (relative 1e-12, the FP64 functional tolerance of the
parity tests)."""
import ctypes

import numpy as np
import pytest

from conftest import haar, smooth_links

pytestmark = pytest.mark.gpu


def _eo_positions(dims, parity):
    lx, ly, lz, lt = dims
    vh = lx * ly * lz * lt // 2
    i = np.arange(vh)
    lxh = lx // 2
    xh, r = i % lxh, i // lxh
    y, r2 = r % ly, r // ly
    z, t = r2 % lz, r2 // lz
    x = 2 * xh + ((parity + y + z + t) & 1)
    return x + lx * (y + ly * (z + lz * t))


def _pack_links(dims, u, nreal):
    """(4V, 18) su3 -> library even/odd layout: [parity][mu][entry][site] complex."""
    u = np.asarray(u).reshape(-1, 9, 2)
    nc = nreal // 2
    out = np.empty((2, 4, nc, len(u) // 8, 2))
    for p in (0, 1):
        pos = _eo_positions(dims, p)
        for mu in range(4):
            out[p, mu] = np.transpose(u[4 * pos + mu, :nc], (1, 0, 2))
    return out


def _pack_trafo(dims, g):
    g = np.asarray(g).reshape(-1, 9, 2)
    out = np.empty((2, 6, len(g) // 2, 2))
    for p in (0, 1):
        out[p] = np.transpose(g[_eo_positions(dims, p), :6], (1, 0, 2))
    return out


def _noalloc(gfx, U, G, dims, nreal, gauge, res):
    f = gfx.lib.gfx_functional_noalloc
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_void_p, ctypes.c_void_p] + [ctypes.c_int] * 6 + [ctypes.c_void_p,
                                                                            ctypes.c_void_p]
    return f(U, G, *dims, nreal, gauge, res, None)


# (8,6,4,10): one block per (slice, parity); (24,16,12,4): 2304 sites per
# slice-parity, so 16 blocks stride over each slice; (2,2,2,1024): the largest time
# extent the fixed scratch holds
CASES = [((8, 6, 4, 10), 12, "landau"), ((8, 6, 4, 10), 18, "landau"),
         ((24, 16, 12, 4), 12, "landau"), ((24, 16, 12, 4), 18, "coulomb"),
         ((8, 6, 4, 10), 12, "coulomb"), ((2, 2, 2, 1024), 12, "landau")]


@pytest.mark.parametrize("dims,nreal,gauge", CASES)
def test_functional_noalloc_matches_context_entry_point(gfx, dims, nreal, gauge):
    torch = pytest.importorskip("torch")
    gauge = gfx.COULOMB if gauge == "coulomb" else gfx.LANDAU
    vol = int(np.prod(dims))
    u = smooth_links(dims, 0.5, 41)
    res = torch.zeros(5, dtype=torch.float64, device="cuda")
    U = torch.from_numpy(_pack_links(dims, u, nreal)).cuda()
    for call, seed in enumerate((42, 43)):
        g = haar(vol, seed)
        G = torch.from_numpy(_pack_trafo(dims, g)).cuda()
        torch.cuda.synchronize()
        assert _noalloc(gfx, U.data_ptr(), G.data_ptr(), dims, nreal, gauge,
                        res.data_ptr()) == 0
        torch.cuda.synchronize()
        got = res.cpu().numpy()
        ctx = gfx.Context(dims, link_reals=nreal)
        ctx.set_links(u)
        ctx.set_trafo(g)
        want = ctx.functional(gauge=gauge, precision=1)
        ctx.close()
        for k, name in enumerate(("F", "dAdA", "maxdAdA", "theta", "theta_slice_max")):
            assert got[k] == pytest.approx(getattr(want, name), rel=1e-12), (call, name)


def test_functional_noalloc_rejects_unknown_gauge(gfx):
    # checked with the other arguments, before any device work
    assert _noalloc(gfx, 16, 16, (4, 4, 4, 4), 12, 7, 16) == 6  # GFX_ERR_ARG


def test_functional_noalloc_rejects_too_many_slices(gfx):
    # lt beyond the 1024 slices of the fixed scratch: refused before any device work
    dims = (2, 2, 2, 1026)
    assert _noalloc(gfx, 16, 16, dims, 12, gfx.LANDAU, 16) == 6  # GFX_ERR_ARG
