"""Field transfers through the tiled layout kernels: from page-locked buffers of
gfx_host_alloc the GPU reads and writes the caller's array itself; from other host
memory the data is staged through device memory.  Both give the same fields bit for
bit (FP64 links, their FP32 copy, g), round-trip exactly, and report their device
times.  6^4 has a partial last tile (Vh = 648 is not a multiple of 32)."""
import numpy as np
import pytest

from conftest import haar, smooth_links

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("dims,nreal", [((6, 6, 6, 6), 12), ((8, 4, 6, 10), 18),
                                        ((16, 16, 16, 16), 12)])
def test_direct_and_staged_transfers_agree(gfx, dims, nreal):
    vol = int(np.prod(dims))
    u = smooth_links(dims, 0.4, 5).reshape(4 * vol, 3, 3, 2)
    g = haar(vol, 6).reshape(vol, 3, 3, 2)
    pu, pg = gfx.pinned_empty(u.shape), gfx.pinned_empty(g.shape)
    pu[...] = u
    pg[...] = g
    out = []
    for direct in (True, False):
        ctx = gfx.Context(dims, precision=gfx.PREC_MIXED, link_reals=nreal)
        ctx.set_links(pu if direct else u.copy())
        ctx.set_trafo(pg if direct else g.copy())
        t = ctx.transfer_times()
        assert t["set_links"][2] == direct and t["set_trafo"][2] == direct
        assert t["set_links"][1] > 0
        back = gfx.pinned_empty(g.shape) if direct else np.empty(g.shape)
        ctx.get_trafo_into(back)
        assert ctx.transfer_times()["get_trafo"][2] == direct
        links = ctx.get_links()
        ctx.or_sweeps(2, omega=1.7, precision=0)  # reads the FP32 copy
        g32 = ctx.get_trafo()
        out.append((links, np.array(back), g32))
        ctx.close()
    (la, ba, sa), (lb, bb, sb) = out
    assert np.array_equal(la, lb) and np.array_equal(ba, bb) and np.array_equal(sa, sb)
    assert np.array_equal(ba[:, :2], g[:, :2])  # rows 0,1 exact, row 2 rebuilt from them
    assert np.max(np.abs(ba[:, 2] - g[:, 2])) < 1e-15
    assert np.max(np.abs(la - u)) < 1e-15
