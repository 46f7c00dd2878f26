"""FP32 convergence checks fused into the last odd half-sweep (or_halfsweep_measure_kernel
+ the even-site measurement) against the separate measurement kernel: the same check
values bit for bit, hence the same loop decisions and the same gauge transformation.
Lattices whose time slices do not hold whole 128-site blocks per parity use the
separate measurement either way."""
import numpy as np
import pytest

from conftest import haar, smooth_links

pytestmark = pytest.mark.gpu


def _solve(gfx, dims, fused, gauge, **kw):
    vol = int(np.prod(dims))
    ctx = gfx.Context(dims, precision=gfx.PREC_MIXED)
    ctx.set_links(smooth_links(dims, 0.45, 77))
    ctx.set_trafo(haar(vol, 78))
    ctx.set_fused_check(fused)
    r = ctx.overrelax(gauge=gauge, **kw)
    out = (r, ctx.history(), ctx.get_trafo())
    ctx.close()
    return out


@pytest.mark.parametrize("dims,gauge", [((8, 8, 8, 8), "landau"), ((16, 8, 8, 16), "landau"),
                                        ((8, 8, 8, 8), "coulomb"), ((4, 6, 8, 10), "landau")])
@pytest.mark.parametrize("use_graph", [1, 0])
def test_fused_check_bit_identical(gfx, dims, gauge, use_graph):
    g = gfx.COULOMB if gauge == "coulomb" else gfx.LANDAU
    crit = gfx.CRIT_THETA_SLICES if gauge == "coulomb" else gfx.CRIT_THETA
    kw = dict(maxit=6000, eps=1e-12, checkinterval=15, omega=1.7, criterion=crit,
              switch_eps=1e-9, checkinterval_double=3, checkinterval_near=5, polish=2,
              use_graph=use_graph)
    (ra, ha, ga), (rb, hb, gb) = (_solve(gfx, dims, f, g, **kw) for f in (1, 0))
    assert ra.converged and rb.converged
    assert ra.sweeps_single == rb.sweeps_single and ra.sweeps == rb.sweeps
    assert len(ha) == len(hb) and len(ha) > 5
    for a, b in zip(ha, hb):
        assert a == b  # every check record bit for bit
    assert np.array_equal(ga, gb)


def test_functional_precision0_matches_fp64(gfx):
    # the FP32 measurement (the star of the FP32 sweep) agrees with FP64 to FP32 rounding
    dims = (8, 8, 8, 8)
    ctx = gfx.Context(dims, precision=gfx.PREC_MIXED)
    ctx.set_links(smooth_links(dims, 0.45, 77))
    ctx.set_trafo(haar(8 ** 4, 78))
    f32, f64 = ctx.functional(precision=0), ctx.functional(precision=1)
    assert f32.F == pytest.approx(f64.F, rel=1e-6)
    assert f32.dAdA == pytest.approx(f64.dAdA, rel=1e-5)
