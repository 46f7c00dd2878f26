"""Double-float polish sweeps (float pairs on the FP32 units): they follow the FP64
sweeps to ~1e-13 and a mixed solve polished with them reaches the FP64-confirmed
target and the same gauge copy as the FP64 polish."""
import numpy as np
import pytest

import cudagfx_gb300 as gfx
from conftest import smooth_links

pytestmark = pytest.mark.gpu

DIMS = (8, 8, 8, 12)
V = int(np.prod(DIMS))


def _ctx(prec=gfx.PREC_MIXED, eps=0.5, seed=3):
    c = gfx.Context(DIMS, precision=prec)
    c.set_links(smooth_links(DIMS, eps, seed))
    c.set_trafo(gfx.random_init_reference(351, V))
    return c


@pytest.mark.parametrize("gauge", [gfx.LANDAU, gfx.COULOMB])
def test_df_sweeps_track_fp64(gauge):
    a, b = _ctx(), _ctx()
    a.or_sweeps(5, omega=1.7, gauge=gauge, precision=1)
    b.or_sweeps(5, omega=1.7, gauge=gauge, precision=2)
    ga, gb = a.get_trafo(), b.get_trafo()
    assert np.max(np.abs(ga - gb)) < 1e-12
    # the functional of the double-float result, measured in FP64
    fa, fb = a.functional(gauge=gauge), b.functional(gauge=gauge)
    assert fb.F == pytest.approx(fa.F, rel=1e-13)


@pytest.mark.parametrize("gauge,crit,eps", [(gfx.LANDAU, gfx.CRIT_THETA, 1e-14),
                                            (gfx.COULOMB, gfx.CRIT_THETA_SLICES, 1e-15)])
def test_df_polish_reaches_target_and_copy(gauge, crit, eps):
    kw = dict(maxit=8000, eps=eps, checkinterval=20, omega=1.7, gauge=gauge, criterion=crit,
              checkinterval_double=5)
    res = {}
    for polish in (0, 1):
        c = _ctx()
        r = c.overrelax(polish=polish, **kw)
        assert r.converged
        value = r.final_values.theta if crit == gfx.CRIT_THETA else r.final_values.theta_slice_max
        assert value < eps
        f = c.functional(gauge=gauge)  # FP64, independent of the loop
        check = f.theta if crit == gfx.CRIT_THETA else f.theta_slice_max
        assert check < eps
        res[polish] = (r, f)
        c.close()
    r0, f0 = res[0]
    r1, f1 = res[1]
    assert r1.sweeps_polish_df > 0 and r0.sweeps_polish_df == 0
    assert r1.sweeps_polish_df <= r1.sweeps_double
    assert f1.F == pytest.approx(f0.F, abs=1e-12)


def test_df_state_round_trips_through_other_precisions():
    c = _ctx()
    c.or_sweeps(2, omega=1.7, precision=2)   # g now held in double-float
    g_df = c.get_trafo()                     # converted back exactly
    c.or_sweeps(1, omega=1.7, precision=0)   # FP32 from it
    c.or_sweeps(1, omega=1.7, precision=2)   # and back
    assert np.isfinite(c.get_trafo()).all()
    d = _ctx()
    d.or_sweeps(2, omega=1.7, precision=2)
    assert np.array_equal(d.get_trafo(), g_df)  # deterministic
