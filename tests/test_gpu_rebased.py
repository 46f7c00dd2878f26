"""Rebased FP32 polish sweeps (g = (1 + a) g_c, cudagfx_gb300/csrc/gfx_rebased.cu): near a
fixed point they follow the FP64 sweeps far below FP32 rounding, their theta agrees
with the FP64 measurement, the base is kept and renewed as the state calls for, and a
mixed solve polished with them reaches the FP64-confirmed target and the same gauge
copy as the FP64 polish."""
import numpy as np
import pytest

import cudagfx_gb300 as gfx
from conftest import smooth_links

pytestmark = pytest.mark.gpu

DIMS = (8, 8, 8, 12)
V = int(np.prod(DIMS))
CRIT = {gfx.LANDAU: gfx.CRIT_THETA, gfx.COULOMB: gfx.CRIT_THETA_SLICES}


def _ctx(g=None, links_seed=3):
    c = gfx.Context(DIMS, precision=gfx.PREC_MIXED)
    c.set_links(smooth_links(DIMS, 0.5, links_seed))
    c.set_trafo(gfx.random_init_reference(351, V) if g is None else g)
    return c


_near = {}


def _near_converged(gauge):
    """g at the FP32 plateau of a fixed point: the state the polish starts from"""
    if gauge not in _near:
        c = _ctx()
        c.overrelax(maxit=8000, eps=1e-11, checkinterval=20, omega=1.7, gauge=gauge,
                    criterion=CRIT[gauge], polish=0)
        _near[gauge] = c.get_trafo()
        c.close()
    return _near[gauge]


@pytest.mark.parametrize("gauge", [gfx.LANDAU, gfx.COULOMB])
def test_rebased_sweeps_track_fp64(gauge):
    g0 = _near_converged(gauge)
    out = {}
    for prec in (0, 1, 3):
        c = _ctx(g0)
        c.or_sweeps(3, omega=1.7, gauge=gauge, precision=prec)
        out[prec] = c.get_trafo()
        c.close()
    d_rebased = np.max(np.abs(out[3] - out[1]))
    d_fp32 = np.max(np.abs(out[0] - out[1]))
    assert d_rebased < 1e-11
    assert d_fp32 > 1e-9              # FP32 sweeps differ by their rounding
    assert d_rebased < d_fp32 / 100


@pytest.mark.parametrize("gauge", [gfx.LANDAU, gfx.COULOMB])
def test_rebased_functional_matches_fp64(gauge):
    c = _ctx(_near_converged(gauge))
    c.or_sweeps(2, omega=1.7, gauge=gauge, precision=3)  # a != 0 on the base
    fr = c.functional(gauge=gauge, precision=3)
    f64 = c.functional(gauge=gauge, precision=1)         # g composed in FP64
    assert fr.theta == pytest.approx(f64.theta, rel=1e-4)
    assert fr.theta_slice_max == pytest.approx(f64.theta_slice_max, rel=1e-4)
    assert fr.F == pytest.approx(f64.F, abs=1e-11)
    # FP32 arithmetic on X itself does not resolve theta here
    f32 = c.functional(gauge=gauge, precision=0)
    assert abs(f32.theta - f64.theta) > 100 * abs(fr.theta - f64.theta)


def test_rebased_calls_continue_on_their_base():
    g0 = _near_converged(gfx.LANDAU)
    a, b = _ctx(g0), _ctx(g0)
    a.or_sweeps(2, omega=1.7, precision=3)
    a.or_sweeps(2, omega=1.7, precision=3)
    b.or_sweeps(4, omega=1.7, precision=3)
    assert np.array_equal(a.get_trafo(), b.get_trafo())


def test_rebased_base_follows_link_changes():
    """new links: the next rebased sweep takes a new base from g = (1 + a) g_c"""
    g0 = _near_converged(gfx.LANDAU)
    links2 = smooth_links(DIMS, 0.5, 4)
    a = _ctx(g0)
    a.or_sweeps(2, omega=1.7, precision=3)
    a.set_links(links2)
    a.or_sweeps(2, omega=1.7, precision=3)
    b = _ctx(g0)
    b.or_sweeps(2, omega=1.7, precision=3)
    g_mid = b.get_trafo()
    c = _ctx(g_mid, links_seed=4)
    c.or_sweeps(2, omega=1.7, precision=3)
    assert np.array_equal(a.get_trafo(), c.get_trafo())


def test_rebased_state_kept_by_tuner_and_checkpoint(tmp_path):
    g0 = _near_converged(gfx.LANDAU)
    a, b = _ctx(g0), _ctx(g0)
    for c in (a, b):
        c.or_sweeps(2, omega=1.7, precision=3)
    a.autotune()
    path = str(tmp_path / "ck.lime")
    a.checkpoint_save(path)
    ga, gb = a.get_trafo(), b.get_trafo()
    assert np.array_equal(ga, gb)
    d = gfx.Context(DIMS, precision=gfx.PREC_MIXED)
    d.checkpoint_load(path)
    assert np.array_equal(d.get_trafo(), gb)


@pytest.mark.parametrize("gauge,eps", [(gfx.LANDAU, 1e-14), (gfx.COULOMB, 1e-15)])
def test_rebased_polish_reaches_target_and_copy(gauge, eps):
    crit = CRIT[gauge]
    kw = dict(maxit=8000, eps=eps, checkinterval=20, omega=1.7, gauge=gauge, criterion=crit,
              checkinterval_double=5)
    res = {}
    for polish in (0, 2):
        c = _ctx()
        r = c.overrelax(polish=polish, **kw)
        assert r.converged
        value = r.final_values.theta if crit == gfx.CRIT_THETA else r.final_values.theta_slice_max
        assert value < eps
        f = c.functional(gauge=gauge)  # FP64, independent of the loop
        check = f.theta if crit == gfx.CRIT_THETA else f.theta_slice_max
        assert check < eps
        res[polish] = (r, f, c.history())
        c.close()
    (r0, f0, _), (r2, f2, h2) = res[0], res[2]
    assert r2.sweeps_polish_fp32 > 0 and r0.sweeps_polish_fp32 == 0
    assert r2.sweeps_polish_df == 0
    assert r2.sweeps_polish_fp32 <= r2.sweeps_double
    assert f2.F == pytest.approx(f0.F, abs=1e-12)
    # the polish needs about as many sweeps as the FP64 one
    assert r2.sweeps_double <= 1.5 * r0.sweeps_double + 20
    assert h2[-1]["phase"] == 1


def test_rebased_polish_rejects_bad_setting():
    c = _ctx()
    with pytest.raises(gfx.GfxError):
        c.overrelax(maxit=100, eps=1e-12, checkinterval=20, polish=3)
