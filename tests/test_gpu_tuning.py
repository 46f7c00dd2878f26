"""Launch tuning: every block size, every staging mode (plain loads, L2 bulk prefetch,
odd half-sweep in reverse block order, L2 eviction priorities)
and both FP64 link layouts give bit-identical sweeps; gfx_autotune leaves the fields as it found them, its
choice reproduces the untuned solve exactly, and its cache file round-trips."""
import numpy as np
import pytest

import cudagfx_gb300 as gfx
from conftest import smooth_links

pytestmark = pytest.mark.gpu

DIMS = (8, 8, 8, 12)
V = int(np.prod(DIMS))


def _ctx(prec=gfx.PREC_MIXED):
    c = gfx.Context(DIMS, precision=prec)
    c.set_links(gfx.random_init_haar(5, 4 * V))
    c.set_trafo(gfx.random_init_reference(351, V))
    return c


@pytest.mark.parametrize("prec", [0, 1])
def test_launch_variants_are_bit_identical(prec):
    ref = _ctx()
    ref.or_sweeps(3, omega=1.7, precision=prec)
    want = ref.get_trafo()
    ref.close()
    for nr in ((12, 18) if prec == 1 else (12,)):
        for wide in ((0, 1) if prec == 0 else (1,)):
            for block in (32, 64, 96, 128, 192, 256):
                for pf in (0, 1, 2, 3, 4):
                    c = _ctx()
                    c.set_tuning(block=(block, block), staging=(pf, pf), link_reals64=nr,
                                 wide_regs=wide)
                    c.or_sweeps(3, omega=1.7, precision=prec)
                    assert np.array_equal(c.get_trafo(), want), (nr, wide, block, pf)
                    c.close()


def test_fp32_staging_modes_bit_identical_in_coulomb_gauge():
    # the three-direction FP32 kernels of every staging mode, both register budgets
    ref = _ctx()
    ref.or_sweeps(3, omega=1.7, gauge=gfx.COULOMB, precision=0)
    want = ref.get_trafo()
    ref.close()
    for wide in (0, 1):
        for pf in (0, 1, 2, 3, 4):
            c = _ctx()
            c.set_tuning(block=(64, 64), staging=(pf, pf), wide_regs=wide)
            c.or_sweeps(3, omega=1.7, gauge=gfx.COULOMB, precision=0)
            assert np.array_equal(c.get_trafo(), want), (wide, pf)
            c.close()


def test_autotune_keeps_fields_and_reproduces_solve(tmp_path):
    kw = dict(maxit=3000, eps=1e-12, checkinterval=20, omega=1.7, criterion=gfx.CRIT_THETA)
    a = _ctx()
    g0 = a.get_trafo()
    u0 = a.get_links()
    ra = a.overrelax(**kw)
    ga = a.get_trafo()
    b = _ctx()
    t = b.autotune(expected_sweeps=1000, cache_path=str(tmp_path / "tune.txt"))
    assert t["block"][0] in (64, 128, 192, 256) and t["staging"][1] in (0, 1, 2) and t["staging"][0] in range(5)
    assert t["link_reals64"] in (12, 18) and 5 <= t["checkinterval"] <= 100
    assert t["link_reals32"] in (12, 8) and t["wide_regs"] in (0, 1)
    assert t["sweep_ms"][0] > 0 and t["check_ms"][1] > 0
    assert np.array_equal(b.get_trafo(), g0)
    assert np.max(np.abs(b.get_links() - u0)) < 1e-15
    # every choice but the 8-real FP32 links is bit-identical (those are checked apart)
    b.set_tuning(block=t["block"], staging=t["staging"], link_reals64=t["link_reals64"],
                 link_reals32=12)
    rb = b.overrelax(**kw)
    assert (rb.iterations, rb.sweeps_single, rb.sweeps_double) == \
        (ra.iterations, ra.sweeps_single, ra.sweeps_double)
    assert rb.final_values.F == ra.final_values.F
    assert np.array_equal(b.get_trafo(), ga)
    a.close()
    b.close()


def test_autotune_cache_hit_applies_stored_settings(tmp_path):
    path = str(tmp_path / "tune.txt")
    a = _ctx()
    t1 = a.autotune(cache_path=path)
    a.close()
    lines = open(path).read().splitlines()
    assert len(lines) == 1 and "8x8x8x12" in lines[0]
    b = _ctx()
    t2 = b.autotune(cache_path=path)
    assert (t2["block"], t2["staging"], t2["link_reals64"], t2["link_reals32"]) == \
        (t1["block"], t1["staging"], t1["link_reals64"], t1["link_reals32"])
    assert b.tuning()["block"] == t1["block"]
    assert len(open(path).read().splitlines()) == 1  # a hit appends nothing
    b.close()


def test_set_tuning_rejects_bad_settings():
    c = _ctx()
    for bad in (dict(block=(48, 128)), dict(block=(128, 512)), dict(staging=(5, 0)), dict(staging=(0, -1)),
                dict(link_reals64=8), dict(link_reals32=18)):
        with pytest.raises(gfx.GfxError):
            c.set_tuning(**bad)
    c.close()


@pytest.mark.parametrize("prec", [gfx.PREC_DOUBLE, gfx.PREC_MIXED])
def test_checkinterval_near_shortens_the_end(prec):
    """Below switch_eps the loop continues with checkinterval_near sweeps per check:
    the same sweeps up to that point, the shorter spacing after it, and convergence."""
    kw = dict(maxit=4000, eps=1e-12, checkinterval=40, omega=1.7, criterion=gfx.CRIT_THETA,
              switch_eps=1e-8)
    links = smooth_links(DIMS, 0.4, 77)
    a = _ctx(prec)
    a.set_links(links)
    ra = a.overrelax(**kw)
    ha = a.history()
    b = _ctx(prec)
    b.set_links(links)
    rb = b.overrelax(checkinterval_near=4, **kw)
    hb = b.history()
    assert ra.converged and rb.converged
    assert rb.final_values.theta < 1e-12
    first = next(k for k, h in enumerate(ha) if h["theta"] < 1e-8)
    assert [h["iter"] for h in hb[:first + 1]] == [h["iter"] for h in ha[:first + 1]]
    # the near interval, or the FP64 polish (its first check verifies at the same iteration)
    assert hb[first + 1]["iter"] - hb[first]["iter"] in (0, 2, 4)
    assert rb.sweeps <= ra.sweeps
    a.close()
    b.close()


def test_fp32_link8_matches_link12():
    """The 8-real FP32 links (GF_8 parameters, exact rows kept for the links the form
    cannot hold) give the 12-real FP32 sweep to FP32 rounding, also on unit links,
    which all take the exact rows."""
    for links, tol in ((gfx.random_init_haar(8, 4 * V), 3e-5), (gfx.unit_init(4 * V), 1e-5)):
        out = []
        for nr32 in (12, 8):
            c = _ctx()
            c.set_links(links)
            c.set_tuning(link_reals32=nr32)
            assert c.tuning()["link_reals32"] == nr32
            c.or_sweeps(3, omega=1.7, precision=0)
            out.append(c.get_trafo())
            c.close()
        assert np.max(np.abs(out[0] - out[1])) <= tol


def test_fp32_link8_solve_reaches_the_same_copy():
    links = smooth_links(DIMS, 0.9, 21)  # far from the identity: the 8-real form is used
    kw = dict(maxit=6000, eps=1e-12, checkinterval=20, omega=1.7, criterion=gfx.CRIT_THETA)
    res = []
    for nr32 in (12, 8):
        c = _ctx()
        c.set_links(links)
        c.set_tuning(link_reals32=nr32)
        r = c.overrelax(**kw)
        assert r.converged and r.final_values.theta < 1e-12
        res.append(r.final_values.F)
        c.close()
    assert abs(res[0] - res[1]) < 1e-11


@pytest.mark.parametrize("dims,want", [((32, 32, 32, 32), 4), ((24, 24, 24, 24), 2),
                                       ((32, 32, 32, 48), 2)])
def test_default_staging_keeps_g_in_l2_where_it_fits(dims, want):
    # the FP32 sweep starts with g kept in L2 (staging 4) when its 48 B per site fit in
    # half of the L2 but links and g (240 B per site) do not: on GB300's 126 MB L2 that
    # is 32^4, not 24^4 (all of it fits) nor 32^3 x 48 (g is 75 MB)
    c = gfx.Context(dims, precision=gfx.PREC_MIXED)
    assert c.tuning()["staging"] == [want, 2]
    c.close()
