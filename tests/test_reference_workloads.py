"""Parity on the 8^4 gauge-fixing workload and on the annealing statistics, against the
reference's own CUDA code (tests/golden/reference_workloads.npz, written by
tests/golden/make_reference_fixtures.py --workloads on a GB300).

C1: 8^4 links from this repository's heatbath at beta 6.0 (200 sweeps from a cold
start, MT seed 1234) -- the reference's heatbath update (C1R) and Kennedy-Pendleton
(C1K) -- and the reference's random start (RandSeed 351).  The reference's kernels
ran overrelaxation at omega 1.7 to theta < 1e-12 (checks every 10 sweeps) and its
own overrelax_gauge at omega 1.68 to maxdAdA < 1e-10 (overrelax.cu:677-823).  The
FP64 solve here must stop at the same check with F equal to 1e-12; the mixed solve
must reach theta < 1e-12 on the same gauge copy (F to 1e-12).

SA: 16 twister seeds of simannealing_gauge (simulated_annealing.cu:309-476) on the
C1K links.  Both sides draw the same random numbers, but a single-precision
accept/reject decision that falls the other way (dev_get_a0 runs in float)
separates the chains, so the functional and dAdA after annealing are compared as
distributions over the seeds: means within 3 standard errors."""
import hashlib
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
_FX_PATH = os.path.join(HERE, "golden", "reference_workloads.npz")
FX = np.load(_FX_PATH) if os.path.exists(_FX_PATH) else None
pytestmark = [pytest.mark.gpu,
              pytest.mark.skipif(FX is None, reason="reference_workloads.npz not generated")]
D8 = (8, 8, 8, 8)
V8 = 8 ** 4


def _sha(a):
    return np.frombuffer(hashlib.sha256(np.ascontiguousarray(a).tobytes()).digest(),
                         dtype=np.uint8)


def _params():
    import oracle as orc
    p = orc.load_mt_params()
    if p is None:
        pytest.skip("the reference's twister parameter file is not present")
    return p


_LINKS = {}


def c1_links(gfx, tag):
    """8^4 beta 6.0 heatbath links (200 sweeps from cold, MT seed 1234), checked against
    the SHA-256 the fixture stored"""
    if tag not in _LINKS:
        variant = gfx.HB_REFERENCE if tag == "C1R" else gfx.HB_KENNEDY_PENDLETON
        c = gfx.Context(D8)
        c.set_links(gfx.unit_init(4 * V8))
        c.mt_load_params(_params())
        c.mt_seed(1234)
        c.mt_init(2 * V8, 8 * V8)
        c.thermalize(6.0, 200, variant=variant)
        u = np.ascontiguousarray(c.get_links())
        c.close()
        assert np.array_equal(_sha(u), FX[tag + "_links_sha"]), \
            "the heatbath no longer gives the fixture's links; regenerate the fixture"
        _LINKS[tag] = u
    return _LINKS[tag]


def _solve(gfx, tag, precision, **kw):
    ctx = gfx.Context(D8, precision=precision)
    ctx.set_links(c1_links(gfx, tag))
    ctx.set_trafo(gfx.random_init_reference(351, V8))
    r = ctx.overrelax(maxit=20000, **kw)
    ctx.close()
    return r


@pytest.mark.parametrize("tag", ["C1R", "C1K"])
def test_c1_fp64_theta_solve_matches_reference(gfx, tag):
    want = FX[tag + "_theta"]
    assert want[0] > 0
    r = _solve(gfx, tag, gfx.PREC_DOUBLE, eps=1e-12, checkinterval=10, omega=1.7,
               criterion=gfx.CRIT_THETA)
    assert r.converged and r.iterations == int(want[0])
    assert r.final_values.F == pytest.approx(want[1], rel=1e-12)
    assert r.final_values.theta < 1e-12
    assert abs(r.final_values.dAdA - want[2]) < 3e-13


@pytest.mark.parametrize("tag", ["C1R", "C1K"])
@pytest.mark.parametrize("polish", [2, 0])
def test_c1_mixed_theta_solve_reaches_reference_copy(gfx, tag, polish):
    want = FX[tag + "_theta"]
    r = _solve(gfx, tag, gfx.PREC_MIXED, eps=1e-12, checkinterval=10, omega=1.7,
               criterion=gfx.CRIT_THETA, polish=polish)
    assert r.converged and r.final_values.theta < 1e-12
    assert r.sweeps_single > 0
    # the same gauge copy as the reference's FP64 solve
    assert r.final_values.F == pytest.approx(want[1], rel=1e-12)


@pytest.mark.parametrize("tag", ["C1R", "C1K"])
def test_c1_stock_loop_matches_reference(gfx, tag):
    want = FX[tag + "_stock"]
    assert want[0] > 0
    r = _solve(gfx, tag, gfx.PREC_DOUBLE, eps=1e-10, checkinterval=10, omega=1.68,
               criterion=gfx.CRIT_MAXDADA)
    assert r.iterations == int(want[0])
    assert r.final_values.F == pytest.approx(want[1], rel=1e-12)
    assert r.final_values.dAdA == pytest.approx(want[2], rel=1e-6)
    assert r.final_values.maxdAdA == pytest.approx(want[3], rel=1e-6)


def test_simanneal_statistics_match_reference(gfx):
    params = _params()
    u = c1_links(gfx, "C1K")
    g0 = gfx.random_init_reference(351, V8)
    seeds = [int(s) for s in FX["SA_seeds"]]
    ref = FX["SA_results"]  # (seed, [FUNC, DADA, maxDADA])
    got = []
    for seed in seeds:
        ctx = gfx.Context(D8)
        ctx.set_links(u)
        ctx.set_trafo(g0)
        ctx.mt_load_params(params)
        ctx.mt_seed(seed)
        ctx.mt_init(V8 // 2, 2 * V8)  # the reference main's field sizes
        ctx.simanneal(0.01, 1.45, 300, expo=-1.0, checkint=300)
        f = ctx.functional()
        got.append([f.F, f.dAdA, f.maxdAdA])
        ctx.close()
    got = np.array(got)
    k = len(seeds)
    assert k >= 16
    for col, name in ((0, "F"), (1, "dAdA")):
        a, b = got[:, col], ref[:, col]
        se = np.sqrt(a.var(ddof=1) / k + b.var(ddof=1) / k)
        assert abs(a.mean() - b.mean()) <= 3 * se + 1e-14, (name, a.mean(), b.mean(), se)
        # and the spread over seeds agrees to a factor that 16 samples resolve
        sa, sb = a.std(ddof=1), b.std(ddof=1)
        assert 0.4 * sb <= sa <= 2.5 * sb + 1e-14, (name, sa, sb)
