"""Batched Gribov copies: every copy of every configuration, fixed together in one
device loop, follows the same trajectory as the same start fixed alone (same check
iterations, same FP32/FP64 sweep split, same functional to 1e-13), with the FP64 and
with the rebased FP32 polish."""
import numpy as np
import pytest

from conftest import smooth_links

pytestmark = pytest.mark.gpu

DIMS = [(8, 8, 8, 8), (4, 6, 8, 10)]


def _batch(gfx, prec, ncopies, seed=900):
    b = gfx.Batch(DIMS, ncopies, precision=prec)
    links = [smooth_links(d, 0.3 + 0.1 * c, 50 + c) for c, d in enumerate(DIMS)]
    for c, u in enumerate(links):
        b.set_links(c, u)
    b.random_haar(seed)
    return b, links


@pytest.mark.parametrize("prec,ncopies,polish", [(2, [5, 3], 0), (2, [1, 7], 0), (0, [3, 2], 0),
                                                 (2, [5, 3], 2)])
def test_batch_copies_match_single_contexts(gfx, prec, ncopies, polish):
    b, links = _batch(gfx, prec, ncopies)
    kw = dict(maxit=4000, eps=1e-12 if not polish else 1e-14, checkinterval=20, omega=1.7,
              criterion=gfx.CRIT_THETA, switch_eps=1e-9, checkinterval_double=5, polish=polish)
    res, ms = b.overrelax(**kw)
    assert all(r["converged"] for r in res)
    base = 0
    for c, dims in enumerate(DIMS):
        ctx = gfx.Context(dims, precision=prec)
        ctx.set_links(links[c])
        for k in range(ncopies[c]):
            ctx.random_trafo_haar(900 + base + k)
            r = ctx.overrelax(**kw)
            got = res[base + k]
            assert (got["conf"], got["copy"]) == (c, k)
            assert got["iterations"] == r.iterations
            assert got["sweeps_single"] == r.sweeps_single
            assert got["sweeps_double"] == r.sweeps_double
            assert got["F"] == pytest.approx(r.final_values.F, rel=1e-13)
            assert got["theta"] == pytest.approx(r.final_values.theta, rel=1e-9)
            g_single = ctx.get_trafo()
            assert np.max(np.abs(b.get_trafo(c, k) - g_single)) < 1e-12
        base += ncopies[c]


def test_batch_best_copy(gfx):
    b, links = _batch(gfx, 2, [6, 2])
    res, _ = b.overrelax(maxit=4000, eps=1e-12, checkinterval=20, omega=1.7,
                         criterion=gfx.CRIT_THETA)
    k, f = b.best(0)
    fs = [r["F"] for r in res[:6]]
    assert k == int(np.argmax(fs)) and f == max(fs)


@pytest.mark.parametrize("ncopies", [[5, 3], [2, 7]])
def test_paired_sweeps_bit_identical_to_one_copy_per_thread(gfx, ncopies):
    # two copies per thread in packed FP32 arithmetic give every copy the bits of the
    # one-copy-per-thread kernel, also when the two copies of a pair stop at different
    # checks (the finished copy's lane then repeats its partner)
    kw = dict(maxit=4000, eps=1e-12, checkinterval=20, omega=1.7, criterion=gfx.CRIT_THETA,
              switch_eps=1e-9, checkinterval_double=5, polish=0)
    out = []
    for paired in (1, 0):
        b, _ = _batch(gfx, 2, ncopies)
        b.set_paired(paired)
        res, _ = b.overrelax(**kw)
        out.append((res, [b.get_trafo(c, k) for c in range(2) for k in range(ncopies[c])]))
        b.close()
    (rp, gp), (r1, g1) = out
    assert [r["iterations"] for r in rp] == [r["iterations"] for r in r1]
    assert len({r["sweeps_single"] for r in rp}) > 1  # copies leave the FP32 phase apart
    assert [r["F"] for r in rp] == [r["F"] for r in r1]
    for a, b in zip(gp, g1):
        assert np.array_equal(a, b)


def _heatbath_links(gfx, dims, beta, sweeps, seed, mt_params):
    V = int(np.prod(dims))
    c = gfx.Context(dims, precision=gfx.PREC_MIXED)
    c.set_links(gfx.unit_init(4 * V))
    c.mt_load_params(mt_params)
    c.mt_seed(seed)
    c.mt_init(2 * V, 8 * V)
    c.thermalize(beta, sweeps, variant=gfx.HB_KENNEDY_PENDLETON)
    u = c.get_links()
    c.close()
    return u


def test_batch_at_c4_sizes_matches_single_solves(gfx, mt_params):
    # the C4 lattices themselves (16^4 and 24^4, whose slices hold whole 128-site blocks,
    # so the FP32-phase checks read the odd sites), a few copies each, on Kennedy-
    # Pendleton heatbath links at beta 6.0 / 6.2: every copy as its single mixed solve
    # (the same checks, the same sweep split, g to 1e-12)
    dims = [(16, 16, 16, 16), (24, 24, 24, 24)]
    ncopies = [3, 2]
    b = gfx.Batch(dims, ncopies, precision=gfx.PREC_MIXED)
    links = [_heatbath_links(gfx, d, beta, 40, 70 + c, mt_params)
             for c, (d, beta) in enumerate(zip(dims, (6.0, 6.2)))]
    for c, u in enumerate(links):
        b.set_links(c, u)
    b.random_haar(4000)
    kw = dict(maxit=10000, eps=1e-12, checkinterval=25, omega=1.7, criterion=gfx.CRIT_THETA,
              polish=2)
    res, _ = b.overrelax(**kw)
    assert all(r["converged"] for r in res), [(r["iterations"], r["theta"]) for r in res]
    base = 0
    for c, d in enumerate(dims):
        ctx = gfx.Context(d, precision=gfx.PREC_MIXED)
        ctx.set_links(links[c])
        for k in range(ncopies[c]):
            ctx.random_trafo_haar(4000 + base + k)
            r = ctx.overrelax(**kw)
            got = res[base + k]
            assert (got["iterations"], got["sweeps_single"], got["sweeps_double"]) == \
                (r.iterations, r.sweeps_single, r.sweeps_double)
            assert got["F"] == pytest.approx(r.final_values.F, rel=1e-13)
            assert got["theta"] == pytest.approx(r.final_values.theta, rel=1e-9)
            assert np.max(np.abs(b.get_trafo(c, k) - ctx.get_trafo())) < 1e-12
        ctx.close()
        base += ncopies[c]
