"""The Kennedy-Pendleton link heatbath (gfx_heatbath.cu, variant 1) against the oracle's
restatement of the same algorithm (orc_link_heatbath_halfsweep_kp), as distributions
over twister seeds.

Both chains draw the same uniforms (the twister bank is bit-exact) and gaussians that
agree to ~1e-6, but a trial decided at the acceptance boundary can fall the other way
and the chains then separate, so a heatbath is compared statistically: for each of 16
seeds, 4^4 at beta 6.0 from a cold start, 30 sweeps, the plaquette after each sweep;
per seed the mean and the variance over sweeps 10..29.  The means over seeds of both
must agree within 3 standard errors.  The fields are 38 outputs per twister (a
multiple of 19, so the stream is the twister's canonical one)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

DIMS = (4, 4, 4, 4)
V = 256
SEEDS = list(range(500, 516))
NSWEEP, NSKIP = 30, 10
NFIELD = 4096 * 38


def _gpu_chain(gfx, params, seed, beta):
    c = gfx.Context(DIMS)
    c.set_links(gfx.unit_init(4 * V))
    c.mt_load_params(params)
    c.mt_seed(seed)
    c.mt_init(NFIELD, NFIELD)
    p = c.thermalize(beta, NSWEEP, checkint=1, variant=gfx.HB_KENNEDY_PENDLETON)
    c.close()
    return np.asarray(p)


def _oracle_chain(gfx, oracle, params, seed, beta):
    lat = oracle.lattice(DIMS)
    gf12 = oracle.to2v(gfx.unit_init(4 * V))
    m = oracle.mt_new(params, seeds=oracle.glibc_rand(seed, 4096).astype(np.uint32))
    ng = nu = oracle.mt_nper(NFIELD)
    fields = oracle.mt_init_fields(m, ng, nu)
    plaq, _ = oracle.thermalize(lat, gf12, m, fields, ng, nu, beta, NSWEEP, variant=1)
    return plaq


def _compare(a, b, what):
    k = len(a)
    se = np.sqrt(np.var(a, ddof=1) / k + np.var(b, ddof=1) / k)
    assert abs(np.mean(a) - np.mean(b)) <= 3 * se + 1e-12, (what, np.mean(a), np.mean(b), se)


@pytest.mark.parametrize("beta", [6.0, 2.0])
def test_kp_heatbath_plaquette_distribution_matches_oracle(gfx, oracle, mt_params, beta):
    gm, gv, om, ov = [], [], [], []
    for seed in SEEDS:
        pg = _gpu_chain(gfx, mt_params, seed, beta)[NSKIP:]
        po = _oracle_chain(gfx, oracle, mt_params, seed, beta)[NSKIP:]
        gm.append(pg.mean())
        gv.append(pg.var(ddof=1))
        om.append(po.mean())
        ov.append(po.var(ddof=1))
    _compare(np.array(gm), np.array(om), "plaquette mean")
    _compare(np.array(gv), np.array(ov), "plaquette variance")
    # the Wilson-action plaquette band on 4^4: ~0.60 at beta 6 (0.5937 in large volume),
    # ~0.13 at beta 2 (strong coupling: beta/18 to leading order)
    lo, hi = (0.57, 0.63) if beta == 6.0 else (0.09, 0.17)
    assert lo < np.mean(gm) < hi
