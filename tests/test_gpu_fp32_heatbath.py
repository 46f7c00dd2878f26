"""FP32-arithmetic heatbaths: the SA heatbath of g in FP32 sweeps and the FP32
thermalization (gfx_therm_params.precision = 1).  With the same random fields they
follow their FP64 counterparts to FP32 rounding, except at accept/reject decisions
that sit at the rounding boundary, and the FP32 thermalization samples the Wilson
action: the beta = 6.0 plaquette, links in SU(3) to ~1e-14 (the new link is
reunitarized in double-float arithmetic)."""
import numpy as np
import pytest

import cudagfx_gb300 as gfx
from conftest import haar, smooth_links

pytestmark = pytest.mark.gpu

DIMS = (8, 8, 8, 8)
V = 4096


def _close_fp32(got, want, tol=2e-5, max_flips=0.01):
    d = np.max(np.abs(np.asarray(got).reshape(-1, 18) - np.asarray(want).reshape(-1, 18)), axis=1)
    flips = d > tol
    assert flips.mean() <= max_flips, (flips.sum(), d.max())
    return d


def _mt(c, mt_params, seed, ng, nu):
    c.mt_load_params(mt_params)
    c.mt_seed(seed)
    c.mt_init(ng, nu)


def test_fp32_sa_halfsweep_follows_fp64(mt_params):
    u, g = smooth_links(DIMS, 0.35, 25), haar(V, 26)
    out = []
    for prec in (0, 1):
        c = gfx.Context(DIMS, precision=gfx.PREC_MIXED)
        c.set_links(u)
        c.set_trafo(g)
        _mt(c, mt_params, 7, V // 2, 2 * V)
        for parity, beta in ((0, 1.0 / 1.45), (1, 1.0 / 0.3)):
            c.sa_halfsweep(parity, beta, precision=prec)
            c.mt_update()
        out.append(c.get_trafo())
        c.close()
    d = _close_fp32(out[0], out[1])
    assert np.median(d) < 1e-6


@pytest.mark.parametrize("variant", [gfx.HB_REFERENCE, gfx.HB_KENNEDY_PENDLETON])
def test_fp32_thermalization_follows_fp64(mt_params, variant):
    out = []
    for prec in (0, 1):
        c = gfx.Context(DIMS, precision=gfx.PREC_MIXED)
        c.set_links(smooth_links(DIMS, 0.5, 29))
        _mt(c, mt_params, 11, 2 * V, 8 * V)
        c.thermalize(6.0, 1, variant=variant, precision=prec)
        out.append(c.get_links())
        c.close()
    d = _close_fp32(out[0], out[1])
    assert np.median(d) < 1e-6


def test_fp32_thermalization_samples_wilson_action(mt_params):
    """as test_kennedy_pendleton_heatbath_reaches_beta6_plaquette, FP32 arithmetic"""
    c = gfx.Context(DIMS, precision=gfx.PREC_MIXED)
    c.set_links(gfx.unit_init(4 * V))
    _mt(c, mt_params, 2024, 38 * V, 152 * V)
    plaq = c.thermalize(6.0, 300, checkint=1, variant=gfx.HB_KENNEDY_PENDLETON, precision=1)
    mean = float(np.mean(plaq[150:]))
    assert 0.585 < mean < 0.605, mean
    u = c.get_links().reshape(-1, 3, 3, 2)
    m = u[..., 0] + 1j * u[..., 1]
    assert np.max(np.abs(m @ np.conj(np.swapaxes(m, 1, 2)) - np.eye(3))) < 1e-12
    # the FP32 copy the sweeps read is the rounding of the FP64 links
    f32, f64 = c.functional(precision=0), c.functional(precision=1)
    assert f32.F == pytest.approx(f64.F, rel=1e-6)


def test_fp32_thermalization_keeps_8_real_layout(mt_params):
    c = gfx.Context(DIMS, precision=gfx.PREC_MIXED)
    c.set_links(smooth_links(DIMS, 0.5, 31))
    t = c.tuning()
    c.set_tuning(block=t["block"], staging=t["staging"], link_reals32=8)
    _mt(c, mt_params, 13, 2 * V, 8 * V)
    c.thermalize(6.0, 2, variant=gfx.HB_KENNEDY_PENDLETON, precision=1)
    assert c.tuning()["link_reals32"] == 8
    f32, f64 = c.functional(precision=0), c.functional(precision=1)
    assert f32.F == pytest.approx(f64.F, rel=1e-5)


def test_fp32_thermalization_needs_fp32_copy(mt_params):
    c = gfx.Context(DIMS, precision=gfx.PREC_DOUBLE)
    c.set_links(gfx.unit_init(4 * V))
    _mt(c, mt_params, 1, 2 * V, 8 * V)
    with pytest.raises(gfx.GfxError):
        c.thermalize(6.0, 1, precision=1)
