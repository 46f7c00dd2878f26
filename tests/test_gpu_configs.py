"""BASELINE's workloads as GPU test cases at their lattice sizes (size-independent
checks: convergence verified in FP64, mixed vs all-FP64 agreement, gauge invariants).

  C2  16^3x32, beta 6.0 (500 KP heatbath sweeps, seed 7): SA 2000 steps T 1.45 -> 0.01
      (linear), 3 microcanonical steps per heatbath step, then OR omega 1.7 to
      theta < 1e-12, mixed against all-FP64 from the same annealed g.
  C3  32^4, beta 6.0 (seed 42), Coulomb gauge: every time slice to theta_t < 1e-15,
      mixed (rebased FP32 polish) against all-FP64; plaquette and Polyakov loop
      unchanged to 1e-12.
  C5  48^3x96, beta 6.2, FP64 18-real links: SA then mixed OR (rebased FP32 polish,
      FP64-confirmed) to theta < 1e-14.  The
      thermalization (20 instead of 1000 heatbath sweeps) and the annealing (50 instead
      of 1000 steps) are shortened to keep the test under a minute; the lattice size,
      link layout and target are the workload's.
C1 (8^4) is the smoke test and the parity tests; C4 (Gribov batch) is
tests/test_gpu_batch.py and bench.py."""
import numpy as np
import pytest

import cudagfx_gb300 as gfx

pytestmark = pytest.mark.gpu


def _thermalized(dims, beta, sweeps, seed, mt_params, link_reals=12):
    V = int(np.prod(dims))
    c = gfx.Context(dims, precision=gfx.PREC_MIXED, link_reals=link_reals)
    c.set_links(gfx.unit_init(4 * V))
    c.mt_load_params(mt_params)
    c.mt_seed(seed)
    c.mt_init(2 * V, 8 * V)
    c.thermalize(beta, sweeps, variant=gfx.HB_KENNEDY_PENDLETON)
    return c


def test_c2_annealing_then_overrelaxation(mt_params):
    dims = (16, 16, 16, 32)
    V = int(np.prod(dims))
    src = _thermalized(dims, 6.0, 500, 7, mt_params)
    links = src.get_links()
    assert 0.58 < src.plaquette() < 0.61
    src.close()
    sa = gfx.Context(dims, precision=gfx.PREC_DOUBLE)
    sa.set_links(links)
    sa.set_trafo(gfx.random_init_reference(351, V))
    f0 = sa.functional().F
    sa.mt_load_params(mt_params)
    sa.mt_seed(7)
    sa.mt_init(2 * V, 8 * V)
    fs = sa.simanneal(0.01, 1.45, 2000, expo=-1.0, checkint=500, nmicro=3)
    assert fs.F > f0 + 0.1  # annealing raised the functional from the random start
    g_sa = sa.get_trafo()
    kw = dict(maxit=20000, eps=1e-12, checkinterval=50, omega=1.7, criterion=gfx.CRIT_THETA)
    r64 = sa.overrelax(**kw)
    mixed = gfx.Context(dims, precision=gfx.PREC_MIXED)
    mixed.set_links(links)
    mixed.set_trafo(g_sa)
    r = mixed.overrelax(**kw)
    assert r.converged and r64.converged
    assert r.final_values.theta < 1e-12 and r64.final_values.theta < 1e-12
    # the same gauge copy: the functional agrees far below the copies' spread
    assert abs(r.final_values.F - r64.final_values.F) < 1e-10
    assert r.sweeps_double < r.sweeps // 10


def test_c3_coulomb_slices(mt_params):
    dims = (32, 32, 32, 32)
    V = int(np.prod(dims))
    src = _thermalized(dims, 6.0, 200, 42, mt_params)
    links = src.get_links()
    plaq0, poly0 = src.plaquette(), src.polyakov()
    src.close()
    g0 = gfx.random_init_reference(351, V)
    kw = dict(maxit=20000, eps=1e-15, checkinterval=50, omega=1.7, gauge=gfx.COULOMB,
              criterion=gfx.CRIT_THETA_SLICES, polish=2)
    out = {}
    for prec in (gfx.PREC_MIXED, gfx.PREC_DOUBLE):
        c = gfx.Context(dims, precision=prec)
        c.set_links(links)
        c.set_trafo(g0)
        r = c.overrelax(**kw)
        assert r.converged and r.final_values.theta_slice_max < 1e-15
        f = c.functional(gauge=gfx.COULOMB, precision=1)
        c.apply_trafo()
        assert c.plaquette() == pytest.approx(plaq0, rel=1e-12)
        assert abs(c.polyakov() - poly0) < 1e-12
        out[prec] = (r, f)
        c.close()
    (rm, fm), (rd, fd) = out[gfx.PREC_MIXED], out[gfx.PREC_DOUBLE]
    assert abs(fm.F - fd.F) < 1e-11
    assert rm.ms < rd.ms  # the mixed path is the faster one


def test_c5_large_lattice_fp64_links(mt_params):
    dims = (48, 48, 48, 96)
    V = int(np.prod(dims))
    c = _thermalized(dims, 6.2, 20, 2024, mt_params, link_reals=18)
    plaq0 = c.plaquette()
    c.set_trafo(gfx.random_init_reference(351, V))
    c.simanneal(0.01, 1.0, 50, expo=-1.0, checkint=50, nmicro=3)
    r = c.overrelax(maxit=20000, eps=1e-14, checkinterval=100, omega=1.7,
                    criterion=gfx.CRIT_THETA, checkinterval_near=10, polish=2)
    assert r.converged and r.final_values.theta < 1e-14
    assert r.sweeps_double > 0  # below the FP32 floor only FP64 sweeps get there
    f = c.functional(precision=1)
    assert f.theta < 1e-14
    c.apply_trafo()
    assert c.plaquette() == pytest.approx(plaq0, rel=1e-12)
