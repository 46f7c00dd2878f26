"""Parity against the reference's own CUDA code.

tests/golden/reference_fixtures.npz holds outputs of the reference's GPU kernels and
drivers (cudagaugefix.cu and the files it includes, built for sm_103a with the shim of
oracle/ref_gpu.py) on seeded inputs, produced by tests/golden/make_reference_fixtures.py.
CPU tests pin the oracle to them; GPU tests compare the sm_103a kernels of libgfx."""
import hashlib
import os

import numpy as np
import pytest

from golden_inputs import links_for

HERE = os.path.dirname(os.path.abspath(__file__))
FX = np.load(os.path.join(HERE, "golden", "reference_fixtures.npz"))
D4, D8 = (4, 4, 4, 4), (8, 8, 8, 8)


def _sha(a):
    return np.frombuffer(hashlib.sha256(np.ascontiguousarray(a).tobytes()).digest(),
                         dtype=np.uint8)


def _links(dims, seed, key):
    u = links_for(dims, seed)
    assert np.array_equal(_sha(u), FX[key]), "input generator drifted; regenerate fixtures"
    return u


def _start(gfx, dims, seed, key):
    u = _links(dims, seed, key)
    g = gfx.random_init_reference(351, int(np.prod(dims))).reshape(-1, 18)
    return u, g


# ---------------------------------------------------------------------------- oracle
def test_reference_start_matches(gfx):
    # The fixture was made by the reference's host C compiled on aarch64, where gcc
    # contracts a*b+c into FMA by default; bit-equality with it holds only per
    # platform (tests/test_abi.py checks it against the same-platform build).
    g = gfx.random_init_reference(351, 256).reshape(-1, 18)
    assert np.max(np.abs(g[:, :12] - FX["A_g0"])) < 1e-14


def test_oracle_or_halfsweeps_match_reference_gpu(gfx, oracle):
    u, g = _start(gfx, D4, 101, "A_links_sha")
    lat = oracle.lattice(D4)
    gf12, g12 = oracle.to2v(u), np.ascontiguousarray(g[:, :12])
    oracle.or_halfsweep(lat, gf12, g12, 0, 1.68)
    assert np.max(np.abs(g12 - FX["A_g_even"])) < 1e-13
    oracle.or_halfsweep(lat, gf12, g12, 1, 1.68)
    assert np.max(np.abs(g12 - FX["A_g_sweep1"])) < 1e-13
    oracle.or_sweeps(lat, gf12, g12, 10, 1.68)
    assert np.max(np.abs(g12 - FX["A_g_sweep11"])) < 1e-12
    f = oracle.functional(lat, gf12, g12)
    assert np.allclose([f["F"], f["dAdA"], f["maxdAdA"]], FX["A_functional"], rtol=1e-12)
    assert oracle.plaquette(lat, gf12) == pytest.approx(FX["A_plaquette"][0], rel=1e-14)


def test_oracle_overrelax_gauge_matches_reference_gpu(gfx, oracle):
    u, g = _start(gfx, D8, 202, "B_links_sha")
    lat = oracle.lattice(D8)
    gf12, g12 = oracle.to2v(u), np.ascontiguousarray(g[:, :12])
    it, last = -1, None
    for i in range(3000):
        oracle.or_halfsweep(lat, gf12, g12, 0, 1.68)
        oracle.or_halfsweep(lat, gf12, g12, 1, 1.68)
        if i % 10 == 0:
            last = oracle.functional(lat, gf12, g12)
            if last["maxdAdA"] < 1e-10:
                it = i
                break
    want = FX["B_result"]
    assert it == int(want[0])
    assert last["F"] == pytest.approx(want[1], rel=1e-12)
    assert last["dAdA"] == pytest.approx(want[2], rel=1e-6)
    assert last["maxdAdA"] == pytest.approx(want[3], rel=1e-6)


def test_oracle_twister_uniforms_bit_exact_with_reference_gpu(oracle, mt_params):
    import oracle as orc
    if orc.load_mt_params() is None:
        pytest.skip("the reference's twister parameter file is not present")
    ng, nu = (int(x) for x in FX["C_nper"])
    m = oracle.mt_new(mt_params, seeds=oracle.glibc_rand(1234, 4096).astype(np.uint32))
    g, u = oracle.mt_init_fields(m, ng, nu)
    for step in range(3):
        assert np.array_equal(_sha(u), FX["C_unif_sha_%d" % step]), step
        assert np.max(np.abs(g[:512] - FX["C_gauss_head_%d" % step])) < 2e-4
        g, u = oracle.mt_update_fields(m, ng, nu)


def test_oracle_sa_halfsweeps_match_reference_gpu(gfx, oracle):
    u, g = _start(gfx, D4, 101, "A_links_sha")
    lat = oracle.lattice(D4)
    gf12, g12 = oracle.to2v(u), np.ascontiguousarray(g[:, :12])
    for k, (parity, beta) in enumerate(((0, 1.0 / 1.45), (1, 1.0 / 0.3))):
        oracle.heatbath_halfsweep(lat, gf12, g12, parity, FX["D_gauss_%d" % k],
                                  FX["D_unif_%d" % k], beta)
        d = np.max(np.abs(g12 - FX["D_g_%d" % k]), axis=1)
        # single-precision trial (see test_gpu_parity._heatbath_close)
        assert np.mean(d > 1e-6) <= 0.01, np.sum(d > 1e-6)
        g12[:] = FX["D_g_%d" % k]


# ---------------------------------------------------------------------------- GPU
@pytest.mark.gpu
def test_gpu_or_halfsweeps_match_reference_gpu(gfx):
    u, g = _start(gfx, D4, 101, "A_links_sha")
    ctx = gfx.Context(D4)
    ctx.set_links(u)
    ctx.set_trafo(g)
    ctx.or_halfsweep(0, 1.68)
    got = ctx.get_trafo().reshape(-1, 18)[:, :12]
    assert np.max(np.abs(got - FX["A_g_even"])) < 1e-13
    ctx.or_halfsweep(1, 1.68)
    assert np.max(np.abs(ctx.get_trafo().reshape(-1, 18)[:, :12] - FX["A_g_sweep1"])) < 1e-13
    ctx.or_sweeps(10, 1.68)
    assert np.max(np.abs(ctx.get_trafo().reshape(-1, 18)[:, :12] - FX["A_g_sweep11"])) < 1e-12
    f = ctx.functional()
    assert np.allclose([f.F, f.dAdA, f.maxdAdA], FX["A_functional"], rtol=1e-12)
    assert ctx.plaquette() == pytest.approx(FX["A_plaquette"][0], rel=1e-14)


@pytest.mark.gpu
@pytest.mark.parametrize("use_graph", [1, 0])
def test_gpu_overrelax_gauge_matches_reference_gpu(gfx, use_graph):
    u, g = _start(gfx, D8, 202, "B_links_sha")
    ctx = gfx.Context(D8)
    ctx.set_links(u)
    ctx.set_trafo(g)
    r = ctx.overrelax(maxit=3000, eps=1e-10, checkinterval=10, omega=1.68,
                      criterion=gfx.CRIT_MAXDADA, use_graph=use_graph)
    want = FX["B_result"]
    assert r.iterations == int(want[0])
    assert r.final_values.F == pytest.approx(want[1], rel=1e-12)
    assert r.final_values.dAdA == pytest.approx(want[2], rel=1e-6)
    assert r.final_values.maxdAdA == pytest.approx(want[3], rel=1e-6)


@pytest.mark.gpu
def test_gpu_twister_bank_matches_reference_gpu(gfx):
    import oracle as orc
    params = orc.load_mt_params()
    if params is None:
        pytest.skip("the reference's twister parameter file is not present")
    ctx = gfx.Context(D8)
    ctx.mt_load_params(params)
    ctx.mt_seed(1234)
    ctx.mt_init(4096 // 2, 2 * 4096)
    assert tuple(ctx.mt_sizes()) == tuple(int(x) for x in FX["C_nper"])
    for step in range(3):
        g, u, _, _ = ctx.mt_read()
        assert np.array_equal(_sha(u), FX["C_unif_sha_%d" % step]), step
        # same CUDA intrinsics and flags as the reference build: gaussians agree to 1e-6
        assert np.max(np.abs(g[:512] - FX["C_gauss_head_%d" % step])) < 1e-6, step
        ctx.mt_update()


@pytest.mark.gpu
def test_gpu_sa_halfsweeps_match_reference_gpu(gfx):
    import oracle as orc
    params = orc.load_mt_params()
    if params is None:
        pytest.skip("the reference's twister parameter file is not present")
    u, g = _start(gfx, D4, 101, "A_links_sha")
    ctx = gfx.Context(D4)
    ctx.set_links(u)
    ctx.set_trafo(g)
    ctx.mt_load_params(params)
    ctx.mt_seed(7)
    ctx.mt_init(128, 512)
    for k, (parity, beta) in enumerate(((0, 1.0 / 1.45), (1, 1.0 / 0.3))):
        gs, us, _, _ = ctx.mt_read()
        assert np.array_equal(us[:512], FX["D_unif_%d" % k])
        ctx.sa_halfsweep(parity, beta)
        got = ctx.get_trafo().reshape(-1, 18)[:, :12]
        d = np.max(np.abs(got - FX["D_g_%d" % k]), axis=1)
        assert np.mean(d > 1e-6) <= 0.01, np.sum(d > 1e-6)
        # continue from the reference's state so the next half-sweep compares alone
        ctx.set_trafo(_complete(FX["D_g_%d" % k]))
        ctx.mt_update()


@pytest.mark.gpu
def test_gpu_simanneal_matches_reference_gpu(gfx):
    import oracle as orc
    params = orc.load_mt_params()
    if params is None:
        pytest.skip("the reference's twister parameter file is not present")
    u, g = _start(gfx, D4, 101, "A_links_sha")
    ctx = gfx.Context(D4)
    ctx.set_links(u)
    ctx.set_trafo(g)
    ctx.mt_load_params(params)
    ctx.mt_seed(7)
    ctx.mt_init(128, 512)
    f = ctx.simanneal(0.01, 1.45, 20, expo=-1.0, checkint=5)
    # same random numbers; trajectories agree unless a single-precision accept/reject
    # decision flips, so compare the functional statistically
    assert f.F == pytest.approx(FX["E_functional"][0], rel=2e-2)


def _complete(g12):
    """rows 0,1 -> su3 with row 2 = conj(row0 x row1)"""
    g = g12.reshape(-1, 6, 2)
    a = g[:, 0:3, 0] + 1j * g[:, 0:3, 1]
    b = g[:, 3:6, 0] + 1j * g[:, 3:6, 1]
    m = np.stack([a, b, np.conj(np.cross(a, b))], axis=1)
    return np.stack([m.real, m.imag], axis=-1).reshape(-1, 18)
