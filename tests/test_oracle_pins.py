"""Pins of the CPU oracle: known-answer tests of its generators and bit-for-bit
agreement with the reference's own host C code (observables.c, su3manip.c, rngs.c)
compiled from the reference checkout.  CPU only."""
import ctypes
import ctypes.util

import numpy as np
import pytest

from conftest import haar, smooth_links


def test_park_miller_known_answers(oracle):
    # TestRandom (rngs.c:153-179): state 399268537 after 10000 draws from seed 1,
    # and stream 1 after PlantSeeds(1) equals the jump multiplier 22925.
    import oracle as orc
    pm = orc.OrcPM()
    pm.seed[0] = 1
    pm.stream = 0
    for _ in range(10000):
        oracle.pm_random(pm)
    assert pm.seed[0] == 399268537
    pm = oracle.pm_new(1)
    assert pm.seed[1] == 22925


def test_park_miller_against_reference(refhost):
    assert refhost.test_random_state() == (399268537, 22925)


def test_glibc_rand_restatement_matches_libc(oracle):
    libc = ctypes.CDLL(ctypes.util.find_library("c"))
    for seed in (0, 1, 351, 1234, 2024, 2 ** 31 + 5):
        libc.srand(ctypes.c_uint(seed))
        want = np.array([libc.rand() for _ in range(700)], dtype=np.int32)
        assert np.array_equal(oracle.glibc_rand(seed, 700), want), seed


def _mt19937_init(seed):
    mt = np.zeros(624, dtype=np.uint64)
    mt[0] = seed
    for i in range(1, 624):
        mt[i] = (1812433253 * (int(mt[i - 1]) ^ (int(mt[i - 1]) >> 30)) + i) & 0xFFFFFFFF
    return mt.astype(np.uint32)


def test_generic_mersenne_twister_known_answers(oracle):
    # std::mt19937 with the default seed 5489: the first outputs and the 10000th
    # output 4123659995 (the value the C++ standard requires).
    out = oracle.mt_generic(_mt19937_init(5489), 624, 397, 0x80000000, 0x7FFFFFFF,
                            0x9908B0DF, 11, 7, 0x9D2C5680, 15, 0xEFC60000, 18, 10000)
    assert list(out[:5]) == [3499211612, 581869302, 3890346734, 3586334585, 545404204]
    assert out[9999] == 4123659995


def test_mt607_bank_call_structure(oracle, mt_params):
    """The bank restates RandomGPU's call quirks: each call restarts the 19-word ring
    at slot 0, and an initialized=0 call re-seeds from seed = state[0]."""
    m = oracle.mt_new(mt_params, seeds=np.arange(1, 4097, dtype=np.uint32))
    a = oracle.mt_generate(m, 38, 0)
    # a single generic MT607 run of twister r reproduces lane r of the first call
    for r in (0, 1, 4095):
        st = np.zeros(19, dtype=np.uint64)
        st[0] = r + 1
        for k in range(1, 19):
            st[k] = (1812433253 * (int(st[k - 1]) ^ (int(st[k - 1]) >> 30)) + k) & 0xFFFFFFFF
        x = oracle.mt_generic(st.astype(np.uint32), 19, 9, 0xFFFFFFFE, 0x1,
                              int(mt_params[r, 0]), 12, 7, int(mt_params[r, 1]), 15,
                              int(mt_params[r, 2]), 18, 38)
        want = ((x.astype(np.float32) + np.float32(1.0)) / np.float32(4294967296.0))
        assert np.array_equal(a[r::4096], want)
    # with 38 = 2 x 19 outputs the ring ends at slot 0, so the next call continues
    # the canonical stream
    b = oracle.mt_generate(m, 19, 1)
    st = np.zeros(19, dtype=np.uint64)
    st[0] = 1
    for k in range(1, 19):
        st[k] = (1812433253 * (int(st[k - 1]) ^ (int(st[k - 1]) >> 30)) + k) & 0xFFFFFFFF
    x = oracle.mt_generic(st.astype(np.uint32), 19, 9, 0xFFFFFFFE, 0x1, int(mt_params[0, 0]), 12,
                          7, int(mt_params[0, 1]), 15, int(mt_params[0, 2]), 18, 57)
    want = ((x.astype(np.float32) + np.float32(1.0)) / np.float32(4294967296.0))
    assert np.array_equal(b[0::4096], want[38:])


def test_mt_nper(oracle):
    # iAlignUp(iDivUp(n, 4096), 2) (MersenneTwister.cu:246-253)
    assert oracle.mt_nper(4096) == 2
    assert oracle.mt_nper(8192) == 2
    assert oracle.mt_nper(8193) == 4
    assert oracle.mt_nper(1) == 2
    assert oracle.mt_nper(3 * 4096) == 4


def test_random_init_matches_reference(oracle, refhost):
    dims = (4, 4, 4, 4)
    lat = oracle.lattice(dims)
    refhost.set_lattice(dims, lat._keep[0])
    want = refhost.random_init_trafo(351, 256)
    got = oracle.random_init(oracle.pm_new(351), 256)
    assert np.array_equal(got, want)
    want_g = refhost.random_init_gauge(7, 1024)
    got_g = oracle.random_init(oracle.pm_new(7), 1024)
    assert np.array_equal(got_g, want_g)


def test_layout_conversion_matches_reference(oracle, refhost):
    dims = (4, 4, 4, 4)
    lat = oracle.lattice(dims)
    refhost.set_lattice(dims, lat._keep[0])
    g = haar(256, 3)
    v_ref = refhost.su3to2v(np.concatenate([g] * 4), 1024)
    assert np.array_equal(oracle.to2v(np.concatenate([g] * 4)), v_ref)
    assert np.array_equal(oracle.from2v(v_ref[:256]), refhost.from2vtosu3_trafo(v_ref[:256], 256))


def test_host_observables_match_reference(oracle, refhost):
    dims = (4, 4, 4, 8)
    lat = oracle.lattice(dims)
    refhost.set_lattice(dims, lat._keep[0])
    u = smooth_links(dims, 0.3, 11)
    g = haar(512, 12)
    assert oracle.mean_plaq18(lat, u) == refhost.mean_plaq(u)
    assert oracle.gauge_functional18(lat, u) == refhost.gauge_functional(u)
    assert oracle.dAdA18(lat, u) == refhost.dAdA(u)
    ut = oracle.g_trafo18(lat, u, g)
    assert np.array_equal(ut, refhost.g_trafo(u, g))


def test_device_functional_restatement_matches_host(oracle, refhost):
    """dev_functional (F, dAdA, max on g applied on the fly) equals the host
    observables on the explicitly transformed field to rounding."""
    dims = (4, 4, 4, 8)
    lat = oracle.lattice(dims)
    refhost.set_lattice(dims, lat._keep[0])
    u = smooth_links(dims, 0.4, 21)
    g = haar(512, 22)
    dev = oracle.functional(lat, oracle.to2v(u), oracle.to2v(g))
    ut = refhost.g_trafo(u, g)
    F = refhost.gauge_functional(ut)
    dada, mx = refhost.dAdA(ut)
    assert dev["F"] == pytest.approx(F, rel=1e-13)
    assert dev["dAdA"] == pytest.approx(dada, rel=1e-11)
    assert dev["maxdAdA"] == pytest.approx(mx, rel=1e-11)


def test_plaquette_gauge_invariant(oracle, refhost):
    dims = (4, 4, 4, 4)
    lat = oracle.lattice(dims)
    refhost.set_lattice(dims, lat._keep[0])
    u = smooth_links(dims, 0.5, 5)
    p0 = oracle.plaquette(lat, oracle.to2v(u))
    assert p0 == pytest.approx(refhost.mean_plaq(u), rel=1e-14)
    ut = refhost.g_trafo(u, haar(256, 6))
    assert oracle.plaquette(lat, oracle.to2v(ut)) == pytest.approx(p0, rel=1e-13)


def test_overrelaxation_increases_functional(oracle):
    dims = (4, 4, 4, 4)
    lat = oracle.lattice(dims)
    gf = oracle.to2v(smooth_links(dims, 0.3, 1))
    g = oracle.to2v(haar(256, 2))
    f0 = oracle.functional(lat, gf, g)
    oracle.or_sweeps(lat, gf, g, 20)
    f1 = oracle.functional(lat, gf, g)
    oracle.or_sweeps(lat, gf, g, 40)
    f2 = oracle.functional(lat, gf, g)
    assert f0["F"] < f1["F"] < f2["F"]
    assert f2["dAdA"] < 1e-2 * f1["dAdA"]


def test_micro_step_keeps_functional(oracle):
    dims = (4, 4, 4, 4)
    lat = oracle.lattice(dims)
    gf = oracle.to2v(smooth_links(dims, 0.3, 8))
    g = oracle.to2v(haar(256, 9))
    f0 = oracle.functional(lat, gf, g)["F"]
    oracle.micro_halfsweep(lat, gf, g, 0)
    oracle.micro_halfsweep(lat, gf, g, 1)
    assert oracle.functional(lat, gf, g)["F"] == pytest.approx(f0, rel=1e-12)
