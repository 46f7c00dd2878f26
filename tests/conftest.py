import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def oracle():
    import oracle as orc
    return orc.Oracle()


@pytest.fixture(scope="session")
def refhost():
    import oracle as orc
    try:
        return orc.RefHost()
    except FileNotFoundError as e:
        pytest.skip(str(e))


@pytest.fixture(scope="session")
def gfx():
    from cudagfx_gb300 import build
    build.build()
    import cudagfx_gb300
    return cudagfx_gb300


@pytest.fixture(scope="session")
def mt_params():
    """The reference's twister parameters when available, else a stand-in set."""
    import oracle as orc
    p = orc.load_mt_params()
    return p if p is not None else orc.synthetic_mt_params()


def su3_from_rows(a):
    """(n, 2, 3) complex rows -> (n, 18) su3 with Gram-Schmidt and row 2 = conj(r0 x r1)."""
    r0 = a[:, 0] / np.linalg.norm(a[:, 0], axis=1, keepdims=True)
    r1 = a[:, 1] - np.sum(a[:, 1] * np.conj(r0), axis=1, keepdims=True) * r0
    r1 = r1 / np.linalg.norm(r1, axis=1, keepdims=True)
    r2 = np.conj(np.cross(r0, r1))
    m = np.stack([r0, r1, r2], axis=1)
    out = np.empty(m.shape + (2,))
    out[..., 0] = m.real
    out[..., 1] = m.imag
    return out.reshape(-1, 18)


def smooth_links(dims, eps, seed):
    """Links near the identity, U = GramSchmidt(1 + eps * complex Gaussian): a
    weak-coupling-like configuration on which gauge fixing converges quickly."""
    rng = np.random.default_rng(seed)
    n = 4 * int(np.prod(dims))
    z = rng.normal(size=(n, 2, 3)) + 1j * rng.normal(size=(n, 2, 3))
    a = np.zeros((n, 2, 3), dtype=complex)
    a[:, 0, 0] = 1.0
    a[:, 1, 1] = 1.0
    return su3_from_rows(a + eps * z)


def haar(n, seed):
    rng = np.random.default_rng(seed)
    z = rng.normal(size=(n, 2, 3)) + 1j * rng.normal(size=(n, 2, 3))
    return su3_from_rows(z)


def lexi(dims):
    lx, ly, lz, lt = dims
    return lx * ly * lz * lt
