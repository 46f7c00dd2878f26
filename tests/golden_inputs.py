"""Deterministic input fields for the golden fixtures (shared by the fixture generator
and the tests): links near the identity, U = GramSchmidt(1 + 0.35 z) with z complex
Gaussian from numpy's PCG64 stream of the given seed.  The fixtures store the SHA-256
of the generated links so a change of the generator is detected."""
import numpy as np


def links_for(dims, seed, eps=0.35):
    rng = np.random.default_rng(seed)
    n = 4 * int(np.prod(dims))
    z = rng.normal(size=(n, 2, 3)) + 1j * rng.normal(size=(n, 2, 3))
    a = np.zeros((n, 2, 3), dtype=complex)
    a[:, 0, 0] = 1.0
    a[:, 1, 1] = 1.0
    a = a + eps * z
    r0 = a[:, 0] / np.sqrt(np.sum(np.abs(a[:, 0]) ** 2, axis=1, keepdims=True))
    r1 = a[:, 1] - np.sum(a[:, 1] * np.conj(r0), axis=1, keepdims=True) * r0
    r1 = r1 / np.sqrt(np.sum(np.abs(r1) ** 2, axis=1, keepdims=True))
    r2 = np.conj(np.cross(r0, r1))
    m = np.stack([r0, r1, r2], axis=1)
    return np.ascontiguousarray(np.stack([m.real, m.imag], axis=-1).reshape(n, 18))
