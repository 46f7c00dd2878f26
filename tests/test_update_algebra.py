"""The identities the reduced FP32 / double-float update relies on, checked in FP64
numpy on random SU(3) matrices (CPU):

1. the composed form -- S = S3 S2 S1 from the three Cabibbo-Marinari subgroup steps,
   R = S - 1, g_new = normalize(g_old + (w R + w(w-1)/2 R^2) g_old) -- equals the
   reference's sequence (rotate g per subgroup from X = g w, normalize, R =
   g_relax g_old^+ - 1, Rw = 1 + w R + w(w-1)/2 R^2, normalize(normalize(Rw) g_old));
2. an SU(3) product's row 2 is conj(row 0 x row 1) (the row-product star terms);
3. the 8-parameter form (a2, a3, arg a1, arg c1, b1) rebuilds the matrix."""
import numpy as np

RNG = np.random.default_rng(11)


def haar(n):
    z = RNG.normal(size=(n, 3, 3)) + 1j * RNG.normal(size=(n, 3, 3))
    q, r = np.linalg.qr(z)
    d = np.diagonal(r, axis1=1, axis2=2)
    q = q * (d / abs(d))[:, None, :]
    q[:, 2, :] /= np.linalg.det(q)[:, None]
    return q


def normalize(u):
    u = u.copy()
    u[0] /= np.linalg.norm(u[0])
    u[1] -= np.vdot(u[0], u[1]) * u[0]
    u[1] /= np.linalg.norm(u[1])
    u[2] = np.conj(np.cross(u[0], u[1]))
    return u


def su2(xaa, xbb, xab, xba):
    """(p, q) of the relaxed subgroup element (overrelax.cu:184-223)"""
    w0, w3 = xaa.real + xbb.real, xbb.imag - xaa.imag
    w1, w2 = -xab.imag - xba.imag, xba.real - xab.real
    r = 1.0 / np.sqrt(w0 * w0 + w1 * w1 + w2 * w2 + w3 * w3)
    return complex(w0 * r, w3 * r), complex(w2 * r, w1 * r)


def reference_update(gold, w, om):
    g = gold.copy()
    for a, b in ((0, 1), (0, 2), (1, 2)):
        X = g @ w
        p, q = su2(X[a, a], X[b, b], X[a, b], X[b, a])
        ra, rb = g[a].copy(), g[b].copy()
        g[a], g[b] = p * ra + q * rb, -np.conj(q) * ra + np.conj(p) * rb
    g = normalize(g)
    R = g @ gold.conj().T - np.eye(3)
    Rw = np.eye(3) + om * R + om * (om - 1) / 2 * R @ R
    return normalize(normalize(Rw) @ gold)


def composed_update(gold, w, om):
    X = gold @ w
    hi = lambda p, q, x, y: p * x + q * y
    lo = lambda p, q, x, y: -np.conj(q) * x + np.conj(p) * y
    p1, q1 = su2(X[0, 0], X[1, 1], X[0, 1], X[1, 0])
    x00, x01, x02 = (hi(p1, q1, X[0, j], X[1, j]) for j in range(3))
    x11, x12 = lo(p1, q1, X[0, 1], X[1, 1]), lo(p1, q1, X[0, 2], X[1, 2])
    p2, q2 = su2(x00, X[2, 2], x02, X[2, 0])
    y21, y22 = lo(p2, q2, x01, X[2, 1]), lo(p2, q2, x02, X[2, 2])
    p3, q3 = su2(x11, y22, x12, y21)
    s0 = [p2 * p1, p2 * q1, q2]
    t2 = [-np.conj(q2) * p1, -np.conj(q2) * q1, np.conj(p2)]
    r1 = [-np.conj(q1), np.conj(p1), 0]
    S = np.array([s0, [hi(p3, q3, r1[j], t2[j]) for j in range(3)],
                  [lo(p3, q3, r1[j], t2[j]) for j in range(3)]])
    R = S - np.eye(3)
    return normalize(gold + (om * R + om * (om - 1) / 2 * R @ R) @ gold)


def test_composed_update_equals_reference_sequence():
    worst = 0.0
    for _ in range(500):
        gold = haar(1)[0]
        w = sum(haar(1)[0] for _ in range(8))  # a star: a sum of 8 SU(3) terms
        for om in (1.0, 1.68, 1.7, 1.9):
            worst = max(worst, abs(reference_update(gold, w, om) -
                                   composed_update(gold, w, om)).max())
    assert worst < 1e-13


def test_product_row2_is_conjugate_cross_product():
    a, b = haar(1000), haar(1000)
    p = a @ np.conj(np.transpose(b, (0, 2, 1)))      # U g^+
    q = b @ a                                        # g U
    for m in (p, q):
        assert abs(m[:, 2] - np.conj(np.cross(m[:, 0], m[:, 1]))).max() < 1e-14


def test_eight_parameter_reconstruction():
    u = haar(20000)
    a1, a2, a3, b1, c1 = u[:, 0, 0], u[:, 0, 1], u[:, 0, 2], u[:, 1, 0], u[:, 2, 0]
    n2 = abs(a2) ** 2 + abs(a3) ** 2
    A1 = np.sqrt(np.maximum(1 - n2, 0)) * np.exp(1j * np.angle(a1))
    C1 = np.sqrt(np.maximum(n2 - abs(b1) ** 2, 0)) * np.exp(1j * np.angle(c1))
    ca1 = np.conj(A1)
    b2 = -(a2 * ca1 * b1 + np.conj(a3) * np.conj(C1)) / n2
    b3 = (np.conj(a2) * np.conj(C1) - a3 * ca1 * b1) / n2
    c2 = (np.conj(a3) * np.conj(b1) - a2 * ca1 * C1) / n2
    c3 = -(np.conj(a2) * np.conj(b1) + a3 * ca1 * C1) / n2
    rec = np.stack([np.stack([A1, a2, a3], -1), np.stack([b1, b2, b3], -1),
                    np.stack([C1, c2, c3], -1)], 1)
    err = abs(rec - u).max(axis=(1, 2))
    # the conditioning is 1/n2: below the kernel's 1e-2 threshold it takes the exact rows
    assert err[n2 >= 1e-2].max() < 1e-12
