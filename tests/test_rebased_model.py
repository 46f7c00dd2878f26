"""The rebased FP32 polish sweep (cudagfx_gb300/csrc/gfx_rebased.cu) modelled in numpy
complex64/float32 arithmetic on one site, against the exact update in FP64 (CPU).

Near a fixed point (a star whose anti-hermitian part is ~1e-6, neighbours' g = 1 + a
with |a| ~ 1e-6), the rebased form must follow the FP64 overrelaxation step to far
below FP32 rounding -- the property the polish relies on -- while the same step on
FP32-rounded matrices errs by ~1e-7."""
import numpy as np
import pytest

from test_update_algebra import composed_update, normalize

C64, F32 = np.complex64, np.float32
RNG = np.random.default_rng(5)


def small_su3(eps, n=1):
    """g = expm(i eps H) - 1 for random traceless hermitian H (g in SU(3) exactly)"""
    out = []
    for _ in range(n):
        z = RNG.normal(size=(3, 3)) + 1j * RNG.normal(size=(3, 3))
        h = (z + z.conj().T) / 2
        h -= np.trace(h) / 3 * np.eye(3)
        w, v = np.linalg.eigh(h)
        g = v @ np.diag(np.exp(1j * eps * w)) @ v.conj().T
        out.append(normalize(g) - np.eye(3))
    return out


def small_row2(a):
    """row 2 of a = g - 1 from rows 0,1 (the kernel's small_row2)"""
    a = a.copy()
    extra = np.array([-a[0, 2], -a[1, 2], a[0, 0] + a[1, 1]], dtype=a.dtype)
    a[2] = np.conj(extra + np.cross(a[0], a[1]))
    return a


def row2(u):
    u = u.copy()
    u[2] = np.conj(np.cross(u[0], u[1]))
    return u


def split_w0(w0):
    """the stored star: FP32 value, AH(remainder) in FP32, Re tr(remainder)"""
    hi = w0.astype(C64)
    lo = w0 - hi.astype(complex)
    ah = ((lo - lo.conj().T) / 2).astype(C64)
    return hi, ah, F32(np.trace(lo).real)


def rebased_x(w0, uf, ub, af, ab, a_own):
    """X = Xh + Xd in complex64 (rebased_x)"""
    hi, W, _ = split_w0(w0)
    W = W.copy()
    for u, b in zip(uf, af):
        u = u.astype(C64)
        b = small_row2(np.vstack([b[:2].astype(C64), np.zeros((1, 3), C64)]))
        P = u[:2] @ b.conj().T                        # rows 0,1 of U' a^+
        W[:2] += P
        W[2] += np.conj(np.cross(u[0], P[1]) + np.cross(P[0], u[1] + P[1]))
    for u, b in zip(ub, ab):
        u = row2(u.astype(C64))                       # FP32 reconstruction of row 2
        Q = b[:2].astype(C64) @ u                     # rows 0,1 of a U'
        W[:, :2] += Q.conj().T
        W[:, 2] += np.cross(u[0], Q[1]) + np.cross(Q[0], u[1] + Q[1])
    a = small_row2(np.vstack([a_own[:2].astype(C64), np.zeros((1, 3), C64)]))
    Xd = W + a @ (hi + W)
    return hi, Xd, a


def su2_small(xaa, xbb, xab, xba):
    (ha, da), (hb, db), (hab, dab), (hba, dba) = xaa, xbb, xab, xba
    w0 = F32(ha.real + hb.real) + F32(da.real + db.real)
    w3 = F32(hb.imag - ha.imag) + F32(db.imag - da.imag)
    w1 = -F32(hab.imag + hba.imag) - F32(dab.imag + dba.imag)
    w2 = F32(hba.real - hab.real) + F32(dba.real - dab.real)
    s2 = w1 * w1 + w2 * w2 + w3 * w3
    n2 = w0 * w0 + s2
    r = F32(1) / np.sqrt(n2)
    n = n2 * r
    dp = C64(complex(-s2 * r / (w0 + n) if w0 > 0 else w0 * r - 1, w3 * r))
    return dp, C64(complex(w2 * r, w1 * r))


def hd_high(dp, q, x, y):
    return (x[0], x[1] + dp * (x[0] + x[1]) + q * (y[0] + y[1]))


def hd_low(dp, q, x, y):
    return (y[0], y[1] - np.conj(q) * (x[0] + x[1]) + np.conj(dp) * (y[0] + y[1]))


def rsqrt1p_m1(s):
    y = F32(1) / np.sqrt(F32(1) + s)
    return -s * y * y / (F32(1) + y)


def rebased_step(Xh, Xd, a, om):
    """or_update_small: rows 0,1 of the new a"""
    X = lambda r, c: (Xh[r, c], Xd[r, c])
    dp1, q1 = su2_small(X(0, 0), X(1, 1), X(0, 1), X(1, 0))
    x00, x01, x02 = (hd_high(dp1, q1, X(0, j), X(1, j)) for j in range(3))
    x11, x12 = hd_low(dp1, q1, X(0, 1), X(1, 1)), hd_low(dp1, q1, X(0, 2), X(1, 2))
    dp2, q2 = su2_small(x00, X(2, 2), x02, X(2, 0))
    y21, y22 = hd_low(dp2, q2, x01, X(2, 1)), hd_low(dp2, q2, x02, X(2, 2))
    dp3, q3 = su2_small(x11, y22, x12, y21)
    p1, p2, p3 = 1 + dp1, 1 + dp2, 1 + dp3
    c = np.conj
    t0, t1 = c(q2) * p1, c(q2) * q1
    R = np.array([[dp2 + dp1 + dp2 * dp1, p2 * q1, q2],
                  [-(p3 * c(q1) + q3 * t0), dp3 + c(dp1) + dp3 * c(dp1) - q3 * t1, q3 * c(p2)],
                  [c(q3) * c(q1) - c(p3) * t0, -(c(q3) * c(p1) + c(p3) * t1),
                   c(dp3) + c(dp2) + c(dp3) * c(dp2)]], dtype=C64)
    c2 = F32(om * (om - 1) / 2)
    T = F32(om) * R[:2] + c2 * (R[:2] @ R)
    b = a[:2] + T + T @ a
    t = rsqrt1p_m1(F32(2) * b[0, 0].real + F32(np.sum(np.abs(b[0]) ** 2)))
    b[0] = b[0] * (1 + t)
    b[0, 0] += t
    proj = b[1, 0] + np.conj(b[0, 1]) + np.sum(b[1] * np.conj(b[0]))
    b[1, 0] -= proj
    b[1] -= proj * b[0]
    t = rsqrt1p_m1(F32(2) * b[1, 1].real + F32(np.sum(np.abs(b[1]) ** 2)))
    b[1] = b[1] * (1 + t)
    b[1, 1] += t
    return b


def near_fixed_point(ndir, eps_ah, eps_a):
    """rebased links whose star is hermitian up to eps_ah, and small a's.  A gauge-fixed
    configuration's links are close to 1 (Landau gauge maximizes sum Re tr U'), which
    makes X positive: links exp(i H) with |H| ~ 0.6 (Re tr U / 3 ~ 0.85, as at beta 6)"""
    uf = [np.eye(3) + d for d in small_su3(0.6, ndir)]
    # U'_b = (1 + t)^+ U'_f, so U'_f + U'_b^+ = U'_f + U'_f^+ (1 + t) is hermitian up to t
    ub = [np.conj(np.eye(3) + t).T @ u for u, t in zip(uf, small_su3(eps_ah, ndir))]
    w0 = sum(uf) + sum(np.conj(u).T for u in ub)
    af, ab = small_su3(eps_a, ndir), small_su3(eps_a, ndir)
    return w0, uf, ub, af, ab, small_su3(eps_a)[0]


def exact_step(w0, uf, ub, af, ab, a_own, om):
    """the overrelaxation step in FP64 on g_hat = 1 + a_own with the exact star"""
    w = sum(u @ np.conj(np.eye(3) + a).T for u, a in zip(uf, af)) + \
        sum(np.conj((np.eye(3) + a) @ u).T for u, a in zip(ub, ab))
    assert abs(w0 - sum(uf) - sum(np.conj(u).T for u in ub)).max() < 1e-14
    return composed_update(np.eye(3) + a_own, w, om) - np.eye(3)


@pytest.mark.parametrize("ndir", [4, 3])
def test_rebased_step_follows_fp64(ndir):
    worst_rb, worst_32 = 0.0, 0.0
    for _ in range(200):
        w0, uf, ub, af, ab, a_own = near_fixed_point(ndir, 1e-6, 1e-6)
        om = 1.7
        ref = exact_step(w0, uf, ub, af, ab, a_own, om)
        Xh, Xd, a = rebased_x(w0, uf, ub, af, ab, a_own)
        b = rebased_step(Xh, Xd, a, om)
        worst_rb = max(worst_rb, abs(b - ref[:2]).max())
        # the same step with FP32-rounded g and links
        g = (np.eye(3) + a_own).astype(C64)
        w = sum(u.astype(C64) @ np.conj(np.eye(3) + x).astype(C64).T for u, x in zip(uf, af)) + \
            sum(np.conj((np.eye(3) + x).astype(C64) @ u.astype(C64)).T for u, x in zip(ub, ab))
        g32 = composed_update(g.astype(complex), w.astype(complex), om)  # FP32 inputs
        worst_32 = max(worst_32, abs((g32 - np.eye(3))[:2] - ref[:2]).max())
    assert worst_rb < 2e-12, worst_rb     # ~1e-7 x (|a| + |R|)
    assert worst_32 > 1e-9, worst_32      # FP32 rounding of the fields alone
    assert worst_rb < worst_32 / 1000


def test_rebased_theta_follows_fp64():
    """theta's site term from X = Xh + Xd (measure_rebased_kernel) against FP64"""
    for _ in range(50):
        w0, uf, ub, af, ab, a_own = near_fixed_point(4, 1e-6, 1e-6)
        Xh, Xd, a = rebased_x(w0, uf, ub, af, ab, a_own)
        w = sum(u @ np.conj(np.eye(3) + x).T for u, x in zip(uf, af)) + \
            sum(np.conj((np.eye(3) + x) @ u).T for u, x in zip(ub, ab))
        X = (np.eye(3) + a_own) @ w
        ah = (X - X.conj().T) / 2
        ah -= np.trace(ah) / 3 * np.eye(3)
        d_ref = np.sum(abs(ah) ** 2)
        tim = F32(F32(Xh[0, 0].imag + Xh[1, 1].imag + Xh[2, 2].imag)
                  + F32(Xd[0, 0].imag + Xd[1, 1].imag + Xd[2, 2].imag)) / F32(3)
        acc = sum((F32(Xh[m, m].imag + Xd[m, m].imag) - tim) ** 2 for m in range(3))
        off = 0.0
        for m in range(3):
            for n in range(m + 1, 3):
                re = (F32(Xh[m, n].real - Xh[n, m].real) + F32(Xd[m, n].real - Xd[n, m].real)) / 2
                im = (F32(Xh[m, n].imag + Xh[n, m].imag) + F32(Xd[m, n].imag + Xd[n, m].imag)) / 2
                off += re * re + im * im
        d = float(acc) + 2.0 * float(off)
        assert d == pytest.approx(d_ref, rel=1e-4)
        assert d_ref < 1e-9  # near the fixed point: FP32 on X itself would not resolve it
