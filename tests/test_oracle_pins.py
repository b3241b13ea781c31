"""Pins of the CPU restatement (oracle) against independent mathematics.

The reference ships no golden vectors, so the oracle is checked against
facts that do not depend on its own code: the Boys function from mpmath,
the Hermite E-coefficients against direct evaluation of the spinor overlap
densities on points in space, R-integrals against finite differences of
F_0, closed-form (ss|ss) integrals, and the time-reversal phase relations
that the reference uses to derive 12 of its 16 m-sign combinations
(bertha-scf.f:12809-13119).
"""
import math

import mpmath
import numpy as np
import pytest
from scipy.special import eval_hermite, lpmv

from oracle import oracle as orc

RNG = np.random.default_rng(20241203)


def boys_mp(m, T):
    if T == 0:
        return mpmath.mpf(1) / (2 * m + 1)
    T = mpmath.mpf(T)
    return mpmath.gammainc(m + mpmath.mpf(0.5), 0, T) / (2 * T ** (m + mpmath.mpf(0.5)))


@pytest.mark.parametrize("lam", [0, 4, 12, 18])
def test_boys_against_mpmath(lam):
    mpmath.mp.dps = 40
    for T in np.concatenate([[0.0, 1e-12, 1e-3], np.logspace(-2, 6, 60)]):
        F = orc.boys(T, lam)
        for m in range(lam + 1):
            ref = float(boys_mp(m, T))
            err = abs(F[m] - ref)
            if T <= 1e-11:
                # exact T=0 values: error bounded by T
                assert err <= T, (T, m)
            elif T <= 17.0:
                # power series regime: full double precision
                assert err <= 1e-14 * max(ref, 1e-300) + 1e-300, (T, m)
            elif T <= 30.0:
                # rational seed regime: the reference's own ~1e-11 accuracy
                assert err <= 2e-11, (T, m, err)
            else:
                # exp(-T) dropped: error bounded by exp(-T)
                assert err <= 2 * math.exp(-T) + 1e-15 * ref, (T, m)


def test_rints_finite_differences():
    mpmath.mp.dps = 40
    alpha = 0.7
    P = np.array([0.3, -0.4, 0.9])

    def f0(x, y, z):
        return boys_mp(0, alpha * (x * x + y * y + z * z))

    lam = 3
    R = orc.rints(-P, alpha, lam)  # qp = Q - P with Q = 0 -> P-Q = P
    for t in range(lam + 1):
        for u in range(lam + 1 - t):
            for v in range(lam + 1 - t - u):
                d = mpmath.diff(f0, (mpmath.mpf(P[0]), mpmath.mpf(P[1]),
                                     mpmath.mpf(P[2])), (t, u, v))
                assert abs(R[orc.cart_index(t, u, v)] - float(d)) < 1e-12


def ylm(l, m, theta, phi):
    """Spherical harmonic with the Condon-Shortley phase."""
    if abs(m) > l:
        return np.zeros_like(theta, dtype=np.complex128)
    am = abs(m)
    n = math.sqrt((2 * l + 1) / (4 * math.pi) * math.factorial(l - am) / math.factorial(l + am))
    y = n * lpmv(am, l, np.cos(theta)) * np.exp(1j * am * phi)
    if m < 0:
        y = (-1) ** am * np.conj(y)
    return y


def cg(kq, mq, small):
    jq = 2 * abs(kq) - 1
    neg = (kq < 0) != small
    if neg:
        return math.sqrt((jq + mq) / (2 * jq)), math.sqrt((jq - mq) / (2 * jq))
    return -math.sqrt((jq - mq + 2) / (2 * jq + 4)), math.sqrt((jq + mq + 2) / (2 * jq + 4))


def spinor(kq, mq, ex, C, r, small):
    """Two-component G-spinor (large or kinetically balanced small) at points r."""
    l = -kq - 1 if kq < 0 else kq
    d = r - C
    rr = np.linalg.norm(d, axis=1)
    th = np.arccos(np.clip(d[:, 2] / np.maximum(rr, 1e-300), -1, 1))
    ph = np.arctan2(d[:, 1], d[:, 0])
    g = np.exp(-ex * rr ** 2)
    if not small:
        lp = l
        nrm = math.sqrt(2 * (2 * ex) ** (l + 1.5) / math.gamma(l + 1.5))
        rad = nrm * rr ** l * g
    else:
        lp = l + 1 if kq < 0 else l - 1
        nrm = math.sqrt(2 * (2 * ex) ** (l + 0.5) / math.gamma(l + 2.5))
        if kq < 0:
            rad = nrm * (-2 * ex) * rr ** (l + 1) * g
        else:
            rad = nrm * ((2 * l + 1) * rr ** (l - 1) - 2 * ex * rr ** (l + 1)) * g
    cu, cl = cg(kq, mq, small)
    up = cu * ylm(lp, (mq - 1) // 2, th, ph)
    lo = cl * ylm(lp, (mq + 1) // 2, th, ph)
    return rad * up, rad * lo


def hermite_basis(L, p, P, r):
    d = r - P
    sp = math.sqrt(p)
    out = []
    for lam in range(L + 1):
        for t in range(lam + 1):
            for u in range(lam + 1 - t):
                v = lam - t - u
                h = (p ** (lam / 2) * eval_hermite(t, sp * d[:, 0]) * eval_hermite(u, sp * d[:, 1])
                     * eval_hermite(v, sp * d[:, 2]) * np.exp(-p * (d ** 2).sum(1)))
                out.append(h)
    return np.array(out)


@pytest.mark.parametrize("small", [False, True])
@pytest.mark.parametrize("la,lb", [(0, 0), (1, 0), (0, 2), (1, 1), (2, 1), (3, 2)])
def test_eq_coefficients_reproduce_spinor_density(la, lb, small):
    A = RNG.uniform(-1, 1, 3)
    B = RNG.uniform(-1, 1, 3)
    ea, eb = RNG.uniform(0.3, 2.0), RNG.uniform(0.3, 2.0)
    p = ea + eb
    P = (ea * A + eb * B) / p
    r = P + RNG.normal(scale=0.6, size=(25, 3))
    kqs_a = [k for k in (la, -la - 1) if k != 0]
    kqs_b = [k for k in (lb, -lb - 1) if k != 0]
    L = la + lb + (2 if small else 0)
    H = hermite_basis(L, p, P, r)
    for ka in kqs_a:
        for kb in kqs_b:
            for mqa in range(-(2 * abs(ka) - 1), 2 * abs(ka), 2):
                for mqb in range(-(2 * abs(kb) - 1), 2 * abs(kb), 2):
                    E = orc.eq_pair(ka, mqa, ea, A, kb, mqb, eb, B, small)
                    assert E.shape[0] == orc.ntuv(L)
                    ua, la_ = spinor(ka, mqa, ea, A, r, small)
                    ub, lb_ = spinor(kb, mqb, eb, B, r, small)
                    rho = np.conj(ua) * ub + np.conj(la_) * lb_
                    got = E @ H
                    scale = max(np.abs(rho).max(), 1e-3)
                    assert np.abs(got - rho).max() <= 1e-10 * scale, (ka, mqa, kb, mqb)


@pytest.mark.parametrize("small", [False, True])
def test_time_reversal_relations(small):
    """E(+,+) = P conj(E(-,-)) and E(-,+) = -P conj(E(+,-)), the relations
    ERIFAST uses to derive 12 of its 16 combinations."""
    A, B = RNG.uniform(-1, 1, 3), RNG.uniform(-1, 1, 3)
    for ka in (-1, 1, -2, 2, -3):
        for kb in (-1, 1, -2, 3, -4):
            for ma in range(1, abs(ka) + 1):
                for mb in range(1, abs(kb) + 1):
                    mqa, mqb = 2 * ma - 1, 2 * mb - 1
                    pab = (1 if ka * kb > 0 else -1) * (-1) ** ((mqa - mqb) // 2)
                    e11 = orc.eq_pair(ka, -mqa, 0.9, A, kb, -mqb, 1.3, B, small)
                    e21 = orc.eq_pair(ka, mqa, 0.9, A, kb, -mqb, 1.3, B, small)
                    e22 = orc.eq_pair(ka, mqa, 0.9, A, kb, mqb, 1.3, B, small)
                    e12 = orc.eq_pair(ka, -mqa, 0.9, A, kb, mqb, 1.3, B, small)
                    s = max(np.abs(e11).max(), np.abs(e21).max(), 1e-12)
                    assert np.abs(e22 - pab * np.conj(e11)).max() <= 1e-13 * s
                    assert np.abs(e12 + pab * np.conj(e21)).max() <= 1e-13 * s


def test_ssss_closed_form():
    xyz = RNG.uniform(-1.5, 1.5, (4, 3))
    ex = np.array([0.8, 1.7, 0.4, 2.2])
    V = orc.eri_quartet(xyz, [0, 0, 0, 0], ex, 0, 0)
    n = [math.sqrt(2 * (2 * a) ** 1.5 / math.gamma(1.5)) for a in ex]
    p, q = ex[0] + ex[1], ex[2] + ex[3]
    P = (ex[0] * xyz[0] + ex[1] * xyz[1]) / p
    Q = (ex[2] * xyz[2] + ex[3] * xyz[3]) / q
    kab = math.exp(-ex[0] * ex[1] / p * np.sum((xyz[0] - xyz[1]) ** 2))
    kcd = math.exp(-ex[2] * ex[3] / q * np.sum((xyz[2] - xyz[3]) ** 2))
    T = p * q / (p + q) * np.sum((P - Q) ** 2)
    mpmath.mp.dps = 30
    ref = (np.prod(n) * kab * kcd / (4 * math.pi) ** 2 * 2 * math.pi ** 2.5
           / (p * q * math.sqrt(p + q)) * float(boys_mp(0, T)))
    v = V[0, 0, 0, 0]
    # spin-diagonal combinations carry the full value, spin-flips vanish
    for s in range(16):
        sa, sb, sc, sd = (s >> 3) & 1, (s >> 2) & 1, (s >> 1) & 1, s & 1
        want = ref if (sa == sb and sc == sd) else 0.0
        assert abs(v[s] - want) < 1e-13 * ref


def test_eri_particle_exchange_symmetry():
    """(ab|cd) = (cd|ab) for every label and m-sign combination."""
    xyz = RNG.uniform(-1.0, 1.0, (4, 3))
    l4 = [1, 2, 0, 1]
    ex = np.array([0.9, 0.5, 1.4, 0.7])
    for t1, t2 in [(0, 0), (0, 1), (1, 1)]:
        V = orc.eri_quartet(xyz, l4, ex, t1, t2)
        W = orc.eri_quartet(xyz[[2, 3, 0, 1]], [l4[2], l4[3], l4[0], l4[1]],
                            ex[[2, 3, 0, 1]], t2, t1)
        s = np.abs(V).max()
        for sidx in range(16):
            sa, sb, sc, sd = (sidx >> 3) & 1, (sidx >> 2) & 1, (sidx >> 1) & 1, sidx & 1
            w = W[..., 8 * sc + 4 * sd + 2 * sa + sb].transpose(2, 3, 0, 1)
            assert np.abs(V[..., sidx] - w).max() <= 1e-12 * s
