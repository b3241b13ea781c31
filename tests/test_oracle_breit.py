"""Pins of the Breit part of the CPU restatement (oracle) against independent
mathematics.

- sigma-coupled LS/SL E-coefficients (EQLS/EQSL) reproduce i * psi_a^+ sigma_q
  psi_b (LS) and -i * psi_a^+ sigma_q psi_b (SL) evaluated on points;
- the time-reversal relations with the Breit phase (the Coulomb phase
  negated, bertha-scf.f:17528-17533) that BIIFAST uses for 12 of its 16 m-sign
  combinations;
- the Breit kernel against direct quadrature of the Gaussian-smeared
  operator delta_ij/r + r_i r_j/r^3, and its Hermite derivatives against
  finite differences;
- (ab|cd) = (cd|ab) and (ab|cd)* = (ba|dc) for whole Breit quartets;
- Hermitian LL and SS blocks of the Breit exchange matrix for a Hermitian
  density.
"""
import math

import numpy as np
import pytest
from numpy.polynomial.legendre import leggauss

from oracle import oracle as orc
from test_oracle_pins import hermite_basis, spinor

import berthagpu.deck as deck

RNG = np.random.default_rng(770)


def pauli(q):
    return [np.eye(2), np.array([[0, 1], [1, 0]]), np.array([[0, -1j], [1j, 0]]),
            np.array([[1, 0], [0, -1]])][q]


@pytest.mark.parametrize("sa,sb", [(0, 1), (1, 0)])
@pytest.mark.parametrize("la,lb", [(0, 0), (1, 0), (0, 2), (2, 1), (3, 1)])
def test_sigma_e_coefficients_reproduce_spinor_density(la, lb, sa, sb):
    A, B = RNG.uniform(-1, 1, 3), RNG.uniform(-1, 1, 3)
    ea, eb = RNG.uniform(0.3, 2.0), RNG.uniform(0.3, 2.0)
    p = ea + eb
    P = (ea * A + eb * B) / p
    r = P + RNG.normal(scale=0.6, size=(25, 3))
    H = hermite_basis(la + lb + 1, p, P, r)
    phase = 1j if (sa, sb) == (0, 1) else -1j
    for ka in [k for k in (la, -la - 1) if k != 0]:
        for kb in [k for k in (lb, -lb - 1) if k != 0]:
            for mqa in range(-(2 * abs(ka) - 1), 2 * abs(ka), 2):
                for mqb in range(-(2 * abs(kb) - 1), 2 * abs(kb), 2):
                    ua = spinor(ka, mqa, ea, A, r, bool(sa))
                    ub = spinor(kb, mqb, eb, B, r, bool(sb))
                    for q in range(4):
                        E = orc.eq_pair_q(ka, mqa, ea, A, kb, mqb, eb, B, sa, sb, q)
                        assert E.shape[0] == orc.ntuv(la + lb + 1)
                        s = pauli(q)
                        rho = (np.conj(ua[0]) * (s[0, 0] * ub[0] + s[0, 1] * ub[1])
                               + np.conj(ua[1]) * (s[1, 0] * ub[0] + s[1, 1] * ub[1]))
                        got = E @ H
                        scale = max(np.abs(rho).max(), 1e-3)
                        assert np.abs(got - phase * rho).max() <= 1e-10 * scale, \
                            (ka, mqa, kb, mqb, q)


@pytest.mark.parametrize("sa,sb", [(0, 1), (1, 0)])
def test_breit_time_reversal_relations(sa, sb):
    A, B = RNG.uniform(-1, 1, 3), RNG.uniform(-1, 1, 3)
    for ka in (-1, 1, -2, 2, -3):
        for kb in (-1, 1, -2, 3, -4):
            for ma in range(1, abs(ka) + 1):
                for mb in range(1, abs(kb) + 1):
                    mqa, mqb = 2 * ma - 1, 2 * mb - 1
                    pab = -(1 if ka * kb > 0 else -1) * (-1) ** ((mqa - mqb) // 2)
                    for q in (1, 2, 3):
                        e11 = orc.eq_pair_q(ka, -mqa, 0.9, A, kb, -mqb, 1.3, B, sa, sb, q)
                        e21 = orc.eq_pair_q(ka, mqa, 0.9, A, kb, -mqb, 1.3, B, sa, sb, q)
                        e22 = orc.eq_pair_q(ka, mqa, 0.9, A, kb, mqb, 1.3, B, sa, sb, q)
                        e12 = orc.eq_pair_q(ka, -mqa, 0.9, A, kb, mqb, 1.3, B, sa, sb, q)
                        s = max(np.abs(e11).max(), np.abs(e21).max(), 1e-12)
                        assert np.abs(e22 - pab * np.conj(e11)).max() <= 1e-13 * s
                        assert np.abs(e12 + pab * np.conj(e21)).max() <= 1e-13 * s


def _smeared(alpha, X):
    """(alpha/pi)^(3/2) int exp(-alpha|s-X|^2) [1/|s|, s_i s_j/|s|^3] d^3s by
    product quadrature in spherical coordinates about s = 0."""
    rmax = np.linalg.norm(X) + 9.0 / math.sqrt(alpha)
    xr, wr = leggauss(160)
    r = 0.5 * rmax * (xr + 1)
    wr = 0.5 * rmax * wr
    xc, wc = leggauss(64)
    nphi = 64
    phi = 2 * math.pi * np.arange(nphi) / nphi
    ct, ph = np.meshgrid(xc, phi, indexing="ij")
    st = np.sqrt(1 - ct ** 2)
    n = np.stack([st * np.cos(ph), st * np.sin(ph), ct], -1)  # [nc, nphi, 3]
    wang = (wc[:, None] * np.full(nphi, 2 * math.pi / nphi)[None, :])
    s1 = 0.0
    s2 = np.zeros((3, 3))
    for ri, wi in zip(r, wr):
        g = np.exp(-alpha * ((ri * n - X) ** 2).sum(-1)) * wang * wi * ri  # r^2/r
        s1 += g.sum()
        s2 += np.einsum("ab,abi,abj->ij", g, n, n)
    c = (alpha / math.pi) ** 1.5
    return c * s1, c * s2


@pytest.mark.parametrize("X", [(0.0, 0.0, 0.0), (0.4, -0.3, 0.9), (1.2, 0.5, -0.2)])
def test_breit_kernel_against_quadrature(X):
    """W_ij(0) = -1/2 PRE-free smeared (delta_ij/r + r_i r_j/r^3), scaled by
    the factor 2 sqrt(alpha/pi) that maps R_000 = F_0 onto the smeared 1/r."""
    alpha = 0.7
    X = np.array(X)
    W = orc.breit_kernel(-X, alpha, 0, 0, 0)
    one, rr = _smeared(alpha, X)
    f0 = orc.boys(alpha * X @ X, 0)[0]
    c = 2 * math.sqrt(alpha / math.pi)
    assert abs(c * f0 - one) < 1e-10
    want = -0.5 * (np.eye(3) * one + rr)
    assert np.abs(c * W - want).max() < 1e-10
    G = orc.breit_kernel(-X, alpha, 0, 0, 0, gaunt=True)
    assert np.abs(c * G + np.eye(3) * one).max() < 1e-10


def test_breit_kernel_hermite_derivatives():
    """W_ij(N) is the N-th derivative of W_ij(0) with respect to X = P - Q."""
    alpha, h = 0.9, 1e-4
    X = np.array([0.3, -0.5, 0.7])
    for N in [(1, 0, 0), (0, 1, 0), (0, 0, 1), (2, 0, 0), (1, 1, 0), (0, 1, 2)]:
        # derivative of W(N - e_k) along X_k
        k = next(i for i in range(3) if N[i] > 0)
        M = list(N)
        M[k] -= 1
        e = np.zeros(3)
        e[k] = h
        wp = orc.breit_kernel(-(X + e), alpha, *M)
        wm = orc.breit_kernel(-(X - e), alpha, *M)
        fd = (wp - wm) / (2 * h)
        assert np.abs(fd - orc.breit_kernel(-X, alpha, *N)).max() < 1e-7, N


def _quartet():
    xyz = RNG.uniform(-1.0, 1.0, (4, 3))
    return xyz, [1, 0, 2, 1], np.array([0.9, 0.5, 1.4, 0.7])


@pytest.mark.parametrize("gaunt", [False, True])
def test_breit_particle_exchange_symmetry(gaunt):
    xyz, l4, ex = _quartet()
    for t1, t2 in [(0, 0), (0, 1), (1, 0), (1, 1)]:
        V = orc.bii_quartet(xyz, l4, ex, t1, t2, gaunt)
        W = orc.bii_quartet(xyz[[2, 3, 0, 1]], [l4[2], l4[3], l4[0], l4[1]],
                            ex[[2, 3, 0, 1]], t2, t1, gaunt)
        s = np.abs(V).max()
        assert s > 0
        for sidx in range(16):
            sa, sb, sc, sd = (sidx >> 3) & 1, (sidx >> 2) & 1, (sidx >> 1) & 1, sidx & 1
            w = W[..., 8 * sc + 4 * sd + 2 * sa + sb].transpose(2, 3, 0, 1)
            assert np.abs(V[..., sidx] - w).max() <= 1e-12 * s


def test_breit_hermiticity():
    """(ab|cd)* = (ba|dc): LS pairs against SL pairs of the swapped shells."""
    xyz, l4, ex = _quartet()
    V = orc.bii_quartet(xyz, l4, ex, 0, 0)
    W = orc.bii_quartet(xyz[[1, 0, 3, 2]], [l4[1], l4[0], l4[3], l4[2]],
                        ex[[1, 0, 3, 2]], 1, 1)
    s = np.abs(V).max()
    for sidx in range(16):
        sa, sb, sc, sd = (sidx >> 3) & 1, (sidx >> 2) & 1, (sidx >> 1) & 1, sidx & 1
        w = W[..., 8 * sb + 4 * sa + 2 * sd + sc].transpose(1, 0, 3, 2)
        assert np.abs(np.conj(V[..., sidx]) - w).max() <= 1e-12 * s


def test_breit_exchange_blocks_hermitian():
    b = deck.make_basis([((0.0, 0.0, 0.0), {0: [0.3, 2.5], 1: [0.7]}),
                         ((0.3, -0.8, 1.3), {0: [0.45], 1: [1.1]}),
                         ((-1.0, 0.5, 0.4), {0: [0.9]})], hmlt="DHFB")
    dent = deck.density(b, seed=4)
    assert np.abs(dent - dent.conj().T).max() < 1e-14
    bx = orc.brtfast(b, dent, 3)
    n = bx.shape[0] // 2
    s = np.abs(bx).max()
    assert s > 0
    assert np.abs(bx - bx.conj().T).max() <= 1e-12 * s
    for blk in (bx[:n, :n], bx[n:, n:], bx[:n, n:]):
        assert np.abs(blk).max() > 1e-6 * s


def test_breit_kernel_table_is_symmetric():
    """W_ij(N) = W_ji(N): the Cartesian part of the Breit operator,
    delta_ij/r + r_i r_j/r^3, is symmetric, so its Hermite table is too (the
    GPU kernel keeps 6 of the 9 entries per N)."""
    rng = np.random.default_rng(11)
    for _ in range(100):
        qp = rng.normal(size=3) * rng.uniform(0.0, 2.0)
        alpha = float(np.exp(rng.uniform(-3.0, 8.0)))
        t, u, v = (int(x) for x in rng.integers(0, 4, 3))
        for gaunt in (False, True):
            W = orc.breit_kernel(qp, alpha, t, u, v, gaunt=gaunt)
            scale = np.abs(W).max()
            if scale > 0:
                assert np.abs(W - W.T).max() <= 1e-13 * scale
