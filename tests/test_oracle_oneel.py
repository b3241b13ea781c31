"""Pins of the oracle's one-electron matrices (ONEEL) against independent
physics: the Dirac hydrogen-like spectrum (point nucleus), the
non-relativistic hydrogen ground state, the Gaussian-nucleus attraction
against radial quadrature of erf(sqrt(xi) r)/r, and the structure of the
matrices (Hermitian, unit diagonal overlap)."""
import math

import numpy as np
import pytest
import scipy.linalg as sl
from scipy.integrate import quad
from scipy.special import erf

from oracle import oracle as orc
import berthagpu.deck as deck

C = 137.035999084


def _atom(Z, hmlt="DHFR", np_=24):
    ex = deck.geometric(0.01 * Z * Z, 2.0, 34)
    return deck.make_basis([((0, 0, 0), {0: ex, 1: ex[:np_]})], hmlt=hmlt)


def _dirac(Z, n, k):
    g = math.sqrt(k * k - (Z / C) ** 2)
    return C * C * (1.0 / math.sqrt(1.0 + (Z / C / (n - k + g)) ** 2) - 1.0)


@pytest.mark.parametrize("Z,tol", [(1.0, 1e-8), (10.0, 1e-6)])
def test_dirac_hydrogenic_levels(Z, tol):
    b = _atom(Z)
    S, V, T = orc.oneel(b, [Z], [0.0])
    H = V + T
    assert np.abs(S - S.conj().T).max() < 1e-14
    assert np.abs(H - H.conj().T).max() < 1e-9 * np.abs(H).max()
    assert np.abs(np.diag(S) - 1).max() < 1e-13
    w = sl.eigh(H, S, eigvals_only=True)
    pos = w[w > -C * C]
    # 1s1/2 (Kramers pair), then 2s1/2 and 2p1/2 (degenerate in Dirac theory)
    assert abs(pos[0] - _dirac(Z, 1, 1)) < tol * Z * Z
    assert abs(pos[1] - pos[0]) < 1e-10 * Z * Z
    assert abs(pos[2] - _dirac(Z, 2, 1)) < 4 * tol * Z * Z
    # positive-energy count = large-component dimension
    assert len(pos) == b.ndim // 2


def test_nonrelativistic_hydrogen():
    b = _atom(1.0, hmlt="NORL")
    S, V, T = orc.oneel(b, [1.0], [0.0])
    w = sl.eigh(V + T, S, eigvals_only=True)
    assert abs(w[0] + 0.5) < 1e-8
    assert abs(w[2] + 0.125) < 1e-6


def test_gaussian_nucleus_attraction_quadrature():
    """s-s element of a one-centre pair: -Z int rho(r) erf(sqrt(xi) r)/r."""
    Z, xi = 8.0, 1.5 / (3.0e-5) ** 2
    ea, eb = 2.0e4, 3.0e3
    b = deck.make_basis([((0, 0, 0), {0: [ea, eb]})], hmlt="DHFR")
    S, V, T = orc.oneel(b, [Z], [xi])
    na = math.sqrt(2 * (2 * ea) ** 1.5 / math.gamma(1.5))
    nb = math.sqrt(2 * (2 * eb) ** 1.5 / math.gamma(1.5))
    p = ea + eb
    # radial functions R = N r^0 exp(-a r^2), angular Y00 normalised
    f = lambda r: na * nb * math.exp(-p * r * r) * erf(math.sqrt(xi) * r) * r
    ref = -Z * quad(f, 0, 20 / math.sqrt(p), epsabs=1e-14, epsrel=1e-13, limit=200)[0]
    # element (s1/2 m=-1/2 of a, same of b): first large block, functions 0 and 1
    v = V[0, 1].real
    assert abs(v - ref) < 1e-10 * abs(ref)
    # a point nucleus gives the bare 1/r value, which the Gaussian lowers
    S2, V2, T2 = orc.oneel(b, [Z], [0.0])
    assert V2[0, 1].real < v
