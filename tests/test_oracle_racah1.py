"""The one-centre Coulomb matrices by the reference's default route (Racah
algebra and beta-function radial integrals, COULOMB1) against the MD
one-centre quartets of the oracle (RACAH1 off, the route the GPU library
uses for one-centre terms).  The two are independent algorithms for the
same integrals: their agreement pins the MD one-centre path to the
reference's own algorithm."""
import numpy as np
import pytest

from berthagpu import deck, wfn
from oracle import oracle as orc
from oracle import racah1

TOL = 1e-12


def _atom(shells, seed):
    b = deck.make_basis([((0.0, 0.0, 0.0), shells)], hmlt="DHFR", isym=0)
    d = deck.density(b, seed=seed)
    lrge, _ = wfn.fock_layout(b)
    rd, rx = racah1.coulomb1(b, d, lrge)
    md, mx = orc.clmfast(b, d, 3, racah1=False)
    scale = max(np.abs(md).max(), np.abs(mx).max())
    return np.abs(rd - md).max() / scale, np.abs(rx - mx).max() / scale


def test_sym3j_against_sympy():
    wigner = pytest.importorskip("sympy.physics.wigner")
    from sympy import Rational
    for ja in (1, 3, 5, 7):
        for jb in (1, 3, 5):
            for l in range(0, 5):
                for ma in range(-ja, ja + 1, 2):
                    for mb in range(-jb, jb + 1, 2):
                        for m in range(-l, l + 1):
                            ref = float(wigner.wigner_3j(Rational(ja, 2), l, Rational(jb, 2),
                                                         Rational(ma, 2), m, Rational(mb, 2)))
                            assert abs(racah1.sym3j(ja, l, jb, ma, m, mb) - ref) < 1e-14


@pytest.mark.parametrize("case,shells", [
    ("Ne-like s,p", {0: [0.25, 1.9, 14.0, 110.0], 1: [0.4, 3.1, 25.0]}),
    ("Ar-like s,p,d", {0: [0.2, 2.0, 30.0], 1: [0.35, 4.0], 2: [0.9, 5.5]}),
    ("s,p,d,f", {0: [0.3, 9.0], 1: [0.6], 2: [1.2], 3: [1.8]}),
])
def test_racah_matches_md_one_centre(case, shells):
    ej, ek = _atom(shells, seed=len(case))
    assert ej <= TOL and ek <= TOL, (case, ej, ek)


def test_racah_wide_exponent_range():
    """Exponent ratios of 1e4 within one shell (core and valence)."""
    ej, ek = _atom({0: [0.05, 1.0, 40.0, 600.0], 1: [0.1, 8.0]}, seed=11)
    assert ej <= TOL and ek <= TOL, (ej, ek)


@pytest.mark.parametrize("shells", [
    {0: [0.5]},
    {0: [0.25, 1.9, 14.0], 1: [0.4, 3.1]},
    {0: [0.2, 30.0], 1: [0.35, 4.0, 40.0]},
])
def test_racah_breit_matches_md_one_centre(shells):
    """BREIT1's Racah route (Gaunt plus gauge, Grant and Pyper's
    coefficients) against the MD one-centre Breit quartets, s and p shells.
    (From d shells on, BREIT1 limits the tensor orders by the triangle of
    the large components' l and leaves out terms such as (ss|sd) that the
    MD route, like BRTFAST's own RACAH1-off path, includes.)"""
    b = deck.make_basis([((0.0, 0.0, 0.0), shells)], hmlt="DHFB", isym=0)
    d = deck.density(b, seed=9)
    lrge, _ = wfn.fock_layout(b)
    rb = racah1.breit1(b, d, lrge)
    mb = orc.brtfast(b, d, 3, racah1=False)
    assert np.abs(rb - mb).max() <= TOL * np.abs(mb).max()


def test_breit_one_centre_keeps_magnetic_terms():
    """BRTFAST's one-centre selection (RACAH1 off) keeps tensor orders with
    l_a + l_b + nu and l_c + l_d + nu both odd: the p1/2-p3/2 exchange of a
    p1/2 density is nonzero for the Breit interaction (and zero for the
    Coulomb one, where only even orders couple)."""
    b = deck.make_basis([((0.0, 0.0, 0.0), {0: [0.5], 1: [0.8]})], hmlt="DHFB", isym=0)
    lrge, labels = wfn.fock_layout(b)
    kap = np.concatenate([labels[:, 1], labels[:, 1]])
    d0 = deck.density(b, seed=3)
    p12 = kap == 1
    d = np.where(p12[:, None] & p12[None, :], d0, 0)
    bx = orc.brtfast(b, d, 3, racah1=False)
    blk = np.ix_(kap == 1, kap == -2)
    assert np.abs(bx[blk]).max() > 1e-3
    assert np.abs(bx[blk] - racah1.breit1(b, d, lrge)[blk]).max() < 1e-12


def test_reference_default_route_equals_md_route_on_a_molecule():
    """A diatomic by the reference's default route (CLMFAST with RACAH1 on
    for the multi-centre terms, COULOMB1 on each centre, as HFSCF calls them
    at :5401-5421) and by the MD route throughout (RACAH1 off, the GPU
    library's route): the same two-electron Fock matrix, on densities with
    the molecule's symmetry (superposed atomic densities and the SCF's
    first iterations).  (CLMFAST's real digestion for linear molecules
    assumes that symmetry; COULOMB1's digestion does not, so the bound
    allows for the eigensolver's rounding-level breaking of it.)"""
    import multiprocessing as mp
    from concurrent.futures import ProcessPoolExecutor

    import torch

    from berthagpu.scf import DHFSCF, atomic_guess
    from scf_oracle import OracleBackend, ReferenceRouteBackend
    # closed-shell atoms in these functions, so that the atomic densities
    # are spherical (a partly filled degenerate shell would break the
    # symmetry the real digestion assumes)
    A = {0: deck.geometric(0.3, 2.5, 4), 1: deck.geometric(0.5, 2.5, 2), 2: [1.2]}
    B = {0: deck.geometric(0.2, 2.5, 4), 1: deck.geometric(0.4, 2.5, 2), 2: [0.9], 3: [1.5]}
    b = deck.make_basis([((0, 0, 0), A), ((0, 0, 2.1), B)], hmlt="DHFR")
    b.znuc, b.anuc = (10.0, 12.0), (20.0, 24.0)
    md = lambda a: OracleBackend(a, racah1=False)  # noqa: E731
    D0 = torch.as_tensor(atomic_guess(b, torch=torch, backend_factory=md, max_iter=40,
                                      etol=1e-10))
    r = DHFSCF(b, nocc=22, torch=torch, backend=md(b)).run(max_iter=3, guess=D0,
                                                            return_density=True)
    with ProcessPoolExecutor(max_workers=2, mp_context=mp.get_context("spawn")) as pool:
        for D in (D0, r["density"]):
            g_ref = ReferenceRouteBackend(b, pool, torch).fock(D).numpy()
            g_md = md(b).fock(D).numpy()
            assert np.abs(g_ref - g_md).max() <= 1e-10 * np.abs(g_md).max()
