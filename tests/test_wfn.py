"""Wavefunction files, the FOCKIND layout and the atomic-density start, on
the CPU: the layout against the oracle's FOCKIND, `.wfn` round trips
(including the list-directed forms a Fortran runtime writes: records split
over lines, D exponents, repeat counts), DENSTY, and the superposed atomic
guess of an SCF on the oracle backend."""
import numpy as np
import torch

from berthagpu import deck, wfn
from berthagpu.scf import DHFSCF, atomic_guess
from oracle import oracle as orc
from scf_oracle import OracleBackend


def _mol():
    o = {0: [0.2, 1.1, 6.0], 1: [0.5, 2.0], 2: [0.9]}
    h = {0: [0.15, 1.3]}
    b = deck.make_basis([((0, 0, 0), o), ((0.0, 1.2, 0.9), h), ((0.0, -1.2, 0.9), h)],
                        hmlt="DHFR")
    b.znuc, b.anuc = (8.0, 1.0, 1.0), (16.0, 1.0, 1.0)
    return b


def test_fock_layout_matches_oracle():
    for b in (_mol(), deck.tlf_small_basis(), deck.atom_basis(36)):
        lrge, labels = wfn.fock_layout(b)
        ndim, nskp, lr = orc.fock_layout(b)
        assert nskp == b.nskp == len(labels)
        defined = lr >= 0
        assert np.array_equal(lrge[:, :lr.shape[1], :][defined], lr[defined])
        assert np.all(lrge[:, :lr.shape[1], :][~defined] == -1)
        # every large-component index appears once
        assert np.array_equal(np.sort(np.concatenate(
            [np.arange(v, v + b.nfn[c, wfn.lval(wfn.kappa_of(k))])
             for (c, k, m), v in np.ndenumerate(lrge) if v >= 0])), np.arange(nskp))


def test_wfn_round_trip(tmp_path):
    rng = np.random.default_rng(3)
    n = 12
    e = np.sort(rng.normal(size=n)) * 100
    C = rng.normal(size=(n, n)) + 1j * rng.normal(size=(n, n))
    p = tmp_path / "x.wfn"
    wfn.write_wfn(p, e, C)
    e2, C2 = wfn.read_wfn(p, n)
    assert np.array_equal(e, e2) and np.array_equal(C, C2)


def test_wfn_reads_fortran_list_directed(tmp_path):
    # records split over lines, D exponents, spaces inside the parentheses
    # and a repeat count, as Fortran runtimes write list-directed output
    text = (" -1.5D+00 (  1.0D+00,  0.0D+00) (0.5,-0.25)\n"
            "  (0.0,0.0)\n"
            "  2.0 2*(0.0,1.0)\n (3.0E-1,4.0E-1)\n"
            " 7.0  (1,2) (3,4) (5,6)\n")
    p = tmp_path / "f.wfn"
    p.write_text(text)
    e, C = wfn.read_wfn(p, 3)
    assert np.allclose(e, [-1.5, 2.0, 7.0])
    assert np.allclose(C[:, 0], [1.0, 0.5 - 0.25j, 0.0])
    assert np.allclose(C[:, 1], [1j, 1j, 0.3 + 0.4j])
    assert np.allclose(C[:, 2], [1 + 2j, 3 + 4j, 5 + 6j])


def test_density_is_densty():
    rng = np.random.default_rng(5)
    C = rng.normal(size=(8, 8)) + 1j * rng.normal(size=(8, 8))
    D = wfn.density(C, 4, 2)
    ref = np.zeros((8, 8), complex)
    for k in (4, 5):
        ref += np.outer(np.conj(C[:, k]), C[:, k])
    assert np.allclose(D, ref)


def test_centre_blocks_partition_the_molecule():
    b = _mol()
    idx = np.concatenate([wfn.centre_index_map(b, c, wfn.atom_of_centre(b, c))
                          for c in range(b.ncnt)])
    assert np.array_equal(np.sort(idx), np.arange(b.ndim))
    # an atom embedded in itself is the identity placement
    a = wfn.atom_of_centre(b, 0)
    assert np.array_equal(wfn.centre_index_map(a, 0, a), np.arange(a.ndim))


def test_atomic_guess_scf_on_oracle_backend():
    """H2 from two hydrogen atoms: the superposed atomic density starts the
    molecular SCF, which reaches the same energy as from the bare nucleus."""
    h = {0: deck.geometric(0.1, 3.0, 4)}
    b = deck.make_basis([((0, 0, 0), h), ((0, 0, 1.4), h)], hmlt="DHFR")
    b.znuc, b.anuc = (1.0, 1.0), (1.0, 1.0)
    factory = lambda atom: OracleBackend(atom, racah1=False)  # noqa: E731
    D0 = atomic_guess(b, torch=torch, backend_factory=factory)
    assert D0.shape == (b.ndim, b.ndim)
    assert np.allclose(D0, D0.conj().T) and np.abs(D0).max() > 0
    ref = DHFSCF(b, nocc=2, torch=torch, backend=OracleBackend(b, racah1=False))
    r0 = ref.run(max_iter=40, etol=1e-10)
    scf = DHFSCF(b, nocc=2, torch=torch, backend=OracleBackend(b, racah1=False))
    r1 = scf.run(max_iter=40, etol=1e-10, guess=D0)
    assert r0["converged"] and r1["converged"]
    assert abs(r0["energy"] - r1["energy"]) < 1e-8


def test_atomic_guess_energy_of_distant_ions():
    """Two atoms 30 bohr apart with s, p, d (and f) functions, one of them
    an ion (the deck's electron count): the molecule's energy at the
    superposed atomic densities is the sum of the atoms' SCF energies plus
    the ions' Coulomb energy, which checks the placement of every (kappa, m)
    block of both centres."""
    A = {0: deck.geometric(0.3, 2.5, 6), 1: deck.geometric(0.5, 2.5, 3), 2: [1.2]}
    B = {0: deck.geometric(0.2, 2.5, 6), 1: deck.geometric(0.4, 2.5, 3), 2: [0.9], 3: [1.5]}
    R = np.array([0.3, 0.4, 30.0])
    b = deck.make_basis([((0, 0, 0), A), (tuple(R), B)], hmlt="DHFR")
    b.znuc, b.anuc = (10.0, 12.0), (20.0, 24.0)
    nelec = (10, 10)  # neon-like atom and a doubly charged magnesium-like ion
    factory = lambda atom: OracleBackend(atom, racah1=False)  # noqa: E731
    e_atoms = []
    for c in range(2):
        atom = wfn.atom_of_centre(b, c, hmlt="DHFR")
        r = DHFSCF(atom, nocc=nelec[c], torch=torch, backend=factory(atom)).run(
            max_iter=40, etol=1e-10, mom=2)
        assert r["converged"]
        e_atoms.append(r["energy"])
    D0 = atomic_guess(b, torch=torch, backend_factory=factory, max_iter=40, etol=1e-10,
                      nelec=nelec)
    S = factory(b).oneel()[0].numpy()
    assert abs(np.sum(D0 * S).real - sum(nelec)) < 1e-8  # ENRGIES' sum with the overlap
    e = DHFSCF(b, nocc=20, torch=torch, backend=factory(b)).energy_at(torch.as_tensor(D0))
    # the neutral atom sees the ion's charge only through its own tails:
    # the remaining interaction is far below the checked bound
    assert abs(e - sum(e_atoms)) < 1e-6, (e, sum(e_atoms))
