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
