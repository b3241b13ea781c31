"""The SCF loop (berthagpu.scf.DHFSCF) on the oracle backend, on the CPU:
the helium atom's Dirac-Hartree-Fock energy against its published value
(-2.8618133 Eh, finite basis: within 2e-6), which pins the one-electron
matrices, the MD one-centre two-electron integrals with CLMMTZ's real
digestion, and the driver's energy, occupation and DIIS logic at once."""
import pytest
import torch

from berthagpu import deck
from berthagpu.scf import DHFSCF
from scf_oracle import OracleBackend


def test_helium_dhf_energy():
    he = deck.make_basis([((0.0, 0.0, 0.0), {0: deck.geometric(0.06, 2.1, 18)})], hmlt="DHFR")
    he.znuc, he.anuc = (2.0,), (4.0,)
    scf = DHFSCF(he, nocc=2, torch=torch, backend=OracleBackend(he, racah1=False))
    r = scf.run(max_iter=30, etol=1e-10)
    assert r["converged"]
    assert abs(r["energy"] - (-2.8618133)) < 2e-6
    # Kramers-degenerate 1s1/2 pair
    e = r["orbital_energies"]
    assert abs(e[0] - e[1]) < 1e-10 and abs(e[0] - (-0.91799)) < 1e-4


def test_helium_maximum_overlap_and_wfn(tmp_path):
    """Maximum-overlap occupation from the second iteration reaches the same
    helium energy as aufbau, and the `.wfn` file it writes restarts the SCF
    at convergence."""
    from berthagpu import wfn
    he = deck.make_basis([((0.0, 0.0, 0.0), {0: deck.geometric(0.06, 2.1, 18)})], hmlt="DHFR")
    he.znuc, he.anuc = (2.0,), (4.0,)
    path = str(tmp_path / "he.wfn")
    scf = DHFSCF(he, nocc=2, torch=torch, backend=OracleBackend(he, racah1=False))
    r = scf.run(max_iter=30, etol=1e-10, mom=2, wfn_out=path)
    assert r["converged"]
    assert abs(r["energy"] - (-2.8618133)) < 2e-6
    eign, coef = wfn.read_wfn(path, he.ndim)
    assert abs(eign[he.nskp] - r["orbital_energies"][0]) < 1e-12
    scf = DHFSCF(he, nocc=2, torch=torch, backend=OracleBackend(he, racah1=False))
    r2 = scf.run(max_iter=30, etol=1e-10, guess=(eign, coef))
    assert r2["converged"] and r2["iterations"] <= 3
    assert abs(r2["energy"] - r["energy"]) < 1e-9


@pytest.mark.parametrize("hmlt", ["DHFR", "DHFB"])
def test_staged_inclusion_reaches_the_same_solution(hmlt):
    """HFSCF's integral inclusion stages (ILEV 1 with a 3 Eh level shift,
    ILEV 2 with 1 Eh, then ILEV 3; multi-centre Breit terms from ILEV 3 on)
    change the path, not the converged energy: H2 at 1.4 bohr, staged and
    unstaged, Dirac-Coulomb and Dirac-Coulomb-Breit."""
    h = {0: deck.geometric(0.08, 3.0, 6), 1: [0.6]}
    h2 = deck.make_basis([((0.0, 0.0, 0.0), h), ((0.0, 0.0, 1.4), h)], hmlt=hmlt)
    h2.znuc, h2.anuc = (1.0, 1.0), (1.0, 1.0)
    breit = hmlt == "DHFB"
    out = {}
    for staged in (False, True):
        scf = DHFSCF(h2, nocc=2, torch=torch,
                     backend=OracleBackend(h2, racah1=False, breit=breit))
        r = scf.run(max_iter=60, etol=1e-11, dtol=1e-8, shift=0.0,
                    stages=((1, 3.0, 1e-8, 12), (2, 1.0, 5e-11, 15)) if staged else None)
        assert r["converged"], (staged, r["history"][-3:])
        out[staged] = r
    levels = [h["ilev"] for h in out[True]["history"]]
    assert levels[0] == 1 and 2 in levels and levels[-1] == 3
    assert levels == sorted(levels)
    assert all(h["ilev"] == 3 for h in out[False]["history"])
    assert abs(out[True]["energy"] - out[False]["energy"]) < 1e-9
    # stage 1 leaves out the two-centre (LL|SS), (SS|LL) and (SS|SS) terms:
    # its energies differ from the full Hamiltonian's
    e1 = [h["energy"] for h in out[True]["history"] if h["ilev"] == 1][-1]
    assert abs(e1 - out[False]["energy"]) > 1e-7
