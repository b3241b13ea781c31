"""The reference's own recorded Dirac-Coulomb SCF of YbF+ (R = 3.88 bohr,
NDIM 1052, Yb 26s26p15d8f / F 10s6p with exponents up to 1.6e9, Gaussian
nuclei) as a golden result for the whole Fock-build chain: basis and
kinetic balance, one-electron matrices, the two-electron Coulomb terms
(the one-centre ones by the MD route where the reference used its Racah
route) and the closed-shell SCF.  The fixture `golden/ybf_plus_388.json`
holds the deck's data and the energies the reference printed at every
iteration (written by `golden/make_ybf_golden.py` from the deck and the
log of its run).

The reference's run stopped with its last three stage-3 energies spread
over 4.4e-3 Eh (-14167.0575 to -14167.0618) and its occupied spinor
energies still moving by up to 5.0e-5 Eh per iteration, so its results
are known to those amounts, not to their printed digits; the test bounds
follow from them.  (Measured on a GB300: the GPU SCF ends at
-14167.060155 Eh, inside the band and 1.7e-3 Eh above the last printed
total, with all 78 occupied spinor energies within 1.3e-5 Eh of the
reference's.)
"""
import json
import os

import numpy as np
import pytest

from berthagpu import deck
from berthagpu.scf import CLIGHT, nuclear_repulsion

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "ybf_plus_388.json")


def _gold():
    with open(GOLD) as f:
        return json.load(f)


def _basis(g):
    cents = [(c["xyz"], {int(l): e for l, e in c["exponents"].items()}) for c in g["centres"]]
    b = deck.make_basis(cents, hmlt=g["hamiltonian_of_scf"], name="YbFplus_388")
    b.znuc = tuple(c["z"] for c in g["centres"])
    b.anuc = tuple(c["mass"] for c in g["centres"])
    return b


def test_fixture_basis_and_nuclei():
    """The fixture's basis gives the reference's Fock-matrix dimension, its
    geometry the printed nucleus-nucleus energy, and its energy terms add
    up to each printed total (ENRGIES' sum)."""
    g = _gold()
    b = _basis(g)
    assert b.ndim == g["ndim"] == 1052
    assert abs(g["speed_of_light"] - CLIGHT) < 1e-10
    for it in g["iterations"]:
        assert abs(nuclear_repulsion(b) - it["enuc"]) < 1e-9
        tot = it["enuc"] + it["enuc_el"] + it["ekin"] + it["gdir"] - it["gxch"]
        assert abs(tot - it["total"]) < 1e-8
    stage3 = [it["total"] for it in g["iterations"] if it["ilev"] == 3]
    assert len(stage3) == 3 and max(stage3) - min(stage3) < 5e-3


@pytest.mark.gpu
def test_ybf_dirac_coulomb_scf_matches_reference():
    """FP64 SCF on the GPU from the deck's atomic configurations (Yb 68 and
    F 10 electrons), through HFSCF's stages with the deck's level shifts
    (3, 1, 0 Eh), compared with the reference's last stage-3 iteration."""
    import torch

    from berthagpu.scf import DHFSCF, atomic_guess
    g = _gold()
    b = _basis(g)
    nelec = [c["nelec"] for c in g["centres"]]
    guess = atomic_guess(b, torch=torch, nelec=nelec)
    scf = DHFSCF(b, nocc=g["ncls"], precision="fp64", screen=1e-12, racah1=False, torch=torch)
    sh = g["shifts"]
    r = scf.run(max_iter=50, etol=1e-7, shift=sh[2], guess=guess, verbose=True,
                stages=((1, sh[0], 1e-8, 12), (2, sh[1], 5e-11, 15)))
    scf.close()
    last = g["iterations"][-1]
    ref_eps = np.sort([s["energy"] for s in g["spinors_last"]])[:g["ncls"]]
    eps = np.asarray(r["orbital_energies"])
    hist = r["history"]
    print(json.dumps({"energy": r["energy"], "iterations": r["iterations"],
                      "converged": r["converged"], "last_de": hist[-1]["de"],
                      "ddens": hist[-1]["ddens"], "fock_s": r["fock_s"],
                      "linalg_s": r["linalg_s"],
                      "delta_total": r["energy"] - last["total"],
                      "delta_spinors_max": float(np.abs(eps - ref_eps).max()),
                      "delta_spinors": (eps - ref_eps).tolist(),
                      "ilev": [h["ilev"] for h in hist],
                      "energies": [h["energy"] for h in hist]}), flush=True)
    assert r["converged"] and hist[-1]["ilev"] == 3
    stage3 = [it["total"] for it in g["iterations"] if it["ilev"] == 3]
    assert min(stage3) - 1e-3 <= r["energy"] <= max(stage3) + 1e-3
    # the reference's own last-iteration change of its spinor energies
    prev_eps = np.sort([s["energy"] for s in g["spinors_previous"]])[:g["ncls"]]
    drift = np.abs(ref_eps - prev_eps).max()
    assert drift < 6e-5
    assert np.abs(eps - ref_eps).max() < drift


def test_stage_plan_follows_the_deck():
    """The run module's HFSCF stage plan: from the deck's starting stage,
    its level shifts and HFSCF's stage tolerances; stage 3's shift is the
    last one."""
    from berthagpu.run import stage_plan
    plan, last = stage_plan({"ilev": 1, "shifts": (3.0, 1.0, 0.0)}, 0.5, 12)
    assert plan == [(1, 3.0, 1e-8, 12), (2, 1.0, 5e-11, 12)] and last == 0.0
    plan, last = stage_plan({"ilev": 2, "shifts": (3.0, 1.0, 0.25)}, 0.5, 9)
    assert plan == [(2, 1.0, 5e-11, 9)] and last == 0.25
    plan, last = stage_plan({"ilev": 3, "shifts": (3.0, 1.0, 0.0)}, 0.5, 9)
    assert plan == [] and last == 0.0
    plan, last = stage_plan({}, 0.5, 9)
    assert [p[0] for p in plan] == [1, 2] and last == 0.5


def test_log_parser_reads_iterations_and_spinors():
    """The fixture script's parser on a two-iteration excerpt in the log's
    layout: iteration headers, spinor table rows, ENRGIES' terms and the
    inclusion level."""
    import sys
    sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden"))
    from make_ybf_golden import parse_log
    block = """
                           Iteration number  {it}
 ========================================================================
 Orb.  Centre    Term sym.   m_j              Energy (au)      Population
 ------------------------------------------------------------------------
   1   1 (Yb)     1s_1/2    -1/2       -2268.0932706{d}      0.99999999
   2   2 (F )     2p_3/2     3/2          -0.7287{d}      0.50165025
 ========================================================================
 Nucleus-nucleus             (N)                         162.371134020619
 Electron-nucleus            (V)                      -49659.30514789204{d}
 Electron kinetic            (T)                       29887.61797559624{d}
 Coulomb direct (closed)     (GD)                       5738.70418349756{d}
 Coulomb exchange (closed)   (GX)                        298.44982271876{d}
 Molecule total                                       -14169.06167749638{d}
 Iteration number                                                      {it}
 Integral inclusion level                                               {lv}
"""
    text = block.format(it=1, d=1, lv=1) + block.format(it=12, d=2, lv=3)
    its = parse_log(text)
    assert [i["iter"] for i in its] == [1, 12] and [i["ilev"] for i in its] == [1, 3]
    assert its[1]["terms"]["total"] == -14169.061677496382
    assert its[0]["terms"]["gxch"] == 298.449822718761
    sp = its[1]["spinors"]
    assert len(sp) == 2 and sp[0]["term"] == "1s_1/2" and sp[1]["centre"] == 2
    assert sp[1]["energy"] == -0.72872 and sp[1]["mj"] == "3/2"
