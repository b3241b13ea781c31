"""The GPU's one-centre Coulomb matrices (MD one-centre quartets, RACAH1
off) against the reference's Racah route restated in the oracle, FP64."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

import berthagpu  # noqa: E402
from berthagpu import deck, wfn  # noqa: E402
from oracle import racah1  # noqa: E402

TOL = 1e-11


@pytest.mark.parametrize("shells", [
    {0: [0.25, 1.9, 14.0, 110.0], 1: [0.4, 3.1, 25.0]},
    {0: [0.2, 2.0, 30.0], 1: [0.35, 4.0], 2: [0.9, 5.5]},
    {0: [0.3, 9.0], 1: [0.6], 2: [1.2], 3: [1.8]},
])
def test_gpu_one_centre_matches_racah(shells):
    b = deck.make_basis([((0.0, 0.0, 0.0), shells)], hmlt="DHFR", isym=0)
    d = deck.density(b, seed=5)
    lrge, _ = wfn.fock_layout(b)
    rd, rx = racah1.coulomb1(b, d, lrge)
    fb = berthagpu.FockBuilder(b, racah1=False)
    gd, gx = fb.clmfast(d, 3)
    fb.close()
    scale = max(np.abs(rd).max(), np.abs(rx).max())
    assert np.abs(gd - rd).max() <= TOL * scale
    assert np.abs(gx - rx).max() <= TOL * scale


@pytest.mark.parametrize("shells", [
    {0: [0.25, 1.9, 14.0], 1: [0.4, 3.1]},
    {0: [0.2, 30.0], 1: [0.35, 4.0, 40.0]},
])
@pytest.mark.parametrize("prec", ["fp64", "tc32"])
def test_gpu_one_centre_breit_matches_racah(shells, prec):
    """The GPU's one-centre Breit exchange (MD, RACAH1 off) against BREIT1's
    Racah route, s and p shells (FP64 bound 1e-11, tensor cores 2e-5)."""
    b = deck.make_basis([((0.0, 0.0, 0.0), shells)], hmlt="DHFB", isym=0)
    d = deck.density(b, seed=9)
    lrge, _ = wfn.fock_layout(b)
    rb = racah1.breit1(b, d, lrge)
    fb = berthagpu.FockBuilder(b, racah1=False)
    fb.set_precision(prec)
    bx = fb.brtfast(d, 3)
    fb.close()
    tol = TOL if prec == "fp64" else 2e-5
    assert np.abs(bx - rb).max() <= tol * np.abs(rb).max()
