"""GPU Breit exchange build (bertha_gpu_brtfast) against the oracle, through
the C ABI.

Both sides are FP64 and differ only in summation order, so the bound is
1e-11 relative to the largest matrix element.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

import berthagpu  # noqa: E402
from berthagpu import deck  # noqa: E402
from oracle import oracle as orc  # noqa: E402

TOL = 1e-11


def _basis(lmax=1, hmlt="DHFB"):
    cent = [((0.0, 0.0, 0.0), {0: [0.3, 2.5], 1: [0.7]}),
            ((0.3, -0.8, 1.3), {0: [0.45], 1: [1.1]}),
            ((-1.0, 0.5, 0.4), {0: [0.9, 0.2]})]
    if lmax >= 2:
        cent[0][1][2] = [0.8]
    if lmax >= 3:
        cent[1][1][3] = [0.6]
    return deck.make_basis(cent, hmlt=hmlt)


def _cmp(b, dent, ilev, racah1=True, gaunt=False):
    fb = berthagpu.FockBuilder(b, racah1=racah1, gaunt=gaunt)
    bx = fb.brtfast(dent, ilev)
    fb.close()
    ref = orc.brtfast(b, dent, ilev, racah1=racah1, gaunt=gaunt)
    scale = max(np.abs(ref).max(), 1e-300)
    assert np.abs(bx - ref).max() <= TOL * scale
    return ref


@pytest.mark.parametrize("gaunt", [False, True])
def test_breit_small_general(gaunt):
    b = _basis()
    ref = _cmp(b, deck.density(b, seed=31), 3, gaunt=gaunt)
    assert np.abs(ref).max() > 0


@pytest.mark.parametrize("lmax", [2, 3])
def test_breit_high_l(lmax):
    b = _basis(lmax=lmax)
    _cmp(b, deck.density(b, seed=32), 3)


def test_breit_linear_real_digestion():
    b = deck.make_basis([((0, 0, 0), {0: [0.4, 1.9], 1: [0.8], 2: [1.2]}),
                         ((0, 0, 2.1), {0: [0.6], 1: [0.5]})], hmlt="DHFB")
    assert b.isym == 1
    _cmp(b, deck.density(b, seed=33, real=True), 3)


def test_breit_one_centre_by_md():
    """RACAH1 off: one-centre quartets enter at every stage, multi-centre
    ones from stage 3 (bertha-scf.f:17226-17231)."""
    b = _basis()
    d = deck.density(b, seed=34)
    _cmp(b, d, 1, racah1=False)
    _cmp(b, d, 3, racah1=False)


def test_breit_stage_gating():
    b = _basis()
    fb = berthagpu.FockBuilder(b)
    bx = fb.brtfast(deck.density(b, seed=35), 2)
    fb.close()
    assert np.abs(bx).max() == 0.0


def test_breit_needs_small_components():
    b = _basis(hmlt="NORL")
    fb = berthagpu.FockBuilder(b)
    with pytest.raises(berthagpu.BerthaGPUError):
        fb.brtfast(deck.density(b), 3)
    fb.close()


def test_breit_after_coulomb_same_context():
    """Breit and Coulomb builds share one context and its device buffers."""
    b = _basis()
    d = deck.density(b, seed=36)
    fb = berthagpu.FockBuilder(b)
    gd, gx = fb.clmfast(d, 3)
    bx = fb.brtfast(d, 3)
    gd2, gx2 = fb.clmfast(d, 3)
    fb.close()
    assert np.array_equal(gd, gd2) or np.abs(gd - gd2).max() <= 1e-13 * np.abs(gd).max()
    ref = orc.brtfast(b, d, 3)
    assert np.abs(bx - ref).max() <= TOL * np.abs(ref).max()


def test_breit_schwarz_screening():
    """Schwarz screening of the Breit build (bounds from the negative
    semidefinite Breit kernel): at 1e-12 the exchange matrix stays within
    1e-9 of the unscreened oracle; a huge threshold leaves nothing; 0 turns
    it off again."""
    b = deck.make_basis([((0, 0, 0), {0: [0.1, 50.0, 5.0e4], 1: [0.3, 2.0e3]}),
                         ((0, 0, 6.0), {0: [0.2, 8.0e4], 1: [1.0e3]}),
                         ((5.0, 1.0, 2.0), {0: [0.15, 3.0e4]})], hmlt="DHFB")
    dent = deck.density(b, seed=37)
    ref = orc.brtfast(b, dent, 3)
    fb = berthagpu.FockBuilder(b)
    fb.set_screening(1e-12)
    bx = fb.brtfast(dent, 3)
    assert np.abs(bx - ref).max() <= 1e-9
    fb.set_screening(1e3)
    assert np.abs(fb.brtfast(dent, 3)).max() == 0.0
    fb.set_screening(0.0)
    bx = fb.brtfast(dent, 3)
    assert np.abs(bx - ref).max() <= TOL * np.abs(ref).max()
    fb.close()


def _tlf_like():
    """TlF geometry with f functions on Tl and d on F, a few exponents each:
    linear real digestion, high l, sparse E and both contraction orders."""
    tl = {0: deck.geometric(0.5, 12.0, 3), 1: deck.geometric(0.4, 10.0, 2), 2: [0.8, 6.0],
          3: [1.5]}
    f = {0: deck.geometric(0.3, 9.0, 2), 1: [0.6], 2: [1.1]}
    return deck.make_basis([((0, 0, 0), tl), ((0, 0, 3.94), f)], hmlt="DHFB")


def test_tlf_like_coulomb_and_breit():
    b = _tlf_like()
    assert b.isym == 1
    d = deck.density(b, seed=3, real=True)
    fb = berthagpu.FockBuilder(b)
    gd, gx = fb.clmfast(d, 3)
    bx = fb.brtfast(d, 3)
    fb.set_precision("df32")
    gdm, gxm = fb.clmfast(d, 3)
    fb.close()
    rd, rx = orc.clmfast(b, d, 3)
    rb = orc.brtfast(b, d, 3)
    s = max(np.abs(rd).max(), np.abs(rx).max())
    assert np.abs(gd - rd).max() <= TOL * s and np.abs(gx - rx).max() <= TOL * s
    assert np.abs(gdm - rd).max() <= 1e-10 * s and np.abs(gxm - rx).max() <= 1e-10 * s
    assert np.abs(bx - rb).max() <= TOL * np.abs(rb).max()
