"""GPU one-electron matrices (bertha_gpu_oneel) against the oracle."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

import berthagpu  # noqa: E402
from berthagpu import deck  # noqa: E402
from oracle import oracle as orc  # noqa: E402


def _cmp(b, znuc, xi):
    fb = berthagpu.FockBuilder(b)
    got = fb.oneel(znuc, xi)
    fb.close()
    ref = orc.oneel(b, znuc, xi)
    for g, r in zip(got, ref):
        assert np.abs(g - r).max() <= 1e-11 * max(np.abs(r).max(), 1.0)


@pytest.mark.parametrize("hmlt", ["DHFR", "NORL"])
def test_oneel_small(hmlt):
    b = deck.make_basis([((0.0, 0.0, 0.0), {0: [0.3, 2.5], 1: [0.7], 2: [1.1]}),
                         ((0.3, -0.8, 1.3), {0: [0.45], 1: [1.1], 3: [0.9]}),
                         ((-1.0, 0.5, 0.4), {0: [0.9, 0.2]})], hmlt=hmlt)
    _cmp(b, [8.0, 1.0, 3.0], [0.0, 2.0e9, 5.0e8])


def test_oneel_h2o_gaussian_nuclei():
    b = deck.h2o_basis()
    _cmp(b, b.znuc, deck.nuclear_exponents(b.znuc, b.anuc))
