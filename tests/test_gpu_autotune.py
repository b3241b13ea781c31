"""BG_PREC_AUTO: per angular class the faster of the FP64 and the
split-precision kernel, chosen by timing both on the first build.

Its matrices must equal the FP64 build's within the split path's bound
(1e-12 relative to the largest element, as the split-precision tests), and
every listed quartet must be digested by exactly one of the two kernels.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

import torch  # noqa: E402

import berthagpu  # noqa: E402
from berthagpu import deck  # noqa: E402

TOL_DF = 1e-12


def _build(basis, prec, dent, repeat=1):
    fb = berthagpu.FockBuilder(basis)
    fb.set_precision(prec)
    fb.set_screening(1e-12)
    out = None
    for _ in range(repeat):
        out = fb.clmfast(dent, 3)
    stats = fb.auto_stats() if prec == "auto" else None
    fb.close()
    return out, stats


def test_auto_matches_fp64_h2o():
    b = deck.h2o_basis()
    d = deck.density(b, seed=5)
    (rd, rx), _ = _build(b, "fp64", d)
    # the second build replays the tuned runs
    (gd, gx), st = _build(b, "auto", d, repeat=2)
    scale = max(np.abs(rd).max(), np.abs(rx).max())
    assert np.abs(gd - rd).max() <= TOL_DF * scale
    assert np.abs(gx - rx).max() <= TOL_DF * scale
    assert st["runs"] >= 1
    assert st["fp64_quartets"] + st["df32_quartets"] > 0
    # H2O's heavy classes (general shape, complex digestion) run faster split
    assert st["df32_quartets"] > 0


def test_auto_batch_atoms():
    zs = [10, 12, 10, 18]
    bases = [deck.atom_basis(z) for z in zs]
    dens = [deck.density(b, seed=40 + k, real=True) for k, b in enumerate(bases)]
    refs = []
    fbs = []
    for b, d in zip(bases, dens):
        fb = berthagpu.FockBuilder(b, racah1=False)
        fb.set_screening(1e-12)
        refs.append(fb.clmfast(d, 3))
        fb.set_precision("auto")
        fbs.append(fb)
    batch = berthagpu.FockBatch(fbs)
    for fb in fbs:
        fb.close()
    D = torch.from_numpy(np.concatenate([d.ravel(order="F") for d in dens])).cuda()
    J, K = torch.zeros_like(D), torch.zeros_like(D)
    for _ in range(2):
        batch.clmfast_device(D.data_ptr(), J.data_ptr(), K.data_ptr(), 3)
    torch.cuda.synchronize()
    st = batch.auto_stats()
    assert st["fp64_quartets"] + st["df32_quartets"] == batch.quartets()
    Jh, Kh = J.cpu().numpy(), K.cpu().numpy()
    off = 0
    for (rd, rx), d in zip(refs, dens):
        n = d.shape[0]
        gd = Jh[off:off + n * n].reshape(n, n, order="F")
        gx = Kh[off:off + n * n].reshape(n, n, order="F")
        scale = max(np.abs(rd).max(), np.abs(rx).max())
        assert np.abs(gd - rd).max() <= TOL_DF * scale
        assert np.abs(gx - rx).max() <= TOL_DF * scale
        off += n * n
    batch.close()
