"""BG_PREC_AUTO: per angular class and Schwarz-bound decade the fastest of
the FP64, split-precision and tensor-core kernels, chosen by timing all
three on the first build, the tensor-core kernel only within the error
budget (energy error per build, default 1e-7 Eh).

Every listed quartet must be digested by exactly one kernel.  Without a
budget the matrices equal the FP64 build's within the split path's bound
(1e-12 relative to the largest element); with the default budget the energy
terms stay within the budget, and the matrices within the tensor-core bound
where that kernel took part.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

import torch  # noqa: E402

import berthagpu  # noqa: E402
from berthagpu import deck  # noqa: E402

TOL_DF = 1e-12
TOL_TC = 2e-5      # tensor-core bound, relative to the largest element
BUDGET = 1e-7      # the default error budget, Eh per build


def _energies(d, g):
    gd, gx = g
    return 0.5 * np.sum(d * gd).real, 0.5 * np.sum(d * gx).real


def _build(basis, prec, dent, repeat=1, budget=None):
    fb = berthagpu.FockBuilder(basis)
    fb.set_precision(prec)
    fb.set_screening(1e-12)
    if budget is not None:
        fb.set_error_budget(budget)
    out = None
    for _ in range(repeat):
        out = fb.clmfast(dent, 3)
    stats = fb.auto_stats() if prec == "auto" else None
    fb.close()
    return out, stats


def _total(st):
    return st["fp64_quartets"] + st["df32_quartets"] + st["tc32_quartets"]


def test_auto_matches_fp64_h2o():
    b = deck.h2o_basis()
    d = deck.density(b, seed=5)
    ref = _build(b, "fp64", d)[0]
    rd, rx = ref
    scale = max(np.abs(rd).max(), np.abs(rx).max())
    # without a budget: FP64 and split kernels only, FP64-accurate
    # (the second build replays the tuned runs)
    (gd, gx), st = _build(b, "auto", d, repeat=2, budget=0.0)
    assert np.abs(gd - rd).max() <= TOL_DF * scale
    assert np.abs(gx - rx).max() <= TOL_DF * scale
    assert st["runs"] >= 1 and st["tc32_quartets"] == 0
    # H2O's heavy classes (general shape, complex digestion) run faster split
    assert st["df32_quartets"] > 0
    # the default budget: energy terms within it
    g, st2 = _build(b, "auto", d, repeat=2)
    assert _total(st2) == _total(st)
    ej, ek = _energies(d, ref)
    aj, ak = _energies(d, g)
    assert abs(aj - ej) + abs(ak - ek) <= BUDGET
    tol = TOL_TC if st2["tc32_quartets"] else TOL_DF
    assert np.abs(g[0] - rd).max() <= tol * scale
    assert np.abs(g[1] - rx).max() <= tol * scale


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
    assert _total(st) == batch.quartets()
    tol = TOL_TC if st["tc32_quartets"] else TOL_DF
    Jh, Kh = J.cpu().numpy(), K.cpu().numpy()
    off = 0
    err = 0.0
    for (rd, rx), d in zip(refs, dens):
        n = d.shape[0]
        gd = Jh[off:off + n * n].reshape(n, n, order="F")
        gx = Kh[off:off + n * n].reshape(n, n, order="F")
        scale = max(np.abs(rd).max(), np.abs(rx).max())
        assert np.abs(gd - rd).max() <= tol * scale
        assert np.abs(gx - rx).max() <= tol * scale
        ej, ek = _energies(d, (rd, rx))
        aj, ak = _energies(d, (gd, gx))
        err += abs(aj - ej) + abs(ak - ek)
        off += n * n
    # the batch shares one budget
    assert err <= BUDGET
    batch.close()
