"""Tensor-core (3xTF32 tcgen05) Fock build against the oracle, through the C ABI.

The contractions run as TF32 tensor-core GEMMs in three passes
(hi*hi + hi*lo + lo*hi, about 22 significant bits per operand) with FP32
accumulation, and the digestion products are FP32; Boys, R and the J/K sums
stay FP64.  The error is therefore FP32-like: the bound is TC_TOL of the
largest matrix element.  The autotuned mode spends an energy-error budget
on tensor-core classes; its test checks the energy against FP64 within the
budget.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

import berthagpu  # noqa: E402
from berthagpu import _lib, deck, workloads  # noqa: E402
from oracle import oracle as orc  # noqa: E402

TC_TOL = 2e-5


def _small(lmax=1, isym=None):
    cent = [((0.0, 0.0, 0.0), {0: [0.3, 2.5], 1: [0.7]}),
            ((0.3, -0.8, 1.3), {0: [0.45], 1: [1.1]}),
            ((-1.0, 0.5, 0.4), {0: [0.9, 0.2]})]
    if lmax >= 2:
        cent[0][1][2] = [0.8]
    if lmax >= 3:
        cent[1][1][3] = [0.6]
        cent[2][1][3] = [1.3]
    return deck.make_basis(cent, hmlt="DHFR", isym=isym)


def _cmp_tc(b, dent, ilev, tol=TC_TOL, racah1=True):
    fb = berthagpu.FockBuilder(b, racah1=racah1)
    fb.set_precision("tc32")
    gd, gx = fb.clmfast(dent, ilev)
    stats = fb.auto_stats()
    fb.close()
    assert _lib.device_status() == 0
    rd, rx = orc.clmfast(b, dent, ilev, racah1=racah1)
    scale = max(np.abs(rd).max(), np.abs(rx).max(), 1e-300)
    ed = np.abs(gd - rd).max() / scale
    ex = np.abs(gx - rx).max() / scale
    assert ed <= tol and ex <= tol, (ed, ex)
    assert stats["tc32_quartets"] > 0
    return gd, gx, rd, rx


@pytest.mark.parametrize("lmax", [1, 2, 3])
def test_tc_general(lmax):
    b = _small(lmax=lmax)
    _cmp_tc(b, deck.density(b, seed=30 + lmax), 3)


def test_tc_linear_real_digestion():
    b = deck.make_basis([((0, 0, 0), {0: [0.4, 1.9], 1: [0.8], 2: [1.2], 3: [0.9]}),
                         ((0, 0, 2.1), {0: [0.6], 1: [0.5], 2: [0.7]})], hmlt="DHFR")
    assert b.isym == 1
    _cmp_tc(b, deck.density(b, seed=5, real=True), 3)


def test_tc_one_centre_by_md():
    b = _small(lmax=2)
    _cmp_tc(b, deck.density(b, seed=9), 3, racah1=False)


def test_tc_extreme_exponents():
    """Exponent ratios up to 1e7 exercise the power-of-two balancing that
    keeps every operand inside the TF32 exponent range."""
    b = deck.make_basis([((0, 0, 0), {0: [0.05, 2.0e5], 1: [3.0e4], 2: [0.3]}),
                         ((0.4, 1.1, -0.7), {0: [1.0e6, 0.08], 1: [0.1]}),
                         ((1.5, -0.3, 0.9), {0: [0.5], 3: [40.0]})], hmlt="DHFR")
    _cmp_tc(b, deck.density(b, seed=8), 3)


def test_tc_h2o_stage3():
    b = deck.h2o_basis()
    _cmp_tc(b, deck.density(b, seed=1), 3)


def _pool(seed):
    rng = np.random.default_rng(seed)
    cents = [(rng.uniform(0, 6, 3), {l: list(np.exp(rng.uniform(np.log(0.1), np.log(50.0), 2)))
                                      for l in range(4)}) for _ in range(6)]
    return deck.make_basis(cents, hmlt="DHFR", isym=0)


def test_tc_explicit_lists_vs_oracle():
    """bertha_gpu_quartets in tensor-core precision on random quartets of
    every component class (l <= 3), against the oracle's digestion of the
    same lists."""
    import torch
    b = _pool(77)
    fb = berthagpu.FockBuilder(b)
    fb.set_precision("tc32")
    n = fb.ndim
    dent = deck.density(b, seed=6)
    D = torch.from_numpy(np.ascontiguousarray(dent.T).view(np.float64).reshape(n, 2 * n)).cuda()
    quarts = workloads.microbench_quartets(b, 2000, seed=3)
    O = orc.QuartetOracle(b)
    for cls, q in quarts.items():
        GD = torch.zeros(n, 2 * n, dtype=torch.float64, device="cuda")
        GX = torch.zeros_like(GD)
        dq = torch.from_numpy(q).cuda()
        fb.quartets(dq.data_ptr(), q.shape[0], cls[0], cls[1], D.data_ptr(), GD.data_ptr(),
                    GX.data_ptr(), n, torch.cuda.current_stream().cuda_stream)
        torch.cuda.synchronize()
        gd = GD.cpu().numpy().view(np.complex128).reshape(n, n).T
        gx = GX.cpu().numpy().view(np.complex128).reshape(n, n).T
        rd = np.zeros((n, n), complex, order="F")
        rx = np.zeros((n, n), complex, order="F")
        O.prepare(q, *cls)
        O.digest(q, *cls, dent, rd, rx, nthreads=8)
        scale = max(np.abs(rd).max(), np.abs(rx).max())
        assert np.abs(gd - rd).max() <= TC_TOL * scale, cls
        assert np.abs(gx - rx).max() <= TC_TOL * scale, cls
    assert _lib.device_status() == 0
    O.close()
    fb.close()


def test_tc_repeat_and_graph_capture():
    """A second build and a CUDA-graph replay of the tensor-core build give
    the first build's matrices (same density)."""
    import torch
    b = _small(lmax=2)
    n = b.ndim
    dent = deck.density(b, seed=12)
    fb = berthagpu.FockBuilder(b)
    fb.set_precision("tc32")
    D = torch.from_numpy(np.ascontiguousarray(dent.T)).cuda()
    J, K = torch.zeros_like(D), torch.zeros_like(D)
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(s):
        fb.clmfast_device(D.data_ptr(), J.data_ptr(), K.data_ptr(), 3, n, s.cuda_stream)
    s.synchronize()
    J1, K1 = J.clone(), K.clone()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=s):
        fb.clmfast_device(D.data_ptr(), J.data_ptr(), K.data_ptr(), 3, n,
                          torch.cuda.current_stream().cuda_stream)
    J.zero_()
    g.replay()
    torch.cuda.synchronize()
    scale = float(J1.abs().max())
    assert float((J - J1).abs().max()) <= 1e-6 * scale
    assert float((K - K1).abs().max()) <= 1e-6 * scale
    fb.close()


def test_auto_error_budget():
    """BG_PREC_AUTO: the energy terms of the tuned build stay within the
    error budget of the FP64 build's (the estimate is conservative), and a
    zero budget keeps every class FP64-accurate."""
    b = _small(lmax=3)
    dent = deck.density(b, seed=19)

    def energy(prec, budget=None):
        fb = berthagpu.FockBuilder(b)
        fb.set_precision(prec)
        if budget is not None:
            fb.set_error_budget(budget)
        gd, gx = fb.clmfast(dent, 3)
        gd, gx = fb.clmfast(dent, 3)
        st = fb.auto_stats() if prec == "auto" else None
        fb.close()
        return 0.5 * np.sum(dent * gd).real, 0.5 * np.sum(dent * gx).real, st

    ej, ek, _ = energy("fp64")
    for budget in (0.0, 1e-6):
        aj, ak, st = energy("auto", budget)
        assert abs(aj - ej) + abs(ak - ek) <= budget + 1e-11 * (abs(ej) + abs(ek))
        if budget == 0.0:
            assert st["tc32_quartets"] == 0


# ---- Breit on the tensor cores ----

def _breit_basis(lmax=1):
    cent = [((0.0, 0.0, 0.0), {0: [0.3, 2.5], 1: [0.7]}),
            ((0.3, -0.8, 1.3), {0: [0.45], 1: [1.1]}),
            ((-1.0, 0.5, 0.4), {0: [0.9, 0.2]})]
    if lmax >= 2:
        cent[0][1][2] = [0.8]
    if lmax >= 3:
        cent[1][1][3] = [0.6]
        cent[2][1][3] = [1.3]
    return deck.make_basis(cent, hmlt="DHFB")


def _cmp_breit_tc(b, dent, racah1=True, gaunt=False):
    fb = berthagpu.FockBuilder(b, racah1=racah1, gaunt=gaunt)
    fb.set_precision("tc32")
    bx = fb.brtfast(dent, 3)
    st = fb.breit_stats()
    fb.close()
    assert _lib.device_status() == 0
    ref = orc.brtfast(b, dent, 3, racah1=racah1, gaunt=gaunt)
    scale = max(np.abs(ref).max(), 1e-300)
    err = np.abs(bx - ref).max() / scale
    assert err <= TC_TOL, err
    assert st["tc32_quartets"] > 0
    return bx, ref


@pytest.mark.parametrize("gaunt", [False, True])
def test_breit_tc_general(gaunt):
    b = _breit_basis()
    _cmp_breit_tc(b, deck.density(b, seed=31), gaunt=gaunt)


@pytest.mark.parametrize("lmax", [2, 3])
def test_breit_tc_high_l(lmax):
    b = _breit_basis(lmax=lmax)
    _cmp_breit_tc(b, deck.density(b, seed=32))


def test_breit_tc_linear_real_digestion():
    b = deck.make_basis([((0, 0, 0), {0: [0.4, 1.9], 1: [0.8], 2: [1.2], 3: [0.9]}),
                         ((0, 0, 2.1), {0: [0.6], 1: [0.5]})], hmlt="DHFB")
    assert b.isym == 1
    _cmp_breit_tc(b, deck.density(b, seed=33, real=True))


def test_breit_tc_one_centre_by_md():
    b = _breit_basis(lmax=2)
    _cmp_breit_tc(b, deck.density(b, seed=34), racah1=False)


def test_breit_auto_error_budget():
    """BG_PREC_AUTO on the Breit build: energy within the budget of FP64's."""
    b = _breit_basis(lmax=3)
    dent = deck.density(b, seed=35)

    def energy(prec, budget=None):
        fb = berthagpu.FockBuilder(b)
        fb.set_precision(prec)
        if budget is not None:
            fb.set_error_budget(budget)
        fb.brtfast(dent, 3)
        bx = fb.brtfast(dent, 3)
        fb.close()
        return 0.5 * np.sum(dent * bx).real

    e64 = energy("fp64")
    for budget in (0.0, 1e-6):
        assert abs(energy("auto", budget) - e64) <= budget + 1e-12 * abs(e64)
