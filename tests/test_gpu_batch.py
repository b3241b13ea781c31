"""Batched Fock builds of independent instances (FockBatch over the C ABI's
bertha_gpu_batch_* entry points) against one context per instance.

Each instance of a batch must get exactly the matrices its own context
builds: the same quartet lists and kernels, only launched together.  Both
sides are FP64 GPU builds that differ in atomic summation order, so the
bound is 1e-11 relative to the largest element (as the oracle parity tests);
the split-precision batch is held to the split-precision tests' 1e-12.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

import torch  # noqa: E402

import berthagpu  # noqa: E402
from berthagpu import deck  # noqa: E402
from berthagpu.scf import BatchedDHFSCF, DHFSCF  # noqa: E402

TOL = 1e-11
TOL_DF = 1e-12


def _molecules():
    a = deck.make_basis([((0.0, 0.0, 0.0), {0: [0.3, 2.5], 1: [0.7]}),
                         ((0.3, -0.8, 1.3), {0: [0.45], 1: [1.1]}),
                         ((-1.0, 0.5, 0.4), {0: [0.9, 0.2]})], isym=0)
    b = deck.make_basis([((0.1, 0.2, -0.3), {0: [0.6], 1: [1.3], 2: [0.8]}),
                         ((1.2, 0.4, 0.9), {0: [0.35, 3.0]}),
                         ((-0.7, -1.1, 0.2), {0: [0.5], 1: [0.9], 3: [0.7]})], isym=0)
    c = deck.make_basis([((0.0, 0.0, 0.0), {0: [0.25, 1.9]}),
                         ((0.0, 1.4, 0.4), {0: [0.8], 1: [0.6]}),
                         ((1.0, -0.3, 0.2), {0: [1.2]})], isym=0)
    return [a, b, c]


def _single(basis, d, prec="fp64", racah1=True, screen=0.0):
    fb = berthagpu.FockBuilder(basis, racah1=racah1)
    fb.set_precision(prec)
    fb.set_screening(screen)
    gd, gx = fb.clmfast(d, 3)
    fb.close()
    return gd, gx


def _batched(bases, dens, prec="fp64", racah1=True, screen=0.0, padded=False):
    fbs = []
    for b in bases:
        fb = berthagpu.FockBuilder(b, racah1=racah1)
        fb.set_precision(prec)
        fb.set_screening(screen)
        fbs.append(fb)
    nd = [fb.ndim for fb in fbs]
    if padded:
        # every instance in a slot of N x N with ld = N + 3 and gaps between
        N = max(nd) + 3
        ld = [N] * len(bases)
        moff = [k * (N * N + 17) for k in range(len(bases))]
    else:
        ld = nd
        moff = np.concatenate([[0], np.cumsum([n * n for n in nd])[:-1]]).tolist()
    span = max(o + l * n for o, l, n in zip(moff, ld, nd))
    batch = berthagpu.FockBatch(fbs, moff=moff, ld=ld)
    for fb in fbs:
        fb.close()  # the batch holds its own copies
    D = torch.zeros(span, dtype=torch.complex128)
    for k, d in enumerate(dens):
        n = nd[k]
        for j in range(n):
            D[moff[k] + ld[k] * j: moff[k] + ld[k] * j + n] = torch.from_numpy(d[:, j].copy())
    Dd = D.cuda()
    J = torch.full((span,), 7.0 + 0j, dtype=torch.complex128, device="cuda")
    K = torch.full((span,), 7.0 + 0j, dtype=torch.complex128, device="cuda")
    batch.clmfast_device(Dd.data_ptr(), J.data_ptr(), K.data_ptr(), 3)
    torch.cuda.synchronize()
    Jh, Kh = J.cpu().numpy(), K.cpu().numpy()
    out = []
    for k in range(len(bases)):
        n = nd[k]
        idx = moff[k] + np.arange(n)[:, None] + ld[k] * np.arange(n)[None, :]
        out.append((Jh[idx], Kh[idx]))
    # elements outside every instance's block are left alone
    touched = np.zeros(span, bool)
    for k in range(len(bases)):
        n = nd[k]
        touched[moff[k] + np.arange(n)[:, None] + ld[k] * np.arange(n)[None, :]] = True
    assert np.all(Jh[~touched] == 7.0) and np.all(Kh[~touched] == 7.0)
    nq, nl = batch.quartets(), batch.launches()
    batch.close()
    return out, nq, nl


def _check(pairs, refs, tol):
    for (gd, gx), (rd, rx) in zip(pairs, refs):
        scale = max(np.abs(rd).max(), np.abs(rx).max())
        assert np.abs(gd - rd).max() <= tol * scale
        assert np.abs(gx - rx).max() <= tol * scale


@pytest.mark.parametrize("padded", [False, True])
def test_batch_matches_single_contexts(padded):
    bases = _molecules()
    dens = [deck.density(b, seed=11 + k) for k, b in enumerate(bases)]
    refs = [_single(b, d) for b, d in zip(bases, dens)]
    out, nq, nl = _batched(bases, dens, padded=padded)
    _check(out, refs, TOL)
    assert nq > 0
    # two zeroing kernels, one quartet launch per component class, two completions
    assert nl == 2 + 3 + 2


def test_batch_split_precision():
    bases = _molecules()
    dens = [deck.density(b, seed=21 + k) for k, b in enumerate(bases)]
    refs = [_single(b, d) for b, d in zip(bases, dens)]
    out, _, nl = _batched(bases, dens, prec="df32", padded=True)
    _check(out, refs, TOL_DF)
    assert nl == 2 + 1 + 3 + 2  # + the density's double-float copy


def test_batch_atoms_one_centre_screened():
    """Closed-shell atoms (ATOMIC shape, one-centre quartets by the MD route
    with CLMFAST's atomic selection rules), each with Schwarz screening."""
    zs = [2, 4, 2, 10]
    bases = [deck.atom_basis(z) for z in zs]
    dens = [deck.density(b, seed=31 + k, real=True) for k, b in enumerate(bases)]
    refs = [_single(b, d, racah1=False, screen=1e-12) for b, d in zip(bases, dens)]
    out, _, _ = _batched(bases, dens, racah1=False, screen=1e-12)
    _check(out, refs, TOL)


def test_batch_rejects_mixed_shapes():
    a = deck.make_basis([((0.0, 0.0, 0.0), {0: [0.5]}), ((0.0, 0.0, 1.4), {0: [0.5]})])
    b = deck.make_basis([((0.0, 0.0, 0.0), {0: [0.5]}), ((0.3, 0.0, 1.4), {0: [0.5]}),
                         ((1.0, 1.0, 0.0), {0: [0.4]})])
    fa, fb = berthagpu.FockBuilder(a), berthagpu.FockBuilder(b)
    with pytest.raises(berthagpu.BerthaGPUError):
        berthagpu.FockBatch([fa, fb])
    with pytest.raises(berthagpu.BerthaGPUError):
        berthagpu.FockBatch([fa], moff=[0], ld=[a.ndim - 1])  # ld below NDIM
    fa.close()
    fb.close()


def test_batch_graph_replay():
    """After its first call the batched build only launches kernels: one CUDA
    graph replays it with new densities."""
    bases = _molecules()[:2]
    fbs = [berthagpu.FockBuilder(b) for b in bases]
    nd = [fb.ndim for fb in fbs]
    batch = berthagpu.FockBatch(fbs)
    for fb in fbs:
        fb.close()
    span = sum(n * n for n in nd)
    D, J, K = (torch.zeros(span, dtype=torch.complex128, device="cuda") for _ in range(3))
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        batch.clmfast_device(D.data_ptr(), J.data_ptr(), K.data_ptr(), 3, s.cuda_stream)
    s.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=s):
        batch.clmfast_device(D.data_ptr(), J.data_ptr(), K.data_ptr(), 3,
                             torch.cuda.current_stream().cuda_stream)
    for seed in (3, 4):
        dens = [deck.density(b, seed=seed + k) for k, b in enumerate(bases)]
        D.copy_(torch.from_numpy(np.concatenate([d.ravel(order="F") for d in dens])))
        g.replay()
        torch.cuda.synchronize()
        Jh, Kh = J.cpu().numpy(), K.cpu().numpy()
        off = 0
        for b, d, n in zip(bases, dens, nd):
            rd, rx = _single(b, d)
            gd = Jh[off:off + n * n].reshape(n, n, order="F")
            gx = Kh[off:off + n * n].reshape(n, n, order="F")
            scale = max(np.abs(rd).max(), np.abs(rx).max())
            assert np.abs(gd - rd).max() <= TOL * scale
            assert np.abs(gx - rx).max() <= TOL * scale
            off += n * n
    batch.close()


def test_batched_scf_matches_single_scf():
    """Batched SCF of He, Be and He (padded to Be's NDIM) against one DHFSCF
    per atom: the same converged DHF energies."""
    zs = [2, 4, 2]
    bases = [deck.atom_basis(z) for z in zs]
    bs = BatchedDHFSCF(bases, zs, screen=1e-12)
    res = bs.run(etol=1e-10)
    bs.close()
    assert all(res["converged"])
    for z, b, e in zip(zs, bases, res["energy"]):
        s = DHFSCF(b, z, screen=1e-12)
        r = s.run(etol=1e-10)
        s.close()
        assert r["converged"]
        assert abs(r["energy"] - e) < 1e-8
    # the two helium instances agree with each other
    assert abs(res["energy"][0] - res["energy"][2]) < 1e-10
