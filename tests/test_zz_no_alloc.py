"""The allocation-free split-precision entry point, through the C ABI.

bertha_gpu_quartets_noalloc serves callers that cannot call cudaMalloc
(for instance code inside an application whose memory pool already owns the
GPU's memory).  It keeps its scratch -- the double-float copy of the
density -- in a static device array.  This file checks, on a fresh context
whose first digestion is the allocation-free one, that repeated calls leave
the device's free memory unchanged, that two calls in a row agree with the
oracle's digestion of the same quartets and with the allocating entry point
bertha_gpu_quartets in the same precision, and that an oversized basis and
a too-small leading dimension are refused.  It is named so that pytest
collects it last.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

import berthagpu  # noqa: E402
from berthagpu import _lib, deck, workloads  # noqa: E402
from oracle import oracle as orc  # noqa: E402

# same bound as the split-precision parity tests
DF_TOL = 1e-10


def _pool(ncentres, lmax, nexp, seed):
    rng = np.random.default_rng(seed)
    cents = [(rng.uniform(0, 6, 3), {l: list(np.exp(rng.uniform(np.log(0.1), np.log(50.0), nexp)))
                                      for l in range(lmax + 1)}) for _ in range(ncentres)]
    return deck.make_basis(cents, hmlt="DHFR", isym=0)


def _call(fn, fb, dq, cls, D, n, ldf=None, out=None):
    """One digestion into zeroed outputs (out: preallocated (GD, GX) device
    buffers, so that the call itself is the only thing that could allocate)."""
    import torch
    if out is None:
        out = (torch.zeros(n, 2 * n, dtype=torch.float64, device="cuda"),
               torch.zeros(n, 2 * n, dtype=torch.float64, device="cuda"))
    GD, GX = out
    GD.zero_()
    GX.zero_()
    st = torch.cuda.current_stream().cuda_stream
    rc = fn(fb.ctx, ctypes.c_void_p(dq.data_ptr()), dq.shape[0], cls[0], cls[1],
            ctypes.c_void_p(D.data_ptr()), n, ctypes.c_void_p(GD.data_ptr()),
            ctypes.c_void_p(GX.data_ptr()), n if ldf is None else ldf, ctypes.c_void_p(st))
    _lib.check(rc, fb.ctx)
    torch.cuda.synchronize()
    return GD.cpu().numpy(), GX.cpu().numpy()


def _free_bytes():
    import torch
    torch.cuda.synchronize()
    return torch.cuda.mem_get_info()[0]


def test_noalloc_allocates_nothing_and_matches():
    import torch
    b = _pool(ncentres=8, lmax=2, nexp=2, seed=31)
    assert b.ndim <= 1024
    dent = deck.density(b, seed=4)
    quarts = workloads.microbench_quartets(b, 4000, seed=12)
    fb = berthagpu.FockBuilder(b)
    fb.set_precision("df32")  # the allocating entry point in the same precision
    n = fb.ndim
    D = torch.from_numpy(np.ascontiguousarray(dent.T).view(np.float64).reshape(n, 2 * n)).cuda()
    dqs = {cls: torch.from_numpy(q).cuda() for cls, q in quarts.items()}
    L = _lib.lib()
    # the context's first digestion is the allocation-free one; after one
    # warm-up call (module loading), further calls change no free memory
    out = (torch.zeros(n, 2 * n, dtype=torch.float64, device="cuda"),
           torch.zeros(n, 2 * n, dtype=torch.float64, device="cuda"))
    cls0 = next(iter(dqs))
    _call(L.bertha_gpu_quartets_noalloc, fb, dqs[cls0], cls0, D, n, out=out)
    before = _free_bytes()
    got = {}
    for cls, dq in dqs.items():
        got[cls] = [_call(L.bertha_gpu_quartets_noalloc, fb, dq, cls, D, n, out=out)
                    for _ in range(2)]
    assert _free_bytes() == before
    O = orc.QuartetOracle(b)
    for cls, q in quarts.items():
        rd = np.zeros((n, n), complex, order="F")
        rx = np.zeros((n, n), complex, order="F")
        O.prepare(q, *cls)
        O.digest(q, *cls, dent, rd, rx, nthreads=8)
        # the C ABI's column-major complex matrix as the [n, 2n] row buffer
        ref_o = (np.ascontiguousarray(rd.T).view(np.float64), np.ascontiguousarray(rx.T).view(np.float64))
        ref_a = _call(L.bertha_gpu_quartets, fb, dqs[cls], cls, D, n)
        scale = max(np.abs(ref_o[0]).max(), np.abs(ref_o[1]).max())
        for g in got[cls]:  # two calls in a row share the static scratch
            for k in range(2):
                assert np.abs(g[k] - ref_o[k]).max() <= DF_TOL * scale
                assert np.abs(g[k] - ref_a[k]).max() <= DF_TOL * scale
    O.close()
    fb.close()


def test_noalloc_refuses_oversized_basis():
    import torch
    b = _pool(ncentres=16, lmax=2, nexp=2, seed=5)
    assert b.ndim > 1024
    fb = berthagpu.FockBuilder(b)
    n = fb.ndim
    q = torch.zeros((1, 4), dtype=torch.int32, device="cuda")
    D = torch.zeros(n, 2 * n, dtype=torch.float64, device="cuda")
    with pytest.raises(berthagpu.BerthaGPUError) as ei:
        _call(_lib.lib().bertha_gpu_quartets_noalloc, fb, q, (0, 0), D, n)
    assert ei.value.code == _lib.BG_ERR_CAPACITY
    fb.close()


def test_explicit_lists_refuse_short_leading_dimension():
    """An output leading dimension below NDIM would let the kernels write
    past the caller's matrices: both explicit-list entry points refuse it."""
    import torch
    b = _pool(ncentres=2, lmax=1, nexp=1, seed=8)
    fb = berthagpu.FockBuilder(b)
    n = fb.ndim
    q = torch.zeros((1, 4), dtype=torch.int32, device="cuda")
    D = torch.zeros(n, 2 * n, dtype=torch.float64, device="cuda")
    L = _lib.lib()
    for fn in (L.bertha_gpu_quartets, L.bertha_gpu_quartets_noalloc):
        with pytest.raises(berthagpu.BerthaGPUError) as ei:
            _call(fn, fb, q, (0, 0), D, n, ldf=n - 1)
        assert ei.value.code == _lib.BG_ERR_ARG
    fb.close()
