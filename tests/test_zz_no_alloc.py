"""The allocation-free split-precision entry point, through the C ABI.

bertha_gpu_quartets_noalloc serves callers that cannot call cudaMalloc
(for instance code inside an application whose memory pool already owns the
GPU's memory).  It keeps its scratch -- the double-float copy of the
density -- in a static device array.  This file checks it against the
allocating entry point bertha_gpu_quartets in the same precision, on two
calls in a row, and that an oversized basis is refused.  It is named so
that pytest collects it last.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

import berthagpu  # noqa: E402
from berthagpu import _lib, deck, workloads  # noqa: E402

# same bound as the split-precision parity tests
DF_TOL = 1e-10


def _pool(ncentres, lmax, nexp, seed):
    rng = np.random.default_rng(seed)
    cents = [(rng.uniform(0, 6, 3), {l: list(np.exp(rng.uniform(np.log(0.1), np.log(50.0), nexp)))
                                      for l in range(lmax + 1)}) for _ in range(ncentres)]
    return deck.make_basis(cents, hmlt="DHFR", isym=0)


def _call(fn, fb, dq, cls, D, n):
    import torch
    GD = torch.zeros(n, 2 * n, dtype=torch.float64, device="cuda")
    GX = torch.zeros_like(GD)
    st = torch.cuda.current_stream().cuda_stream
    rc = fn(fb.ctx, ctypes.c_void_p(dq.data_ptr()), dq.shape[0], cls[0], cls[1],
            ctypes.c_void_p(D.data_ptr()), n, ctypes.c_void_p(GD.data_ptr()),
            ctypes.c_void_p(GX.data_ptr()), n, ctypes.c_void_p(st))
    _lib.check(rc, fb.ctx)
    torch.cuda.synchronize()
    return GD.cpu().numpy(), GX.cpu().numpy()


def test_noalloc_matches_allocating_entry_point():
    import torch
    b = _pool(ncentres=8, lmax=2, nexp=2, seed=31)
    assert b.ndim <= 1024
    fb = berthagpu.FockBuilder(b)
    fb.set_precision("df32")
    n = fb.ndim
    dent = deck.density(b, seed=4)
    D = torch.from_numpy(np.ascontiguousarray(dent.T).view(np.float64).reshape(n, 2 * n)).cuda()
    quarts = workloads.microbench_quartets(b, 4000, seed=12)
    L = _lib.lib()
    for cls, q in quarts.items():
        dq = torch.from_numpy(q).cuda()
        ref = _call(L.bertha_gpu_quartets, fb, dq, cls, D, n)
        scale = max(np.abs(ref[0]).max(), np.abs(ref[1]).max())
        for _ in range(2):  # two calls in a row share the static scratch
            got = _call(L.bertha_gpu_quartets_noalloc, fb, dq, cls, D, n)
            assert np.abs(got[0] - ref[0]).max() <= DF_TOL * scale
            assert np.abs(got[1] - ref[1]).max() <= DF_TOL * scale
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
