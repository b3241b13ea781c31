"""The device entry points are stream-ordered and allocate nothing after
their first call on a context, so an SCF iteration's Fock build can be
captured once as a CUDA graph and replayed with new density contents."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

import torch  # noqa: E402

import berthagpu  # noqa: E402
from berthagpu import deck  # noqa: E402
from oracle import oracle as orc  # noqa: E402


@pytest.mark.parametrize("prec", ["fp64", "df32"])
def test_fock_build_graph_replay(prec):
    b = deck.make_basis([((0.0, 0.0, 0.0), {0: [0.3, 2.5], 1: [0.7]}),
                         ((0.3, -0.8, 1.3), {0: [0.45], 1: [1.1]}),
                         ((-1.0, 0.5, 0.4), {0: [0.9]})], hmlt="DHFB")
    n = b.ndim
    fb = berthagpu.FockBuilder(b)
    fb.set_precision(prec)
    fb.set_screening(1e-12)
    D = torch.zeros((n, n), dtype=torch.complex128, device="cuda")
    J, K, B = (torch.zeros_like(D) for _ in range(3))
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        # first calls build the quartet lists, bounds and scratch
        fb.clmfast_device(D.data_ptr(), J.data_ptr(), K.data_ptr(), 3, n, s.cuda_stream)
        fb.brtfast_device(D.data_ptr(), B.data_ptr(), 3, n, s.cuda_stream)
    s.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=s):
        st = torch.cuda.current_stream().cuda_stream
        fb.clmfast_device(D.data_ptr(), J.data_ptr(), K.data_ptr(), 3, n, st)
        fb.brtfast_device(D.data_ptr(), B.data_ptr(), 3, n, st)
    for seed in (1, 2):
        d = deck.density(b, seed=seed)
        D.copy_(torch.from_numpy(np.ascontiguousarray(d.T)))  # column-major contents
        g.replay()
        torch.cuda.synchronize()
        rd, rx = orc.clmfast(b, d, 3)
        rb = orc.brtfast(b, d, 3)
        scale = max(np.abs(rd).max(), np.abs(rx).max())
        assert np.abs(J.cpu().numpy().T - rd).max() <= 1e-9 * scale
        assert np.abs(K.cpu().numpy().T - rx).max() <= 1e-9 * scale
        assert np.abs(B.cpu().numpy().T - rb).max() <= 1e-9 * np.abs(rb).max()
    fb.close()
