"""Two-rank (gloo, CPU) check of the replica path used by bench.py --gpus N:
every rank digests the same seeded quartet list (weak scaling), the job step
time is the maximum over ranks and the throughput counts all ranks' work."""
import os
import socket

import numpy as np
import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, out):
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    for p in (root, os.path.join(root, "bertha-program_gb300")):
        sys.path.insert(0, p)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from berthagpu import deck, replicas, workloads
    from oracle import oracle as orc
    b = deck.make_basis([((0, 0, 0), {0: [0.5, 2.0], 1: [0.9]}),
                         ((0.3, 0.8, 1.2), {0: [0.7, 3.0], 1: [1.4]})], isym=0)
    q = workloads.microbench_quartets(b, 64, seed=3)
    O = orc.QuartetOracle(b)
    n = b.ndim
    gd = np.zeros((n, n), complex, order="F")
    gx = np.zeros((n, n), complex, order="F")
    dent = deck.density(b, seed=2)
    for cls, qq in q.items():
        O.digest(qq, *cls, dent, gd, gx)
    my_ms = 10.0 + 5.0 * rank
    job_ms = replicas.job_step_ms(my_ms, dist)
    t = torch.from_numpy(np.concatenate([gd.real.ravel(), gd.imag.ravel()]))
    other = [torch.zeros_like(t) for _ in range(world)]
    dist.all_gather(other, t)
    out[rank] = (job_ms, replicas.job_throughput(64, world, job_ms),
                 float(max((o - other[0]).abs().max() for o in other)))
    dist.destroy_process_group()


def test_two_rank_replicas():
    world = 2
    mgr = mp.get_context("spawn").Manager()  # no fork of a threaded process
    out = mgr.dict()
    mp.spawn(_worker, args=(world, _free_port(), out), nprocs=world, join=True)
    for r in range(world):
        job_ms, thr, spread = out[r]
        assert job_ms == 15.0                      # max over ranks
        assert abs(thr - 64 * 2 / 15e-3) < 1e-6    # all ranks' quartets
        assert spread == 0.0                       # identical replicas
