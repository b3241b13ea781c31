"""Replica bookkeeping for multi-GPU runs (one process per GPU).

The Fock build does not shard across GPUs here (each configuration fits one
GPU), so N ranks run N independent replicas of the same seeded workload.
The step time of the job is the slowest rank's; the throughput is the work
of all ranks over that time.
"""
import os


def rank_info():
    return (int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)),
            int(os.environ.get("LOCAL_RANK", 0)))


def job_step_ms(ms, dist=None, device=None):
    """Max over ranks of a per-rank step time (ms)."""
    import torch
    t = torch.tensor([float(ms)], dtype=torch.float64, device=device)
    if dist is not None and dist.is_available() and dist.is_initialized():
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_throughput(units_per_rank, world, step_ms):
    """Whole-job units per second: all ranks' units over the slowest step."""
    return units_per_rank * world / (step_ms * 1e-3)
