"""Replica accounting for runs on several GPUs (one process per GPU).

Transfer instances (wavelengths, polarisations, rays, requests) are
independent and the layers of one instance are strictly sequential, so N GPUs
run N independent replicas of a workload: no field data crosses ranks.  The
only cross-rank step is the timing reduction here -- the job takes as long as
its slowest rank, and its throughput is the units all ranks processed over
that time (weak scaling: the work per rank is fixed as N grows).
"""
from __future__ import annotations


def job_time_ms(ms, dist=None, device=None):
    """The job's time: the maximum over ranks of each rank's ``ms``.

    ``dist`` is ``torch.distributed`` with an initialised process group (NCCL
    with a CUDA ``device``, or gloo on the CPU), or None for one process.
    """
    if dist is None:
        return float(ms)
    import torch

    t = torch.tensor([float(ms)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_throughput(units_per_rank, ms, world):
    """Units per second of the whole job: every rank's units over the job's time."""
    if ms <= 0:
        raise ValueError("job time must be positive")
    return float(units_per_rank) * int(world) / (float(ms) / 1e3)


__all__ = ["job_time_ms", "job_throughput"]
