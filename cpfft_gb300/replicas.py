"""Replicas across GPUs: one process per GPU, each solving its own RVEs, no collective on
the data path.

The finite-strain FFT solve of one RVE stays on one GPU (the stress update shards by
voxel with no exchange, but the FFT would need an all-to-all per transform direction,
which this library does not do).  Several GPUs therefore run independent RVEs (the
batched-RVE workload is partitioned by RVE) and only the timing summary crosses ranks.
"""
import torch


def partition(n_items, world, rank):
    """Contiguous block of item indices [lo, hi) for `rank`; sizes differ by at most one
    and the blocks cover 0..n_items-1 exactly once."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("rank outside [0, world)")
    base, extra = divmod(n_items, world)
    lo = rank * base + min(rank, extra)
    return lo, lo + base + (1 if rank < extra else 0)


def reduce_timings(t_device, t_e2e, units, device=None):
    """Whole-job figures of a replicated run: the slowest rank's device and end-to-end
    times and the units summed over ranks.  Single-process runs return the inputs."""
    if not (torch.distributed.is_available() and torch.distributed.is_initialized()):
        return t_device, t_e2e, units
    dist = torch.distributed
    t = torch.tensor([t_device, t_e2e], dtype=torch.float64, device=device)
    u = torch.tensor([units], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.all_reduce(u, op=dist.ReduceOp.SUM)
    return t[0].item(), t[1].item(), u[0].item()
