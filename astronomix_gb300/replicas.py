"""Whole-job throughput of independent replicas (one simulation per GPU).

A single FV or FD step does not shard without a halo exchange, so N GPUs run
N independent simulations.  The job's throughput is the sum of the units
every rank processed divided by the slowest rank's time; the only collective
is this one reduction, outside the timed region.
"""


def replica_throughput(units_local: float, seconds_local: float) -> float:
    """sum(units) / max(seconds) over the ranks of the default process group
    (the local ratio when no group is initialised)."""
    import torch
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return units_local / seconds_local
    device = "cuda" if dist.get_backend() == "nccl" else "cpu"
    units = torch.tensor([float(units_local)], dtype=torch.float64, device=device)
    secs = torch.tensor([float(seconds_local)], dtype=torch.float64, device=device)
    dist.all_reduce(units, op=dist.ReduceOp.SUM)
    dist.all_reduce(secs, op=dist.ReduceOp.MAX)
    return float(units.item()) / float(secs.item())
