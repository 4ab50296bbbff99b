"""Multi-GPU runs of the time step are replicas: a lattice does not shard without a halo exchange,
and the batched-body workloads have no coupling at all, so each rank simulates its own scene and
no collective touches the data path.  The only communication is the aggregation of the timing:
whole-job throughput = all ranks' units / the slowest rank's time.  Works with any initialised
torch.distributed backend (nccl on GPUs, gloo in the CPU tests)."""
from __future__ import annotations


def aggregate_rate(local_units: float, local_seconds: float) -> tuple[float, float, float]:
    """Returns (units/s over all ranks, total units, max seconds over ranks)."""
    import torch
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return local_units / local_seconds, float(local_units), float(local_seconds)
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    secs = torch.tensor([float(local_seconds)], dtype=torch.float64, device=dev)
    units = torch.tensor([float(local_units)], dtype=torch.float64, device=dev)
    dist.all_reduce(secs, op=dist.ReduceOp.MAX)
    dist.all_reduce(units, op=dist.ReduceOp.SUM)
    s, u = float(secs.item()), float(units.item())
    return u / s, u, s


def barrier() -> None:
    import torch.distributed as dist

    if dist.is_available() and dist.is_initialized() and dist.get_world_size() > 1:
        dist.barrier()
