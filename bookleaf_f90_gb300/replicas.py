"""Whole-job figures for independent replicas, one process per GPU.

The hydro step does not shard without a halo exchange (the reference's
typhon layer), so a multi-GPU run advances one independent replica of the
mesh per rank and exchanges nothing on the data path.  The only collective
is the end-of-run reduction here: the job's rate is the units all ranks
processed divided by the slowest rank's time.
"""


def job_rate(local_ms, local_units, device=None):
    """(rate per second, max time in ms, total units) over all ranks.

    Without an initialised process group (or with one rank) this is the
    local figure.  ``device`` is where the reduction tensors live: a CUDA
    device under NCCL, None (CPU) under gloo.
    """
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return local_units / (local_ms * 1e-3), float(local_ms), float(local_units)
    t = torch.tensor([float(local_ms)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    z = torch.tensor([float(local_units)], dtype=torch.float64, device=device)
    dist.all_reduce(z, op=dist.ReduceOp.SUM)
    t_max, total = float(t.item()), float(z.item())
    return total / (t_max * 1e-3), t_max, total


def max_over_ranks(value, device=None):
    """Largest value over all ranks (the local value without a group)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())
