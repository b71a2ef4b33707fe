"""Whole-job figures for multi-GPU runs, one process per GPU.

The hydro step of one mesh does not shard without a halo exchange (the
reference's typhon layer), so a multi-GPU run of one mesh advances an
independent replica per rank.  A batch of independent meshes does shard:
each rank takes its share of the meshes (``shard``) and runs them alone.
Neither exchanges anything on the data path.  The only collectives are
the end-of-run reductions here: the job's rate is the units all ranks
processed divided by the slowest rank's time.
"""


def shard(weights, world, rank):
    """The indices of the items rank ``rank`` of ``world`` takes: the
    longest-processing-time rule (items by decreasing weight, each to the
    rank with the least weight so far, the lowest rank on ties), so that
    the ranks' loads differ by at most the largest item.  Deterministic:
    every rank computes the same assignment without communicating.  Each
    rank's indices come back in increasing order."""
    if world <= 1:
        return list(range(len(weights)))
    load = [0.0] * world
    owner = [0] * len(weights)
    for i in sorted(range(len(weights)), key=lambda i: (-float(weights[i]), i)):
        r = min(range(world), key=lambda r: (load[r], r))
        owner[i] = r
        load[r] += float(weights[i])
    return [i for i in range(len(weights)) if owner[i] == rank]


def gather_to_root(obj):
    """[every rank's obj] on rank 0 (None elsewhere); [obj] without a
    group."""
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return [obj]
    out = [None] * dist.get_world_size() if dist.get_rank() == 0 else None
    dist.gather_object(obj, out, dst=0)
    return out


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
