"""Runs on several GPUs of one node, one process per GPU.

The single-scene step has no data-parallel split without a halo exchange, so several GPUs
run independent replicas; batched scenes are independent units and are spread over the
ranks by particle count.  Neither needs a device collective: the ranks only agree on
timings and totals on the host side (any torch.distributed backend: NCCL on GPUs, gloo in
the CPU tests).
"""


def partition_scenes(counts, world):
    """Assigns scenes to ranks, largest first, each to the rank with the fewest particles so
    far (ties to the lower rank): a deterministic balance of the per-rank particle totals.
    Returns one ascending list of scene indices per rank."""
    if world < 1:
        raise ValueError("world must be >= 1")
    load = [0] * world
    parts = [[] for _ in range(world)]
    for s in sorted(range(len(counts)), key=lambda i: (-counts[i], i)):
        r = min(range(world), key=lambda k: (load[k], k))
        parts[r].append(s)
        load[r] += counts[s]
    return [sorted(p) for p in parts]


def aggregate(seconds, units, device=None):
    """(max of seconds over ranks, sum of units over ranks).  Without an initialised process
    group it returns the local values."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(seconds), float(units)
    t = torch.tensor([float(seconds)], dtype=torch.float64, device=device)
    u = torch.tensor([float(units)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.all_reduce(u, op=dist.ReduceOp.SUM)
    return float(t.item()), float(u.item())
