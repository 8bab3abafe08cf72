"""Replicas across GPUs: the filter stage shards by whole images.

Images are independent, so N GPUs run N independent replicas of the stage
with no exchange on the data path: a request-level router assigns whole
images to ranks and the job's time is the slowest rank's. The only
collective is the host-side max of the per-rank times used for reporting.
"""


def shard(weights, rank, world):
    """Indices of the images that `rank` of `world` takes.

    Greedy longest-processing-time assignment on the given per-image weights
    (e.g. luma pixels): images in decreasing weight, each to the currently
    least-loaded rank (ties to the lower rank). Deterministic, so every rank
    computes the same assignment without communicating."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("bad rank/world")
    order = sorted(range(len(weights)), key=lambda i: (-weights[i], i))
    load = [0] * world
    mine = []
    for i in order:
        r = min(range(world), key=lambda k: (load[k], k))
        load[r] += weights[i]
        if r == rank:
            mine.append(i)
    return sorted(mine)


def max_over_ranks(value, device=None):
    """Max of a float over all ranks (torch.distributed; identity when not
    initialised)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()):
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_rate(units_per_rank, world, seconds_max):
    """Whole-job throughput: the units all ranks processed over the slowest
    rank's time (weak scaling: every rank processes the same per-rank work)."""
    return units_per_rank * world / seconds_max
