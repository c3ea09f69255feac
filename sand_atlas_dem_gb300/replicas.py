"""Independent specimen replicas across ranks (one process per GPU).

The mesh-surface step of one specimen does not shard across GPUs: a rank
runs its own specimen(s) with no data-path collective.  After the timed
region the ranks exchange only their timings so that rank 0 can report the
whole-job throughput: grain-steps of all ranks over the slowest rank's time.
"""


def aggregate(grain_steps, seconds, *, device=None):
    """All-gather (grain_steps, seconds) and return the job totals on every rank.

    Works with any initialized ``torch.distributed`` backend (NCCL on GPUs,
    gloo on CPUs).  Returns dict(grain_steps, seconds=max over ranks,
    value=grain_steps/seconds, ranks).
    """
    import torch
    import torch.distributed as dist

    local = torch.tensor([float(grain_steps), float(seconds)], dtype=torch.float64, device=device)
    gathered = [torch.zeros_like(local) for _ in range(dist.get_world_size())]
    dist.all_gather(gathered, local)
    total = sum(float(g[0]) for g in gathered)
    slowest = max(float(g[1]) for g in gathered)
    return dict(grain_steps=total, seconds=slowest, value=total / slowest, ranks=len(gathered))
