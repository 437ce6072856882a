"""Multi-GPU as independent replicas.

The XC build does not shard: every rank builds its own molecules on its own
GPU and no data moves between ranks.  The only collective is the timing
barrier and the max-over-ranks of the elapsed time, so the whole-job rate is
(builds on all ranks) / (slowest rank's time).
"""


def aggregate_rate(local_builds, local_seconds, dist=None):
    """Whole-job builds/s across ranks: total builds / max elapsed seconds.
    With dist = torch.distributed (initialised) the reduction runs over the
    process group; without it this rank's numbers are returned."""
    if dist is None or not dist.is_available() or not dist.is_initialized():
        return local_builds / local_seconds, local_seconds, local_builds
    import torch
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([local_seconds], dtype=torch.float64, device=dev)
    n = torch.tensor([float(local_builds)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.all_reduce(n, op=dist.ReduceOp.SUM)
    return float(n.item()) / float(t.item()), float(t.item()), int(n.item())
