"""One independent system per process (the multi-GPU mode of this path is
replicas only: no data-path collective). Helpers used by bench.py under
torchrun: rank-dependent seeds and the max-over-ranks of a timing."""
import os


def rank_info():
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
            int(os.environ.get("LOCAL_RANK", "0")))


def replica_seed(base_seed, rank):
    """Each rank runs its own replica: a distinct, reproducible seed."""
    return int(base_seed) + 7919 * int(rank)


def max_over_ranks(value, device=None):
    """The slowest rank's time (all ranks must call). Returns value when the
    process group is not initialised."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()):
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device or "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(value, device=None):
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()):
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device or "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())
