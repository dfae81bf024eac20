"""Host-side helpers for running the path as independent replicas.

The slice is the unit of work: a slice couples all of its pixels through the
objective band-pass, so work is sharded by slice (wavelength of a sweep,
request, scene) and never within one.  There is no collective in the data
path; ranks meet only for a barrier and the max-over-ranks timing.
"""
import os


def env():
    """(world_size, rank, local_rank) from the torchrun environment."""
    return (int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0")),
            int(os.environ.get("LOCAL_RANK", "0")))


def shard(items, rank, world):
    """Contiguous block of `items` owned by `rank` (sizes differ by at most one)."""
    n = len(items)
    base, extra = divmod(n, world)
    start = rank * base + min(rank, extra)
    return items[start:start + base + (1 if rank < extra else 0)]


def max_over_ranks(value, device=None):
    """Max of a float over all ranks of the default process group."""
    import torch
    import torch.distributed as dist
    if not dist.is_available() or not dist.is_initialized():
        return value
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())
