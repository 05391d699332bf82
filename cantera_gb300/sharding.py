"""Reactor sharding across GPUs: one process per GPU, contiguous shards, no data-path
collective.

Reactors are independent, so rank r of W integrates reactors [n*r//W, n*(r+1)//W) alone.  The
only cross-rank operations are a barrier around timed regions, the maximum of the step time over
ranks and, when a caller wants the whole batch on one rank, a gather of the results.
"""
import numpy as np


def shard_range(n, rank, world):
    """[lo, hi) of rank `rank` out of `world` for n reactors (sizes differ by at most one)."""
    if world < 1 or not (0 <= rank < world) or n < 0:
        raise ValueError("bad shard request: n=%d rank=%d world=%d" % (n, rank, world))
    return (n * rank) // world, (n * (rank + 1)) // world


def max_over_ranks(x, dist=None, device=None):
    """Maximum of a float over all ranks (x itself without a process group)."""
    if dist is None or not dist.is_initialized() or dist.get_world_size() == 1:
        return float(x)
    import torch
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def gather_shards(local, n, dist=None, axis=-1):
    """Concatenate every rank's shard (numpy, reactors along `axis`) in rank order."""
    if dist is None or not dist.is_initialized() or dist.get_world_size() == 1:
        return np.asarray(local)
    parts = [None] * dist.get_world_size()
    dist.all_gather_object(parts, np.asarray(local))
    out = np.concatenate(parts, axis=axis)
    if out.shape[axis] != n:
        raise RuntimeError("gathered %d reactors, expected %d" % (out.shape[axis], n))
    return out
