"""Several GPUs: independent replicas, no exchange on the data path.

Render pairs are independent (a pair's triangles depend only on its model, mesh
part, lights and camera), so a multi-GPU run is N replicas, each rendering its
own scene on its own GPU. Ranks meet only after the timed region, to combine
the timing (the slowest rank's time) and the totals (the sum over ranks).
shard_models() splits one scene's models over ranks for callers that want
each GPU to draw part of one frame instead of a replica.
"""
import numpy as np


def shard_models(num_models, rank, world):
    """Contiguous block of model indices for `rank` (blocks differ in size by at most one)."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError(f"rank {rank} outside world {world}")
    base, extra = divmod(num_models, world)
    lo = rank * base + min(rank, extra)
    hi = lo + base + (1 if rank < extra else 0)
    return np.arange(lo, hi, dtype=np.int64)


def combine(ms, units, alg_bytes, dist=None, device="cpu"):
    """(max ms over ranks, sum of units, sum of algorithmic bytes). With dist=None: this rank's values."""
    if dist is None:
        return float(ms), float(units), float(alg_bytes)
    import torch
    t = torch.tensor([float(ms), float(units), float(alg_bytes)], dtype=torch.float64, device=device)
    mx = t.clone()
    dist.all_reduce(mx, op=dist.ReduceOp.MAX)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(mx[0]), float(t[1]), float(t[2])
