"""Replica-parallel form of the projection path on several GPUs.

The path shards with no exchange step: (k, spin) blocks, defect bands and
requests are independent (pseudoprojector.c:73-88, projector.c:872-886), so
N ranks (one GPU each) each run independent work and results are concatenated
on the host. The only communication is for timing: a barrier around the timed
region and the max / sum of per-rank figures.
"""


def shard(n, rank, world):
    """Indices of n work items owned by rank (contiguous blocks, sizes differing by at most one)."""
    lo = n * rank // world
    hi = n * (rank + 1) // world
    return list(range(lo, hi))


def barrier(pg):
    if pg is not None:
        pg.barrier()


def max_over_ranks(pg, v):
    if pg is None:
        return v
    import torch

    t = torch.tensor([float(v)], dtype=torch.float64)
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(pg, v):
    if pg is None:
        return v
    import torch

    t = torch.tensor([float(v)], dtype=torch.float64)
    pg.all_reduce(t, op=pg.ReduceOp.SUM)
    return float(t.item())
