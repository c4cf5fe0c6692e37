"""Sharding a particle set across ranks (one process per GPU).

Particles are independent, so ranks share nothing on the data path: each
holds the mesh and field records and a contiguous slice of the particles,
split as the reference's parallel solver splits them
(cylag/core/solver_parallel.pyx:126-138: n // size per rank, the remainder
to the last).  With per-particle PCG32 streams keyed by the global index
(pcg32_seed(seed, tag)) the results do not depend on the split.  The only
collective is the sum of the open-boundary exit counts (and a gather of
results when one rank wants them).
"""
from __future__ import annotations

import numpy as np


def split(n: int, world: int):
    """(start, count) of every rank's slice."""
    nper = n // world
    counts = [nper] * world
    counts[-1] += n % world
    return [(r * nper, counts[r]) for r in range(world)]


def shard_slice(n: int, rank: int, world: int) -> slice:
    start, count = split(n, world)[rank]
    return slice(start, start + count)


def allreduce_sum(values, dist):
    """Element-wise sum over ranks of an integer array (boundary counts)."""
    import torch
    t = torch.as_tensor(np.asarray(values, dtype=np.int64))
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return t.numpy()


def allreduce_max(value: float, dist) -> float:
    """Maximum over ranks (e.g. of a timed region, so that the slowest rank
    sets the job's time)."""
    import torch
    t = torch.tensor([float(value)], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def gather_rows(a, dist, rank, world):
    """Concatenation of every rank's rows on rank 0 (None elsewhere), in rank
    order; rows may differ in count."""
    import torch
    a = np.ascontiguousarray(a)
    n = torch.tensor([a.shape[0]], dtype=torch.int64)
    sizes = [torch.zeros(1, dtype=torch.int64) for _ in range(world)]
    dist.all_gather(sizes, n)
    rows = max(int(s.item()) for s in sizes)
    buf = np.zeros((rows,) + a.shape[1:], dtype=a.dtype)
    buf[:a.shape[0]] = a
    parts = [torch.zeros_like(torch.as_tensor(buf)) for _ in range(world)]
    dist.all_gather(parts, torch.as_tensor(buf))
    if rank != 0:
        return None
    return np.concatenate([p.numpy()[:int(s.item())] for p, s in zip(parts, sizes)])
