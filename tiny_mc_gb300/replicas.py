"""Replicas: the photon walk sharded over ranks (one GPU each).

Photons are independent and their random streams are keyed by photon id, so
rank r walks a contiguous photon-id range and nothing is exchanged until the
end, where the ranks' exact 128-bit tallies are summed.  Integer sums make the
result bit-identical to one GPU walking the whole range.  The only collective
is one all-gather of 2 x shells 128-bit integers (<= 32 KB for 1001 shells).
"""
from __future__ import annotations

import numpy as np

from . import TALLY_DTYPE


def shard(n_photons: int, world: int, rank: int, base: int = 0):
    """(photon_id_base, count) of `rank`'s share of ids base .. base+n-1."""
    if not (0 <= rank < world):
        raise ValueError("rank out of range")
    per, extra = divmod(n_photons, world)
    start = base + rank * per + min(rank, extra)
    return start, per + (1 if rank < extra else 0)


def add128(a: np.ndarray, b: np.ndarray) -> np.ndarray:
    """a + b for TALLY_DTYPE arrays (128-bit sums in 64-bit halves)."""
    out = np.zeros(a.shape, TALLY_DTYPE)
    with np.errstate(over="ignore"):
        for lo, hi in (("w_lo", "w_hi"), ("w2_lo", "w2_hi")):
            s = a[lo] + b[lo]
            carry = (s < a[lo]).astype(np.uint64)
            out[lo] = s
            out[hi] = a[hi] + b[hi] + carry
    return out


def reduce_tallies(local: np.ndarray, group=None) -> np.ndarray:
    """Sum every rank's tally (TALLY_DTYPE [shells]) exactly; all ranks get it."""
    import torch
    import torch.distributed as dist
    t = torch.from_numpy(np.ascontiguousarray(local).view(np.int64).copy())
    world = dist.get_world_size(group)
    parts = [torch.empty_like(t) for _ in range(world)]
    dist.all_gather(parts, t, group=group)
    total = np.zeros(local.shape, TALLY_DTYPE)
    for p in parts:   # rank order: the sum is exact, so the order only fixes the work
        total = add128(total, p.numpy().view(TALLY_DTYPE).reshape(local.shape))
    return total
