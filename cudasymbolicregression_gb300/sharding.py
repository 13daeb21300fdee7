"""Host-side logic for running the fit on several GPUs, one process per GPU.

Every expression is an independent problem, so a batch shards with no exchange on
the data path: rank r fits a contiguous slice of the problems with the replicated X
and Y (weak scaling when every rank gets its own batch).  The only collectives are
bookkeeping: the slowest rank's step time (the job's time), and, in a search round,
the best expression over all ranks, one (MSE, global index) pair per rank.
Everything here works with any torch.distributed backend (gloo on CPU, nccl on GPU).
"""
from __future__ import annotations

from typing import Tuple

import torch


def shard_range(total: int, rank: int, world: int) -> Tuple[int, int]:
    """[start, stop) of rank's contiguous share of `total` problems; the first
    total % world ranks get one more."""
    if world < 1 or not 0 <= rank < world or total < 0:
        raise ValueError(f"bad shard request: total={total} rank={rank} world={world}")
    base, extra = divmod(total, world)
    start = rank * base + min(rank, extra)
    return start, start + base + (1 if rank < extra else 0)


def max_over_ranks(value: float, device=None) -> float:
    """The largest value over all ranks (the job's step time); the value itself
    without an initialised process group."""
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def best_over_ranks(loss: torch.Tensor, offset: int, device=None) -> Tuple[float, int]:
    """(smallest finite loss, its global problem index) over all ranks; rank r's
    losses belong to problems offset .. offset + len - 1.  Ties go to the smaller
    index; (inf, -1) when no rank has a finite loss."""
    import torch.distributed as dist
    finite = torch.isfinite(loss)
    if finite.any():
        masked = torch.where(finite, loss.double(), torch.full_like(loss, float("inf"), dtype=torch.float64))
        i = int(torch.argmin(masked))
        best = (float(masked[i]), offset + i)
    else:
        best = (float("inf"), -1)
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return best
    world = dist.get_world_size()
    mine = torch.tensor([best[0], float(best[1])], dtype=torch.float64, device=device)
    out = [torch.zeros(2, dtype=torch.float64, device=device) for _ in range(world)]
    dist.all_gather(out, mine)
    cands = [(float(o[0]), int(o[1])) for o in out]
    cands = [c for c in cands if c[1] >= 0]
    if not cands:
        return float("inf"), -1
    return min(cands, key=lambda c: (c[0], c[1]))
