"""Host-side logic for running the fit on several GPUs, one process per GPU.

Every expression is an independent problem, so a batch shards with no exchange on
the data path: rank r fits a contiguous slice of the problems with the replicated X
and Y (weak scaling when every rank gets its own batch).  The only collectives are
the gather of the fitted constants and root values of one batch fitted in shards
(``fit_sharded``), the slowest rank's step time (the job's time), and, in a search
round, the best expression over all ranks, one (MSE, global index) pair per rank.
Everything here works with any torch.distributed backend (gloo on CPU, nccl on GPU).
"""
from __future__ import annotations

from typing import Callable, Optional, Tuple

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


def gather_rows(part: torch.Tensor, total: int) -> torch.Tensor:
    """Every rank's contiguous share of the rows of a (total, ...) result, gathered on
    every rank in batch order (rank r holds rows shard_range(total, r, world)).  The
    shares may differ by one row: each is padded to the largest before the all_gather
    and trimmed after."""
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return part
    world = dist.get_world_size()
    spans = [shard_range(total, r, world) for r in range(world)]
    rows = max(b - a for a, b in spans)
    pad = torch.zeros((rows,) + tuple(part.shape[1:]), dtype=part.dtype, device=part.device)
    pad[: part.shape[0]] = part
    out = [torch.empty_like(pad) for _ in range(world)]
    dist.all_gather(out, pad)
    return torch.cat([o[: b - a] for o, (a, b) in zip(out, spans)], dim=0)


def fit_shard(X, Y, Ops, Ch, C_init, start: int, stop: int, fit: Optional[Callable] = None,
              **kw) -> Tuple[torch.Tensor, torch.Tensor]:
    """(C_final, Y_final) of problems [start, stop) of the batch, fitted alone.  Y is one
    row per problem (B, N) or a row that serves every problem.  fit(X, Y, Ops, Ch,
    C_init, **kw) -> (C_final, Y_final) is any fit whose result for a problem does not
    depend on the rest of the batch.  By default it is this package's optimize, run with
    the whole batch's launch shape and constant-slot layout (batch_launch_shape), which
    fix the order of its sums: each problem then gets the bits the whole fit gives it."""
    B = Ops.shape[0]
    Ys = Y[start:stop] if (Y is not None and Y.dim() == 2 and Y.shape[0] == B and B > 1) else Y
    if fit is None:
        from .optimization import batch_launch_shape, optimize_ex
        pin = batch_launch_shape(X, Ops, Ch)
        r = optimize_ex(X, Ys, Ops[start:stop], Ch[start:stop], C_init[start:stop], **kw, **pin)
        return r.C, r.Y
    return fit(X, Ys, Ops[start:stop], Ch[start:stop], C_init[start:stop], **kw)


def fit_sharded(X, Y, Ops, Ch, C_init, fit: Optional[Callable] = None, **kw) -> Tuple[torch.Tensor, torch.Tensor]:
    """``optimize`` of one batch on every rank of the process group: rank r fits the
    contiguous share shard_range(B, r, world) of the problems (fit_shard) with X (and a
    target row that serves every problem) replicated, then C_final (B, M) and Y_final
    (B, N) are gathered on every rank in batch order.  The problems are independent and
    every shard is fitted with the whole batch's launch shape, so the result equals the
    unsharded fit's bit for bit.  A fit that raises on any rank raises on every rank
    (the others learn of it in an all_gather of the error, before the gather of the
    results, so no rank waits for a share that will not come).  fit(X, Y, Ops, Ch,
    C_init, **kw) -> (C_final, Y_final) defaults to this package's ``optimize``.
    Without an initialised process group it is one plain fit."""
    import torch.distributed as dist
    B = Ops.shape[0]
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        if fit is None:
            from .optimization import optimize as fit
        return fit(X, Y, Ops, Ch, C_init, **kw)
    rank, world = dist.get_rank(), dist.get_world_size()
    start, stop = shard_range(B, rank, world)
    failure = None
    try:
        C_part, Y_part = fit_shard(X, Y, Ops, Ch, C_init, start, stop, fit=fit, **kw)
    except Exception as e:  # reported to every rank below, then raised here
        failure = e
    errors = [None] * world
    dist.all_gather_object(errors, None if failure is None else f"{type(failure).__name__}: {failure}")
    if failure is not None:
        raise failure
    failed = [(r, e) for r, e in enumerate(errors) if e is not None]
    if failed:
        raise RuntimeError(f"the fit failed on rank {failed[0][0]}: {failed[0][1]}")
    return gather_rows(C_part, B), gather_rows(Y_part, B)
