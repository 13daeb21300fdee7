"""Multi-process host logic (world_size 2, gloo on CPU): sharding, the job's time as
the slowest rank's, and the best expression over all ranks."""
import os
import socket

import pytest
import torch
import torch.multiprocessing as mp

from cudasymbolicregression_gb300 import sharding


def test_shard_range_partitions_exactly():
    for total in (0, 1, 7, 16384, 16385):
        for world in (1, 2, 3, 8):
            spans = [sharding.shard_range(total, r, world) for r in range(world)]
            assert spans[0][0] == 0 and spans[-1][1] == total
            for (a, b), (c, d) in zip(spans, spans[1:]):
                assert b == c and b >= a
            sizes = [b - a for a, b in spans]
            assert max(sizes) - min(sizes) <= 1
    with pytest.raises(ValueError):
        sharding.shard_range(10, 2, 2)


def test_single_process_fallbacks():
    assert sharding.max_over_ranks(3.5) == 3.5
    loss = torch.tensor([float("nan"), 2.0, 0.5, float("inf")])
    assert sharding.best_over_ranks(loss, offset=10) == (0.5, 12)
    assert sharding.best_over_ranks(torch.tensor([float("nan")]), offset=0) == (float("inf"), -1)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, results):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        total = 1001
        start, stop = sharding.shard_range(total, rank, world)
        # every rank fits its slice; the losses are a known function of the global index
        idx = torch.arange(start, stop, dtype=torch.float64)
        loss = (idx - 637.0).abs() + 0.25
        loss[::7] = float("nan")  # some problems end NaN
        t = sharding.max_over_ranks(0.1 * (rank + 1))
        best = sharding.best_over_ranks(loss.float(), offset=start)
        none = sharding.best_over_ranks(torch.full((3,), float("nan")), offset=start)
        results[rank] = (start, stop, t, best, none)
    finally:
        dist.destroy_process_group()


def test_two_ranks_gloo():
    ctx = mp.get_context("spawn")
    manager = ctx.Manager()
    results = manager.dict()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, results)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    r0, r1 = results[0], results[1]
    assert r0[0] == 0 and r0[1] == r1[0] and r1[1] == 1001
    assert r0[2] == pytest.approx(0.2) and r1[2] == pytest.approx(0.2)  # the slowest rank's time on both
    assert r0[3] == r1[3] == (pytest.approx(0.25), 637)               # the global minimum and its index
    assert r0[4] == r1[4] == (float("inf"), -1)


def _oracle_fit(X, Y, Ops, Ch, C_init, max_iter=30):
    """The oracle's optimize (the reference's float32 arithmetic) as a fit function."""
    import numpy as np
    import oracle
    o = oracle.optimize(X.numpy(), None if Y is None else Y.numpy(), Ops.numpy(), Ch.numpy(), C_init.numpy(),
                        max_iter=max_iter, dot_mode=0)
    return torch.from_numpy(np.ascontiguousarray(o["C"])), torch.from_numpy(np.ascontiguousarray(o["Y"]))


def _fit_batch():
    import numpy as np
    from cudasymbolicregression_gb300 import tapes
    rng = np.random.default_rng(5)
    B, M, N = 37, 16, 24
    X = rng.uniform(-2, 2, (N, 2)).astype(np.float32)
    C = rng.standard_normal((B, M)).astype(np.float32)
    tb = tapes.generate(B, M, seed=6, lengths=rng.integers(3, M + 1, size=B), const_counts=rng.integers(0, 4, size=B),
                        n_vars=2, X_screen=X, C_screen=C)
    Y = (np.sin(X[:, 0]) + 0.5 * X[:, 1]).astype(np.float32)[None, :].repeat(B, 0)
    return tuple(torch.from_numpy(a) for a in (X, Y, tb.ops, tb.ch, C))


def _fit_worker(rank, world, port, results):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        X, Y, O, Ch, C = _fit_batch()
        Cf, Yf = sharding.fit_sharded(X, Y, O, Ch, C, fit=_oracle_fit)
        start, stop = sharding.shard_range(O.shape[0], rank, world)
        results[rank] = (Cf.numpy(), Yf.numpy(), (start, stop))
    finally:
        dist.destroy_process_group()


def test_sharded_fit_equals_the_whole_batch_fit():
    """fit_sharded on two gloo ranks (37 problems: shares of 19 and 18): each rank fits
    its share with the oracle's optimize, and the gathered C_final and Y_final equal the
    fit of the whole batch bit for bit, in batch order, on both ranks."""
    import numpy as np
    ctx = mp.get_context("spawn")
    manager = ctx.Manager()
    results = manager.dict()
    port = _free_port()
    procs = [ctx.Process(target=_fit_worker, args=(r, 2, port, results)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=180)
        assert p.exitcode == 0
    X, Y, O, Ch, C = _fit_batch()
    Cw, Yw = _oracle_fit(X, Y, O, Ch, C)
    for r in (0, 1):
        Cf, Yf, span = results[r]
        assert Cf.shape == tuple(Cw.shape) and Yf.shape == tuple(Yw.shape)
        np.testing.assert_array_equal(np.nan_to_num(Cf, nan=7.0), np.nan_to_num(Cw.numpy(), nan=7.0))
        np.testing.assert_array_equal(np.nan_to_num(Yf, nan=7.0), np.nan_to_num(Yw.numpy(), nan=7.0))
    assert results[0][2] == (0, 19) and results[1][2] == (19, 37)
    # without a process group it is one plain fit
    Cs, Ys = sharding.fit_sharded(X, Y, O, Ch, C, fit=_oracle_fit)
    assert torch.equal(torch.nan_to_num(Cs, nan=7.0), torch.nan_to_num(Cw, nan=7.0))


def _failing_fit(X, Y, Ops, Ch, C_init):
    """A fit that raises on the second rank's share (18 problems) only."""
    if Ops.shape[0] == 18:
        raise RuntimeError("Error during symbolic evaluation backward pass: planted on this share")
    return _oracle_fit(X, Y, Ops, Ch, C_init, max_iter=2)


def _failing_worker(rank, world, port, results):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        X, Y, O, Ch, C = _fit_batch()
        try:
            sharding.fit_sharded(X, Y, O, Ch, C, fit=_failing_fit)
            results[rank] = "returned"
        except RuntimeError as e:
            results[rank] = str(e)
    finally:
        dist.destroy_process_group()


def test_sharded_fit_raises_on_every_rank_when_one_share_fails():
    """A share whose fit raises (the failure made on the host, in the fit function)
    makes fit_sharded raise on every rank, the failing rank with its own exception and
    the other with the failing rank's message, instead of leaving it waiting in the
    gather for a share that never comes."""
    ctx = mp.get_context("spawn")
    manager = ctx.Manager()
    results = manager.dict()
    port = _free_port()
    procs = [ctx.Process(target=_failing_worker, args=(r, 2, port, results)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=180)
        assert p.exitcode == 0
    assert results[1] == "Error during symbolic evaluation backward pass: planted on this share"
    assert results[0].startswith("the fit failed on rank 1: RuntimeError: Error during symbolic evaluation")


def test_fit_shard_slices_per_problem_targets_only():
    """fit_shard hands the fit the shard's rows of Ops, Ch, C_init and of a per-problem
    Y (B, N); a target row that serves every problem ((N,) or (1, N)) goes unchanged."""
    seen = []

    def fit(X, Y, Ops, Ch, C_init, **kw):
        seen.append((tuple(Y.shape), tuple(Ops.shape), tuple(Ch.shape), tuple(C_init.shape), kw))
        return C_init.clone(), torch.zeros(Ops.shape[0], X.shape[0])
    B, M, N = 10, 6, 4
    X = torch.zeros(N, 1)
    Ops, Ch, C = torch.zeros(B, M, dtype=torch.int64), torch.zeros(B, M, 2, dtype=torch.int64), torch.randn(B, M)
    for Y, want in ((torch.randn(B, N), (3, N)), (torch.randn(1, N), (1, N)), (torch.randn(N), (N,))):
        Cp, Yp = sharding.fit_shard(X, Y, Ops, Ch, C, 4, 7, fit=fit, max_iter=5)
        assert seen[-1] == (want, (3, M), (3, M, 2), (3, M), {"max_iter": 5})
        assert torch.equal(Cp, C[4:7]) and tuple(Yp.shape) == (3, N)
