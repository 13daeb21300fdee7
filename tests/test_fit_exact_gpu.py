"""Exact parity of the fused L-BFGS fit against the oracle in the kernel's arithmetic.

The oracle's dot_mode 2 runs the reference's control flow (lbfgs_batch.py:61-326,
optimization.py:72-99, restated in oracle/sr_oracle.c and pinned against the
reference's own fits by tests/test_oracle_golden.py) with the fused kernel's
arithmetic: its per-lane point sums, lane and warp reduction order for a launch
shape, float-pair dots, its direction (the compact representation for histories of
at most 32 pairs, the two-loop recursion for longer ones), and slot vectors.  On tapes whose
operators are IEEE-exact (+ - * /, square, neg) the kernel and this oracle must give
the same bits for every problem: constants, root values, loss, iterations and
closure counts, at 200 iterations, for every launch shape.  A state-machine
difference on a single problem fails these tests.

sin, cos, exp and log are the library's own functions (csrc/sr_fmath.h), which the
oracle compiles from the same source, so fits over tapes with them are bit-identical
too (the reference's fixtures and the ragged workload).  Only CUDA's other
transcendental functions (tan, asin, ..., pow) are not reproduced on the host.
"""
import numpy as np
import pytest
import torch

import oracle
from parity import first_divergence, fit_bits_differ, oracle_fit_like

pytestmark = pytest.mark.gpu

# launch shapes (points per lane V, warps per problem W)
SHAPES = [(1, 1), (1, 2), (1, 4), (1, 8), (2, 1), (2, 2), (2, 4), (4, 1), (4, 2)]


def _sr():
    import cudasymbolicregression_gb300 as sr
    return sr


def cuda(a):
    return torch.as_tensor(np.ascontiguousarray(a)).cuda()


def exact_batch(B, M, N, n_vars=2, seed=0, max_consts=8, min_len=1, noise=0.01):
    """Tapes over the IEEE-exact operators, lengths min_len..M (length 1: a leaf root),
    0..max_consts constants, and noisy targets from hidden tapes of the same kind."""
    from cudasymbolicregression_gb300 import tapes
    from cudasymbolicregression_gb300.operators import Operator as Op
    exact_bin = (int(Op.ADD), int(Op.SUB), int(Op.MUL), int(Op.DIV))
    exact_un = (int(Op.SQUARE), int(Op.NEG))
    rng = np.random.default_rng(seed)
    X = rng.uniform(-3, 3, (N, n_vars)).astype(np.float32)
    C = rng.standard_normal((B, M)).astype(np.float32)
    tb = tapes.generate(B, M, seed=seed + 1, lengths=rng.integers(min_len, M + 1, size=B),
                        const_counts=rng.integers(0, max_consts + 1, size=B), n_vars=n_vars, binary=exact_bin,
                        unary=exact_un, X_screen=X, C_screen=C)
    hid = tapes.generate(B, M, seed=seed + 2, lengths=rng.integers(3, min(M, 12) + 1, size=B),
                         const_counts=rng.integers(0, 3, size=B), n_vars=n_vars, binary=exact_bin, unary=exact_un,
                         X_screen=X, C_screen=C)
    yh = oracle.eval_fwd(X, hid.ops, hid.ch, rng.standard_normal((B, M)).astype(np.float32))
    root = np.maximum((hid.ops != 0).sum(1) - 1, 0)
    Y = yh[np.arange(B), root] + noise * rng.standard_normal((B, N)).astype(np.float32)
    Y = np.where(np.isfinite(Y) & (np.abs(Y) < 1e6), Y, 0.0).astype(np.float32)
    return X, Y, tb.ops, tb.ch, C


def _bits_differ(a, b):
    a = np.ascontiguousarray(a, np.float32)
    b = np.ascontiguousarray(b, np.float32)
    na, nb = np.isnan(a), np.isnan(b)
    return (na != nb) | (~na & ~nb & (a.view(np.uint32) != b.view(np.uint32)))


def assert_bit_identical(r, o, label):
    """Every output of the GPU fit r equals the oracle's o bit for bit (NaN as NaN)."""
    it_g, ev_g = r.iters.cpu().numpy(), r.evals.cpu().numpy()
    bad = (it_g != o["iters"]) | (ev_g != o["evals"])
    for a, b in ((r.C, o["C"]), (r.loss, o["loss"])):
        d = _bits_differ(a.cpu().numpy(), b)
        bad |= d.reshape(d.shape[0], -1).any(1) if d.ndim > 1 else d
    if r.Y is not None:
        bad |= _bits_differ(r.Y.cpu().numpy(), o["Y"]).any(1)
    idx = np.flatnonzero(bad)
    msg = "; ".join(f"problem {i}: iters {it_g[i]}/{o['iters'][i]} evals {ev_g[i]}/{o['evals'][i]} "
                    f"loss {float(r.loss[i])!r}/{float(o['loss'][i])!r}" for i in idx[:5])
    assert idx.size == 0, f"{label}: {idx.size} of {bad.size} problems differ from the oracle ({msg})"


@pytest.mark.parametrize("ls", ["strong_wolfe", "backtracking"])
@pytest.mark.parametrize("ppl,wpb", SHAPES)
def test_bit_identical_to_kernel_arithmetic(ppl, wpb, ls):
    """200 iterations of 192 ragged problems (N = 100: a partial last chunk), every shape."""
    sr = _sr()
    X, Y, ops, ch, C = exact_batch(192, 24, 100, seed=21)
    r = sr.optimize_ex(cuda(X), cuda(Y), cuda(ops), cuda(ch), cuda(C), max_iter=200, line_search_fn=ls,
                       points_per_lane=ppl, warps_per_block=wpb, raise_errors=False)
    o = oracle.optimize(X, Y, ops, ch, C, max_iter=200, line_search_fn=ls, dot_mode=2, warps=wpb,
                        points_per_lane=ppl)
    assert_bit_identical(r, o, f"V={ppl} W={wpb} {ls}")
    # the batch exercises the state machine: converged, capped and zoomed problems
    it = o["iters"]
    assert (it == 200).any() and ((it > 0) & (it < 200)).any() and (o["evals"] > it + 1).any()


@pytest.mark.parametrize("N", [5, 33, 257])
def test_bit_identical_point_counts(N):
    """Fewer points than a warp's lanes, one past a warp, and several chunks per warp."""
    sr = _sr()
    X, Y, ops, ch, C = exact_batch(96, 16, N, seed=30 + N)
    for ppl, wpb in ((1, 4), (2, 2)):
        r = sr.optimize_ex(cuda(X), cuda(Y), cuda(ops), cuda(ch), cuda(C), max_iter=120, points_per_lane=ppl,
                           warps_per_block=wpb, raise_errors=False)
        o = oracle.optimize(X, Y, ops, ch, C, max_iter=120, dot_mode=2, warps=wpb, points_per_lane=ppl)
        assert_bit_identical(r, o, f"N={N} V={ppl} W={wpb}")


@pytest.mark.parametrize("history", [3, 32, 40])
def test_bit_identical_history_wraps_and_many_constants(history):
    """History rings that wrap (3 pairs: every few iterations; 32: the most pairs of the
    compact representation, one lane each; 40: the two-loop recursion) and tapes with
    up to 40 constants (two slot registers per lane), both line searches."""
    sr = _sr()
    X, Y, ops, ch, C = exact_batch(64, 96, 64, seed=41, max_consts=40, min_len=60)
    assert oracle.kernel_slot_registers(ops) == 2
    for ls in ("strong_wolfe", "backtracking"):
        r = sr.optimize_ex(cuda(X), cuda(Y), cuda(ops), cuda(ch), cuda(C), max_iter=150, history_size=history,
                           line_search_fn=ls, points_per_lane=1, warps_per_block=2, raise_errors=False)
        o = oracle.optimize(X, Y, ops, ch, C, max_iter=150, history_size=history, line_search_fn=ls, dot_mode=2,
                            warps=2, points_per_lane=1)
        assert_bit_identical(r, o, f"history {history}, up to 40 constants, {ls}")
        if history > 3:
            assert r.iters.cpu().numpy().max() > history, "the ring never wrapped"


def test_bit_identical_raw_objective_rosenbrock(golden):
    """The raw-objective mode on the batched Rosenbrock function (square, sub, mul:
    IEEE-exact), the reference's LBFGS_batch known answer (tests/test_lbfgs_batch.py:38-75)."""
    sr = _sr()
    x0 = golden("rosenbrock")["x0"]
    B = x0.shape[1]
    # f = (1 - c0)^2 + 100 (c1 - c0^2)^2 over the slots 1 (c0) and 4 (c1)
    ops1 = np.array([2, 1, 41, 14, 1, 14, 41, 14, 6, 6, 42, 5, 42, 42, 40], np.int64)
    ch1 = np.array([(-1, -1), (-1, -1), (0, 1), (2, -1), (-1, -1), (1, -1), (4, 5), (6, -1), (-1, -1), (-1, -1),
                    (8, 9), (-1, -1), (10, 11), (12, 7), (3, 13)], np.int64)
    M = ops1.shape[0]
    ops = np.tile(ops1, (B, 1))
    ch = np.tile(ch1, (B, 1, 1))
    C = np.zeros((B, M), np.float32)
    C[:, 1], C[:, 4] = x0[0], x0[1]
    X = np.zeros((1, 1), np.float32)
    for ls in ("strong_wolfe", "backtracking"):
        r = sr.optimize_ex(cuda(X), None, cuda(ops), cuda(ch), cuda(C), max_iter=250, history_size=15,
                           line_search_fn=ls, objective=1, points_per_lane=1, warps_per_block=1)
        o = oracle.optimize(X, None, ops, ch, C, max_iter=250, history_size=15, line_search_fn=ls, dot_mode=2,
                            warps=1, points_per_lane=1)
        assert_bit_identical(r, o, f"Rosenbrock {ls}")
        np.testing.assert_allclose(o["C"][:, [1, 4]], 1.0, atol=1e-3)


def _transcendental_sets(golden):
    from cudasymbolicregression_gb300 import workloads
    sets = []
    for name, ls in (("optimize_readme", "strong_wolfe"), ("optimize_ragged", "strong_wolfe"),
                     ("optimize_ragged_bt", "backtracking")):
        g = golden(name)
        sets.append((name, ls, int(g["max_iter"]), g["X"], g["Y"], g["ops"], g["ch"], g["C"]))
    wl = workloads.ragged_fit(B=2048, N=128, M=32, seed=5)
    sets.append(("ragged_2048", "strong_wolfe", 200, wl.X, wl.Y, wl.ops, wl.ch, wl.C))
    return sets


@pytest.mark.parametrize("class_width", [0, 16])
def test_bit_identical_with_sin_cos_exp_log(golden, class_width):
    """Tapes with sin, cos, exp and log (the library's own functions, which the oracle
    compiles from the same source): the reference's three fixtures at their own
    iteration counts and 2048 ragged problems at 200 iterations, with the launch shape
    the library picks by itself (one launch, or one per class of tape lengths).  A
    problem that differs is reported with the first iteration at which its constants
    part from the oracle's by more than 1e-4 relative."""
    sr = _sr()
    report = []
    for name, ls, mi, X, Y, ops, ch, C in _transcendental_sets(golden):
        r = sr.optimize_ex(cuda(X), cuda(Y), cuda(ops), cuda(ch), cuda(C), max_iter=mi, line_search_fn=ls,
                           class_width=class_width, raise_errors=False)
        o = oracle_fit_like(r, X, Y, ops, ch, C, max_iter=mi, line_search_fn=ls)
        bad = np.flatnonzero(fit_bits_differ(r, o))
        if bad.size:
            shape = {int(i): (V, W) for idx, V, W in r.shapes for i in idx.cpu().numpy()}
            V, W = shape[int(bad[0])]

            def gpu_c(k, idx):
                rr = sr.optimize_ex(cuda(X), cuda(Y[idx]), cuda(ops[idx]), cuda(ch[idx]), cuda(C[idx]), max_iter=k,
                                    line_search_fn=ls, points_per_lane=V, warps_per_block=W, raise_errors=False)
                return rr.C.cpu().numpy()

            def ora_c(k, idx):
                return oracle.optimize(X, Y[idx], ops[idx], ch[idx], C[idx], max_iter=k, line_search_fn=ls, dot_mode=2,
                                       warps=W, points_per_lane=V, slot_registers=oracle.kernel_slot_registers(ops))["C"]
            sel = bad[:4]
            first = first_divergence(gpu_c, ora_c, sel, mi)
            report.append(f"{name}: {bad.size} of {len(ops)} problems differ; " + ", ".join(
                f"[{i}] iters {int(r.iters[i])}/{o['iters'][i]}, apart after {f} iterations" for i, f in zip(sel, first)))
    assert not report, "; ".join(report)
