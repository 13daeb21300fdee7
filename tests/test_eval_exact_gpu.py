"""Exact parity of the evaluation kernels against the oracle in the kernels' arithmetic.

A forward value depends only on per-point arithmetic, and sin, cos, exp and log are the
library's own functions (csrc/sr_fmath.h), which the oracle compiles from the same
source.  On tapes whose other operators are IEEE-exact (+ - * /, square, sqrt, neg, inv,
cube, fourth, fifth, floor, ceil) the whole (B, M, N) cache must therefore equal the
oracle's bit for bit, NaN placement included, along entire tapes and not just node by
node.  The gradient of the constants is a sum over the points in a fixed order (per
lane over the 32-point chunks, then a lane butterfly), which
oracle.eval_gc_kernel_order restates: grad_C must equal it bit for bit as well.  The
X gradient is an atomic sum over the tapes and variable nodes, in the reference too, so
its order is not fixed; its terms are (each variable node's adjoint at each point), and
every entry must be a float32 sum of exactly those terms in some order: within the
worst-case error bound of such a sum where they are finite, NaN or the right infinity
where they are not (oracle.check_gx_bound), on every entry.
"""
import numpy as np
import pytest
import torch

import oracle

pytestmark = pytest.mark.gpu

EXACT_UNARY = (10, 11, 12, 13, 14, 15, 23, 24, 25, 27, 28, 29, 30, 31)  # sin cos exp log square sqrt floor ceil ln neg inv cube fourth fifth
EXACT_BINARY = (40, 41, 42, 43)


def cuda(a):
    return torch.as_tensor(np.ascontiguousarray(a)).cuda()


def _bits_equal(a, b):
    a = np.ascontiguousarray(a, np.float32)
    b = np.ascontiguousarray(b, np.float32)
    na, nb = np.isnan(a), np.isnan(b)
    return np.array_equal(na, nb) and np.array_equal(a.view(np.uint32)[~na], b.view(np.uint32)[~nb])


# operators that keep every value finite at these inputs (sin cos square neg; + - *):
# most grad_X entries are then finite sums of a few hundred terms
FINITE_UNARY = (10, 11, 14, 28)
FINITE_BINARY = (40, 41, 42)


def _batch(seed, B, M, N, nx, unary=EXACT_UNARY, binary=EXACT_BINARY):
    from cudasymbolicregression_gb300 import tapes
    rng = np.random.default_rng(seed)
    X = rng.uniform(-3, 3, (N, nx)).astype(np.float32)
    C = rng.standard_normal((B, M)).astype(np.float32)
    tb = tapes.generate(B, M, seed=seed, mean_length=M / 3, n_vars=nx, unary=unary, binary=binary,
                        p_const_leaf=0.3, X_screen=X, C_screen=C)
    return rng, X, C, tb.ops, tb.ch


def _assert_gx_bound(gx, terms):
    ok, slack = oracle.check_gx_bound(gx, terms)
    bad = np.argwhere(~ok)
    assert ok.all(), f"{len(bad)} grad_X entries outside the float-sum bound, first {bad[:4].tolist()}: " \
                     f"got {gx[tuple(bad[0])]}, terms sum {terms['sum'][tuple(bad[0])]}, flags {terms['flags'][tuple(bad[0])]}"
    return slack


@pytest.mark.parametrize("seed,B,M,N,nx", [(1, 300, 40, 45, 3), (2, 64, 64, 1000, 4), (3, 7, 5, 1, 1),
                                             (4, 33, 17, 129, 2), (5, 512, 64, 256, 4)])
def test_cache_and_constant_gradient_bit_identical(seed, B, M, N, nx):
    import cudasymbolicregression_gb300 as sr
    rng, X, C, ops, ch = _batch(seed, B, M, N, nx)
    Ct = cuda(C).requires_grad_(True)
    out = sr.evaluation.evaluate(cuda(X), cuda(ops), cuda(ch), Ct)
    got = out.detach().cpu().numpy()
    want = oracle.eval_fwd(X, ops, ch, C, kernel_math=True)
    assert _bits_equal(got, want), "forward cache differs from the oracle"
    gout = rng.standard_normal(got.shape).astype(np.float32)
    gout[np.isnan(got)] = 0.0
    gc_want, err = oracle.eval_gc_kernel_order(X, ops, ch, C, gout)
    if err:
        pytest.skip("seeded tapes hit a zero denominator under a nonzero gradient")
    out.backward(cuda(gout))
    assert _bits_equal(Ct.grad.cpu().numpy(), gc_want), "grad_C differs from the oracle"


def test_reference_fixture_cache_bit_identical(golden):
    """The reference's own random tapes over +,-,*,/,sin,cos,exp,log (the evaluation
    workload's operators): the device cache equals the kernel-arithmetic oracle's
    everywhere, the constant gradient of the fixture's dense output gradient too, and
    grad_X is within the float-sum bound of its terms on every entry."""
    import cudasymbolicregression_gb300 as sr
    g = golden("random_default_ops")
    assert np.isin(g["ops"], (0, 1, 2, 3, 4, 5, 6, 7, 8) + EXACT_UNARY + EXACT_BINARY + tuple(range(50, 60))).all()
    Xt = cuda(g["X"]).requires_grad_(True)
    Ct = cuda(g["C"]).requires_grad_(True)
    out = sr.evaluation.evaluate(Xt, cuda(g["ops"]), cuda(g["ch"]), Ct)
    assert _bits_equal(out.detach().cpu().numpy(), oracle.eval_fwd(g["X"], g["ops"], g["ch"], g["C"], kernel_math=True))
    gc_want, err, terms = oracle.eval_gc_kernel_order(g["X"], g["ops"], g["ch"], g["C"], g["gout"], gx_terms=True)
    assert err == 0
    out.backward(cuda(g["gout"]))
    assert _bits_equal(Ct.grad.cpu().numpy(), gc_want)
    _assert_gx_bound(Xt.grad.cpu().numpy(), terms)


@pytest.mark.parametrize("seed,B,M,N,nx,finite", [(1, 300, 40, 45, 3, False), (2, 64, 64, 1000, 4, False),
                                                    (7, 200, 64, 64, 4, True), (8, 1000, 24, 33, 2, True),
                                                    (9, 64, 64, 1000, 4, True), (10, 3, 6, 1, 1, True)])
def test_variable_gradient_within_the_float_sum_bound(seed, B, M, N, nx, finite):
    """grad_X on every entry: a float32 sum of the oracle's variable-node adjoints (the
    same terms bit for bit, as grad_C shows) in some order.  The exact-operator tapes
    (log, sqrt, division) put a NaN term into most entries, which checks NaN placement;
    the finite-operator tapes check the bound itself, a few 1e-5 of the sums here."""
    import cudasymbolicregression_gb300 as sr
    ops_set = (FINITE_UNARY, FINITE_BINARY) if finite else ()
    rng, X, C, ops, ch = _batch(seed, B, M, N, nx, *ops_set)
    Xt = cuda(X).requires_grad_(True)
    Ct = cuda(C).requires_grad_(True)
    out = sr.evaluation.evaluate(Xt, cuda(ops), cuda(ch), Ct)
    got = out.detach().cpu().numpy()
    assert _bits_equal(got, oracle.eval_fwd(X, ops, ch, C, kernel_math=True))
    gout = rng.standard_normal(got.shape).astype(np.float32)
    gout[np.isnan(got)] = 0.0
    gc_want, err, terms = oracle.eval_gc_kernel_order(X, ops, ch, C, gout, gx_terms=True)
    if err:
        pytest.skip("seeded tapes hit a zero denominator under a nonzero gradient")
    out.backward(cuda(gout))
    assert _bits_equal(Ct.grad.cpu().numpy(), gc_want)
    gx = Xt.grad.cpu().numpy()
    slack = _assert_gx_bound(gx, terms)
    if finite:
        assert np.isfinite(gx).mean() > 0.9
        # over many terms the rounding errors partly cancel: far below the worst case
        many = terms["count"] >= 10
        if many.any():
            assert np.median(slack[many]) < 0.5


def test_multiple_sets_bit_identical():
    """evaluate_multiple: every constant set's cache and grad_C equal the oracle's for
    that set (the sets are evaluated one after the other inside one launch)."""
    import cudasymbolicregression_gb300 as sr
    rng, X, C, ops, ch = _batch(7, 96, 32, 200, 3)
    K = 3
    C3 = rng.standard_normal((C.shape[0], C.shape[1], K)).astype(np.float32)
    Xt = cuda(X).requires_grad_(True)
    Ct = cuda(C3).requires_grad_(True)
    out = sr.evaluation.evaluate_multiple(Xt, cuda(ops), cuda(ch), Ct)
    got = out.detach().cpu().numpy()
    gout = rng.standard_normal(got.shape).astype(np.float32)
    gout[np.isnan(got)] = 0.0
    want_gc, terms = [], None
    for k in range(K):
        assert _bits_equal(got[..., k], oracle.eval_fwd(X, ops, ch, C3[:, :, k], kernel_math=True)), f"set {k}"
        gc, err, t = oracle.eval_gc_kernel_order(X, ops, ch, C3[:, :, k], gout[..., k], gx_terms=True)
        if err:
            pytest.skip("seeded tapes hit a zero denominator under a nonzero gradient")
        want_gc.append(gc)
        # grad_X adds the terms of every set: sums and counts add, flags combine
        terms = t if terms is None else {"sum": terms["sum"] + t["sum"], "abs": terms["abs"] + t["abs"],
                                         "count": terms["count"] + t["count"], "flags": terms["flags"] | t["flags"]}
    out.backward(cuda(gout))
    assert _bits_equal(Ct.grad.cpu().numpy(), np.stack(want_gc, axis=2))
    _assert_gx_bound(Xt.grad.cpu().numpy(), terms)
