"""The summation bound that grad_X is held to, checked on the CPU.

grad_X is an atomic float32 sum over tapes and variable nodes on the device (as in the
reference's adjoint, which adds with atomics too), so its order of addition is not
fixed and it has no single bit pattern to compare with.  Its terms are fixed, though:
each variable node's adjoint at each point, which the oracle forms in the kernels'
arithmetic.  oracle.check_gx_bound accepts a grad_X only if every entry is a float32 sum
of those terms in some order: within the recursive-summation error bound where the
terms are finite, NaN or the right infinity where they are not.  These tests pin that
checker: the oracle's own float32 sums (another order of the same terms) pass, the
bound is a few 1e-5 of the sums (the worst case over every order of a few hundred
terms), and planted mistakes fail.
"""
import numpy as np

import oracle

EXACT_UNARY = (10, 11, 12, 13, 14, 15, 23, 24, 25, 27, 28, 29, 30, 31)
EXACT_BINARY = (40, 41, 42, 43)
# operators that keep every value finite at these inputs (sin cos square neg; + - *), so
# that most grad_X entries are finite sums and the bound itself is exercised
FINITE_UNARY = (10, 11, 14, 28)
FINITE_BINARY = (40, 41, 42)


def _batch(seed, B, M, N, nx, unary=EXACT_UNARY, binary=EXACT_BINARY):
    from cudasymbolicregression_gb300 import tapes
    rng = np.random.default_rng(seed)
    X = rng.uniform(-3, 3, (N, nx)).astype(np.float32)
    C = rng.standard_normal((B, M)).astype(np.float32)
    tb = tapes.generate(B, M, seed=seed, mean_length=M / 3, n_vars=nx, unary=unary, binary=binary,
                        p_const_leaf=0.3, X_screen=X, C_screen=C)
    gout = rng.standard_normal((B, M, N)).astype(np.float32)
    gout[np.isnan(oracle.eval_fwd(X, tb.ops, tb.ch, C, kernel_math=True))] = 0.0
    return X, C, tb.ops, tb.ch, gout


def test_oracle_sums_in_another_order_pass():
    for seed, B, M, N, nx, ops_set in ((1, 300, 40, 45, 3, 0), (4, 33, 17, 129, 2, 0), (6, 200, 64, 64, 4, 0),
                                       (7, 200, 64, 64, 4, 1), (8, 1000, 24, 33, 2, 1)):
        X, C, ops, ch, gout = _batch(seed, B, M, N, nx, *((FINITE_UNARY, FINITE_BINARY) if ops_set else ()))
        gc, err, terms = oracle.eval_gc_kernel_order(X, ops, ch, C, gout, gx_terms=True)
        assert err == 0
        # per tape, then over the tapes: a different order of the same float32 terms
        _, gx, err2 = oracle.eval_bwd(X, ops, ch, C, gout, kernel_math=True)
        assert err2 == 0
        ok, slack = oracle.check_gx_bound(gx, terms)
        assert ok.all(), (seed, np.argwhere(~ok)[:5], slack.max())
        assert (terms["count"] > 1).any()


def test_bound_is_near_the_float32_rounding_and_rejects_what_exceeds_it():
    X, C, ops, ch, gout = _batch(7, 200, 64, 64, 4, FINITE_UNARY, FINITE_BINARY)
    _, _, terms = oracle.eval_gc_kernel_order(X, ops, ch, C, gout, gx_terms=True)
    _, gx, _ = oracle.eval_bwd(X, ops, ch, C, gout, kernel_math=True)
    n, a, s = terms["count"], terms["abs"], terms["sum"]
    fin = np.isfinite(gx) & (n >= 10) & (s != 0)
    assert fin.mean() > 0.5
    # the worst case over all orders of about 300 terms: (n - 1) u |terms|, a few 1e-5
    # of the sum here (the oracle's own order uses well under a tenth of it)
    bound = (n - 1) * 2.0 ** -24 * a
    assert np.median(bound[fin] / np.abs(s[fin])) < 1e-4
    ok, slack = oracle.check_gx_bound(gx, terms)
    assert ok.all() and np.median(slack[fin]) < 0.1
    # moved by three bounds (many float32 ulps at n >= 10): rejected
    i = np.flatnonzero(fin)[:64]
    bad = gx.astype(np.float64)
    bad.flat[i] = s.flat[i] + 3 * bound.flat[i] * np.sign(s.flat[i])
    ok, _ = oracle.check_gx_bound(bad.astype(np.float32), terms)
    assert not ok.flat[i].any()


def test_non_finite_placement_is_checked():
    # tapes with log, sqrt and division: most entries have a NaN term somewhere
    X, C, ops, ch, gout = _batch(1, 300, 40, 45, 3)
    _, _, terms = oracle.eval_gc_kernel_order(X, ops, ch, C, gout, gx_terms=True)
    _, gx, _ = oracle.eval_bwd(X, ops, ch, C, gout, kernel_math=True)
    ok, _ = oracle.check_gx_bound(gx, terms)
    assert ok.all() and np.isnan(gx).any()
    X, C, ops, ch, gout = _batch(7, 200, 64, 64, 4, FINITE_UNARY, FINITE_BINARY)
    _, _, terms = oracle.eval_gc_kernel_order(X, ops, ch, C, gout, gx_terms=True)
    _, gx, _ = oracle.eval_bwd(X, ops, ch, C, gout, kernel_math=True)
    fin = np.flatnonzero(np.isfinite(gx))
    planted = gx.copy()
    planted.flat[fin[0]] = np.nan
    assert not oracle.check_gx_bound(planted, terms)[0].flat[fin[0]]
    planted = gx.copy()
    planted.flat[fin[1]] = np.inf
    assert not oracle.check_gx_bound(planted, terms)[0].flat[fin[1]]
    # a NaN term must give NaN, both infinities NaN, one infinity that infinity
    t = {"sum": np.zeros((1, 4)), "abs": np.zeros((1, 4)), "count": np.ones((1, 4), np.int32),
         "flags": np.array([[1, 6, 2, 4]], np.int32)}
    ok, _ = oracle.check_gx_bound(np.array([[np.nan, np.nan, np.inf, -np.inf]], np.float32), t)
    assert ok.all()
    ok, _ = oracle.check_gx_bound(np.array([[0.0, np.inf, -np.inf, np.inf]], np.float32), t)
    assert not ok.any()


def test_no_terms_means_zero():
    t = {"sum": np.zeros((2, 1)), "abs": np.zeros((2, 1)), "count": np.zeros((2, 1), np.int32),
         "flags": np.zeros((2, 1), np.int32)}
    ok, _ = oracle.check_gx_bound(np.array([[0.0], [1e-30]], np.float32), t)
    assert ok[0, 0] and not ok[1, 0]
