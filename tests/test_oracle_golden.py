"""The CPU oracle against the reference's own outputs (tests/golden/*.npz).

The fixtures were written by tests/golden/make_golden.py from the reference
compiled from its sources.  Forward values must be bit-exact (same libm, same
operation order); adjoints within float32 summation-order noise; optimize()
within the chaos that summation-order differences cause in L-BFGS.
"""
import numpy as np
import pytest

import oracle


@pytest.mark.parametrize("name", ["single_ops", "random_dags", "random_default_ops"])
def test_forward_bit_exact(golden, name):
    g = golden(name)
    cache = oracle.eval_fwd(g["X"], g["ops"], g["ch"], g["C"])
    assert np.array_equal(cache, g["cache"], equal_nan=True)


@pytest.mark.parametrize("name", ["single_ops", "random_dags", "random_default_ops"])
def test_backward(golden, name):
    g = golden(name)
    gC, gX, err = oracle.eval_bwd(g["X"], g["ops"], g["ch"], g["C"], g["gout"])
    assert err == 0
    for mine, ref in ((gC, g["gC"]), (gX, g["gX"])):
        assert np.array_equal(np.isnan(mine), np.isnan(ref))
        fin = np.isfinite(ref)
        np.testing.assert_allclose(mine[fin], ref[fin], rtol=1e-5, atol=1e-5 * max(1.0, np.abs(ref[fin]).max(initial=0)))


def test_multiple_constants_against_reference(golden):
    """evaluate_multiple (reference symbolic_torch/evaluation.py:36-65): every set is
    a single-set evaluation; gradients per set, X gradient summed over the sets."""
    g = golden("multiple")
    cache = oracle.eval_fwd_multi(g["X"], g["ops"], g["ch"], g["C"])
    assert np.array_equal(cache, g["cache"], equal_nan=True)
    gC, gX, err = oracle.eval_bwd_multi(g["X"], g["ops"], g["ch"], g["C"], g["gout"])
    assert err == 0
    for mine, ref in ((gC, g["gC"]), (gX, g["gX"])):
        assert np.array_equal(np.isnan(mine), np.isnan(ref))
        fin = np.isfinite(ref)
        np.testing.assert_allclose(mine[fin], ref[fin], rtol=1e-5, atol=1e-5 * max(1.0, np.abs(ref[fin]).max(initial=0)))


def test_single_op_x_gradients_per_row(golden):
    g = golden("single_ops")
    B = g["ops"].shape[0]
    for b in range(B):
        _, gX, err = oracle.eval_bwd(g["X"], g["ops"][b:b + 1], g["ch"][b:b + 1], g["C"][b:b + 1], g["gout"][b:b + 1])
        assert err == 0
        ref = g["gX_rows"][b]
        assert np.array_equal(np.isnan(gX), np.isnan(ref)), b
        fin = np.isfinite(ref)
        np.testing.assert_allclose(gX[fin], ref[fin], rtol=1e-6, atol=1e-6)


def test_error_codes(golden):
    g = golden("errors")
    expect = {"child_geq": 101, "unary_nochild": 102, "binary_onechild": 102, "leaf_child": 102}
    for name, code in expect.items():
        assert oracle.validate(g[name + "__ops"], g[name + "__ch"]) == code
        assert oracle.ERR_MESSAGES[code] in str(g[name + "__msg"])
    # backward errors
    for name, code in (("noop_grad", 201), ("div_zero", 204)):
        ops, ch, X = g[name + "__ops"], g[name + "__ch"], g[name + "__X"]
        C = np.zeros(ops.shape, np.float32)
        cache = oracle.eval_fwd(X, ops, ch, C)
        gout = np.zeros_like(cache)
        gout[:, -1, :] = 1.0
        _, _, err = oracle.eval_bwd(X, ops, ch, C, gout)
        assert err == code
        assert oracle.ERR_MESSAGES[code] in str(g[name + "__msg"])


def test_optimize_linear_known_answer(golden):
    g = golden("optimize_linear")
    for mode in (0, 1):
        r = oracle.optimize(g["X"], g["Y"], g["ops"], g["ch"], g["C"], dot_mode=mode)
        assert r["err"] == 0
        np.testing.assert_allclose(r["C"][:, 1], [2.5, -1.5], atol=1e-3)
        np.testing.assert_allclose(r["C"][:, 3], [0.5, 3.0], atol=1e-3)
        np.testing.assert_allclose(r["C"], g["C_final"], rtol=1e-5, atol=1e-6)


@pytest.mark.parametrize("name,ls,min_frac", [("optimize_readme", "strong_wolfe", 0.95),
                                              ("optimize_ragged", "strong_wolfe", 0.8),
                                              ("optimize_ragged_bt", "backtracking", 0.9)])
def test_optimize_matches_reference(golden, name, ls, min_frac):
    g = golden(name)
    mi = int(g["max_iter"])
    r = oracle.optimize(g["X"], g["Y"], g["ops"], g["ch"], g["C"], max_iter=mi, dot_mode=0, line_search_fn=ls)
    assert r["err"] == 0
    mse_r = ((g["Y_final"] - g["Y"]) ** 2).mean(1)
    mse_o = ((r["Y"] - g["Y"]) ** 2).mean(1)
    with np.errstate(invalid="ignore", divide="ignore"):
        rel = np.abs(mse_o - mse_r) / np.maximum(np.abs(mse_r), 1e-30)
    same = (rel < 1e-4) | (np.isnan(mse_r) & np.isnan(mse_o))
    # float32 summation order differs from torch's cascade sums; L-BFGS
    # amplifies ulp differences on ill-conditioned problems.
    assert same.mean() >= min_frac
    # no systematic quality shift: the oracle is not worse on the median
    assert np.nanmedian(mse_o) <= np.nanmedian(mse_r) * 1.5 + 1e-6


def test_optimize_first_iteration_bit_exact(golden):
    """With one L-BFGS iteration every summation is short enough to agree bit for bit."""
    g = golden("optimize_ragged")
    r1 = oracle.optimize(g["X"], g["Y"], g["ops"], g["ch"], g["C"], max_iter=0, dot_mode=0)
    assert np.array_equal(r1["C"], g["C"])


def _rosenbrock_tape():
    """f = (1 - c0)^2 + 100 (c1 - c0^2)^2 as a postfix tape over two constants (slots 1, 4)."""
    ops = [2, 1, 41, 14, 1, 14, 41, 14, 6, 6, 42, 5, 42, 42, 40]
    ch = [(-1, -1), (-1, -1), (0, 1), (2, -1), (-1, -1), (1, -1), (4, 5), (6, -1), (-1, -1), (-1, -1), (8, 9),
          (-1, -1), (10, 11), (12, 7), (3, 13)]
    return np.array(ops, np.int64), np.array(ch, np.int64)


@pytest.mark.parametrize("ls,key", [("strong_wolfe", "x_wolfe"), ("backtracking", "x_backtracking")])
def test_optimize_rosenbrock_known_answer(golden, ls, key):
    """reference tests/test_lbfgs_batch.py:38-75: LBFGS_batch from ten starts reaches
    (1, 1); the oracle, in the reference's float32 arithmetic, reaches the reference's
    own end points (tests/golden/rosenbrock.npz)."""
    g = golden("rosenbrock")
    x0 = g["x0"]
    B = x0.shape[1]
    ops1, ch1 = _rosenbrock_tape()
    ops, ch = np.tile(ops1, (B, 1)), np.tile(ch1, (B, 1, 1))
    C = np.zeros((B, ops1.shape[0]), np.float32)
    C[:, 1], C[:, 4] = x0[0], x0[1]
    o = oracle.optimize(np.zeros((1, 1), np.float32), None, ops, ch, C, max_iter=250, history_size=15,
                        line_search_fn=ls, dot_mode=0)
    np.testing.assert_allclose(o["C"][:, [1, 4]], 1.0, atol=1e-3)
    np.testing.assert_allclose(o["C"][:, [1, 4]], g[key].T, atol=1e-3)


def test_evaluation_known_answers():
    """reference tests/test_symbolic_evaluation.py:435-478 (C = 3.14 gives 1 + C = 4.14
    and sin(3.14)) and :192-217 (a NO_OP row evaluates to NaN and passes zero
    gradients), on the oracle."""
    X = np.random.default_rng(0).standard_normal((4, 1)).astype(np.float32)
    C = np.array([[3.14, 0, 0]], np.float32)
    ch = np.array([[[-1, -1], [-1, -1], [0, 1]]], np.int64)
    cache = oracle.eval_fwd(X, np.array([[1, 2, 40]], np.int64), ch, C)
    np.testing.assert_allclose(cache[0, 2], np.float32(3.14) + np.float32(1), atol=1e-6)
    ch = np.array([[[-1, -1], [0, -1]]], np.int64)
    cache = oracle.eval_fwd(X, np.array([[1, 10]], np.int64), ch, C[:, :2])
    np.testing.assert_allclose(cache[0, 1], np.sin(np.float32(3.14)), atol=1e-6)
    ops, ch, C0 = np.zeros((1, 1), np.int64), -np.ones((1, 1, 2), np.int64), np.zeros((1, 1), np.float32)
    X2 = np.random.default_rng(1).standard_normal((10, 2)).astype(np.float32)
    assert np.isnan(oracle.eval_fwd(X2, ops, ch, C0)).all()
    gC, gX, err = oracle.eval_bwd(X2, ops, ch, C0, np.zeros((1, 1, 10), np.float32))
    assert err == 0 and not gC.any() and not gX.any()
