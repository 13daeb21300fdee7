"""GPU parity of optimize() (the fused batched L-BFGS kernel).

Two references.  The oracle's kernel-arithmetic mode (oracle/sr_oracle.c, dot_mode 2)
runs the reference's control flow with the kernel's arithmetic, and the kernel must
equal it bit for bit (here and in tests/test_fit_exact_gpu.py).  The reference's own
fits (tests/golden, written by the reference's CPU path on one thread) are matched
statistically: the reference's float32 sums differ from the kernel's float-pair
sums, and L-BFGS amplifies such rounding on ill-conditioned problems.  The reference
itself is not reproducible run to run: its CPU path sums gradients with OpenMP
atomics (its CUDA path with atomicAdd), and rerun on 2, 4 or 8 threads it matches its
own single-thread fixture within 1e-4 on 97.7-99.2% of the README problems and
95.8-97.9% of the backtracking set (medians 10.24-11.07 against 10.56), and on the
strong-Wolfe ragged set every multi-thread rerun aborts with error 204.  The bars
below sit at or under those figures.
"""
import numpy as np
import pytest
import torch

import oracle

pytestmark = pytest.mark.gpu


def _sr():
    import cudasymbolicregression_gb300 as sr
    return sr


def cuda(a, dtype=None):
    t = torch.as_tensor(np.ascontiguousarray(a))
    if dtype is not None:
        t = t.to(dtype)
    return t.cuda()


def mse(Yf, Y):
    return ((np.asarray(Yf, np.float64) - np.asarray(Y, np.float64)) ** 2).mean(1)


def rel_close(a, b, rtol):
    with np.errstate(invalid="ignore", divide="ignore"):
        r = np.abs(a - b) / np.maximum(np.abs(b), 1e-30)
    return (r <= rtol) | (np.isnan(a) & np.isnan(b)) | (a == b)


def assert_no_systematic_loss(m_dev, m_ref, diff):
    """Paired quality check over the problems whose final MSEs differ (finite in both).
    Two fits of one ill-conditioned problem that part by a rounding end in unrelated
    local minima: the log ratio of their MSEs has a spread of several units, so a
    fixed bound on its mean is noise at any affordable sample size.  Instead: the
    device is worse on no more problems than a fair coin gives within two standard
    deviations (sign test), and the mean log ratio lies within two standard errors of
    zero or below it."""
    if diff.sum() < 2:
        return
    lr = np.log(np.maximum(m_dev[diff], 1e-30) / np.maximum(m_ref[diff], 1e-30))
    n = lr.size
    assert (lr > 0).sum() <= n / 2 + np.sqrt(n) + 1, f"device worse on {(lr > 0).sum()} of {n}"
    assert lr.mean() <= 2 * lr.std(ddof=1) / np.sqrt(n), f"mean log ratio {lr.mean():.3f} over {n}"


def test_linear_known_answer(golden):
    """reference tests/test_optimization.py:10-80."""
    sr = _sr()
    g = golden("optimize_linear")
    C_init = cuda(g["C"])
    Cf, Yf = sr.optimize(cuda(g["X"]), cuda(g["Y"]), cuda(g["ops"]), cuda(g["ch"]), C_init)
    Cf = Cf.cpu().numpy()
    np.testing.assert_allclose(Cf[:, 1], [2.5, -1.5], atol=1e-3)
    np.testing.assert_allclose(Cf[:, 3], [0.5, 3.0], atol=1e-3)
    mask = g["ops"] == 1
    np.testing.assert_array_equal(Cf[~mask], g["C"][~mask])
    np.testing.assert_allclose(Yf.cpu().numpy(), g["Y"], atol=1e-3)
    np.testing.assert_allclose(Cf, g["C_final"], rtol=1e-4, atol=1e-5)


@pytest.mark.parametrize("name,ls,min_frac", [("optimize_readme", "strong_wolfe", 0.97),
                                              ("optimize_ragged", "strong_wolfe", 0.8),
                                              ("optimize_ragged_bt", "backtracking", 0.95)])
def test_matches_reference_golden(golden, name, ls, min_frac):
    """Final MSE against the reference's own fits: within 1e-4 relative on at least
    min_frac of the problems (the reference's own reruns reach 0.977 and 0.958 on the
    first and last set and cannot run the second).  Quality, paired over the problems
    finite in both whose MSE differs by more than 1e-4: no systematic loss (sign test
    and mean log ratio, assert_no_systematic_loss), and the device leaves at most 2
    more problems non-finite than the reference."""
    sr = _sr()
    g = golden(name)
    r = sr.optimize_ex(cuda(g["X"]), cuda(g["Y"]), cuda(g["ops"]), cuda(g["ch"]), cuda(g["C"]),
                       max_iter=int(g["max_iter"]), line_search_fn=ls, raise_errors=False)
    ok = r.iters.cpu().numpy() >= 0  # ill-conditioned trajectories may reach a/0 (error 204)
    assert ok.mean() >= 0.95
    m_gpu = mse(r.Y.cpu().numpy(), g["Y"])
    m_ref = mse(g["Y_final"], g["Y"])
    close = rel_close(m_gpu, m_ref, 1e-4)
    assert close[ok].mean() >= min_frac
    fin = ok & np.isfinite(m_gpu) & np.isfinite(m_ref)
    assert_no_systematic_loss(m_gpu, m_ref, fin & ~close)
    assert (ok & ~np.isfinite(m_gpu) & np.isfinite(m_ref)).sum() <= (ok & np.isfinite(m_gpu) & ~np.isfinite(m_ref)).sum() + 2
    # NaN placement of the constants: NaN expressions end with every slot NaN
    nan_ref = np.isnan(g["C_final"]).all(1)
    nan_gpu = np.isnan(r.C.cpu().numpy()).all(1)
    assert (nan_ref == nan_gpu)[ok].mean() >= min_frac


def _ragged_problems(seed, B, N=64, M=32):
    """Problems of the fixture's kind (tests/golden/make_golden.py case_optimize_ragged):
    ragged tapes of 3..M nodes with 0..8 constants over 2 variables, targets from hidden
    random tapes plus noise, evaluated by the oracle."""
    from cudasymbolicregression_gb300 import tapes
    rng = np.random.default_rng(seed)
    X = rng.uniform(-3, 3, (N, 2)).astype(np.float32)
    C = rng.standard_normal((B, M)).astype(np.float32)
    tb = tapes.generate(B, M, seed=seed + 1, lengths=rng.integers(3, M + 1, size=B),
                        const_counts=rng.integers(0, 9, size=B), n_vars=2, X_screen=X, C_screen=C)
    hid = tapes.generate(B, M, seed=seed + 2, lengths=rng.integers(3, 16, size=B),
                         const_counts=rng.integers(0, 4, size=B), n_vars=2, X_screen=X, C_screen=C)
    yh = oracle.eval_fwd(X, hid.ops, hid.ch, rng.standard_normal((B, M)).astype(np.float32))
    Y = yh[np.arange(B), np.maximum((hid.ops != 0).sum(1) - 1, 0)] + 0.01 * rng.standard_normal((B, N))
    return X, np.where(np.isfinite(Y), Y, 0.0).astype(np.float32), tb.ops, tb.ch, C


@pytest.mark.parametrize("ls,max_iter", [("strong_wolfe", 40), ("backtracking", 30)])
def test_quality_against_reference_arithmetic_large_sample(ls, max_iter):
    """2048 problems of the fixtures' kind, fitted by the device and by the oracle in
    the reference's float32 arithmetic (pinned to the reference's own fits by
    tests/test_oracle_golden.py): at least 90% within 1e-4 relative, no systematic loss
    over the rest, and at most 1% more problems left non-finite."""
    sr = _sr()
    X, Y, ops, ch, C = _ragged_problems(11, 2048)
    r = sr.optimize_ex(cuda(X), cuda(Y), cuda(ops), cuda(ch), cuda(C), max_iter=max_iter, line_search_fn=ls,
                       raise_errors=False)
    o = oracle.optimize(X, Y, ops, ch, C, max_iter=max_iter, line_search_fn=ls, dot_mode=0)
    ok = (r.iters.cpu().numpy() >= 0) & (o["iters"] >= 0)
    assert ok.mean() >= 0.97
    with np.errstate(over="ignore"):
        m_gpu, m_ref = mse(r.Y.cpu().numpy(), Y), mse(o["Y"], Y)
    close = rel_close(m_gpu, m_ref, 1e-4)
    assert close[ok].mean() >= 0.9
    assert_no_systematic_loss(m_gpu, m_ref, ok & np.isfinite(m_gpu) & np.isfinite(m_ref) & ~close)
    assert (ok & ~np.isfinite(m_gpu) & np.isfinite(m_ref)).sum() <= (ok & np.isfinite(m_gpu) & ~np.isfinite(m_ref)).sum() + 20


@pytest.mark.parametrize("ls", ["strong_wolfe", "backtracking"])
def test_matches_oracle_kernel_arithmetic(golden, ls):
    """The oracle in the kernel's arithmetic, with the launch shape the library picks:
    every problem bit-identical at 25 iterations (constants, root values, loss,
    iterations, closures), and the reported loss is the MSE of the reported Y."""
    from parity import fit_bits_differ, oracle_fit_like
    sr = _sr()
    g = golden("optimize_ragged")
    mi = 25
    r = sr.optimize_ex(cuda(g["X"]), cuda(g["Y"]), cuda(g["ops"]), cuda(g["ch"]), cuda(g["C"]), max_iter=mi,
                       line_search_fn=ls, raise_errors=False)
    o = oracle_fit_like(r, g["X"], g["Y"], g["ops"], g["ch"], g["C"], max_iter=mi, line_search_fn=ls)
    assert not fit_bits_differ(r, o).any()
    it_gpu = r.iters.cpu().numpy()
    m = mse(r.Y.cpu().numpy(), g["Y"])
    fin = np.isfinite(m) & (it_gpu >= 0)
    np.testing.assert_allclose(r.loss.cpu().numpy()[fin], m[fin], rtol=1e-5, atol=1e-6)


def test_initial_closure_matches_oracle(golden):
    """max_iter=0: only the first closure runs; C is returned unchanged and the loss is
    the oracle's in the kernel's arithmetic, bit for bit."""
    from parity import oracle_fit_like
    sr = _sr()
    g = golden("optimize_ragged")
    r = sr.optimize_ex(cuda(g["X"]), cuda(g["Y"]), cuda(g["ops"]), cuda(g["ch"]), cuda(g["C"]), max_iter=0,
                       raise_errors=False)
    o = oracle_fit_like(r, g["X"], g["Y"], g["ops"], g["ch"], g["C"], max_iter=0)
    np.testing.assert_array_equal(r.C.cpu().numpy(), g["C"])
    np.testing.assert_array_equal(r.loss.cpu().numpy(), o["loss"])
    assert (r.iters.cpu().numpy() == 0).all()


def _rosenbrock_tape():
    """f = (1 - c0)^2 + 100 (c1 - c0^2)^2 as a postfix tape over two constants."""
    ops = [2, 1, 41, 14, 1, 14, 41, 14, 6, 6, 42, 5, 42, 42, 40]
    ch = [(-1, -1), (-1, -1), (0, 1), (2, -1), (-1, -1), (1, -1), (4, 5), (6, -1), (-1, -1), (-1, -1), (8, 9),
          (-1, -1), (10, 11), (12, 7), (3, 13)]
    return np.array(ops, np.int64), np.array(ch, np.int64)


@pytest.mark.parametrize("ls,key", [("strong_wolfe", "x_wolfe"), ("backtracking", "x_backtracking")])
def test_rosenbrock_known_answer(golden, ls, key):
    """reference tests/test_lbfgs_batch.py:38-75 through the raw-objective mode."""
    sr = _sr()
    g = golden("rosenbrock")
    x0 = g["x0"]  # (2, B)
    B = x0.shape[1]
    ops1, ch1 = _rosenbrock_tape()
    M = ops1.shape[0]
    ops = np.tile(ops1, (B, 1))
    ch = np.tile(ch1, (B, 1, 1))
    C = np.zeros((B, M), np.float32)
    C[:, 1] = x0[0]
    C[:, 4] = x0[1]
    X = np.zeros((1, 1), np.float32)
    r = sr.optimize_ex(cuda(X), None, cuda(ops), cuda(ch), cuda(C), max_iter=250, history_size=15,
                       line_search_fn=ls, objective=1)
    Cf = r.C.cpu().numpy()
    np.testing.assert_allclose(Cf[:, 1], 1.0, atol=1e-3)
    np.testing.assert_allclose(Cf[:, 4], 1.0, atol=1e-3)
    np.testing.assert_allclose(Cf[:, 1], g[key][0], atol=1e-3)
    np.testing.assert_allclose(Cf[:, 4], g[key][1], atol=1e-3)
    o = oracle.optimize(X, None, ops, ch, C, max_iter=250, history_size=15, line_search_fn=ls, dot_mode=1)
    np.testing.assert_allclose(Cf[:, [1, 4]], o["C"][:, [1, 4]], atol=1e-4)


def test_error_all_noop_row():
    """An all-NO_OP row sends a NaN gradient into a NO_OP node: error 201, as the reference."""
    sr = _sr()
    ops = torch.tensor([[50, 1, 40], [0, 0, 0]], dtype=torch.int64).cuda()
    ch = -torch.ones(2, 3, 2, dtype=torch.int64).cuda()
    ch[0, 2, 0], ch[0, 2, 1] = 0, 1
    X = torch.randn(10, 1).cuda()
    Y = torch.randn(2, 10).cuda()
    with pytest.raises(RuntimeError, match="A non-zero gradient was passed to a NO_OP node"):
        sr.optimize(X, Y, ops, ch, torch.zeros(2, 3).cuda())


def test_per_problem_error_reporting():
    """raise_errors=False: the offending problem reports -204, the others finish."""
    sr = _sr()
    ops = torch.tensor([[1, 50, 43], [1, 50, 40]], dtype=torch.int64).cuda()
    ch = -torch.ones(2, 3, 2, dtype=torch.int64).cuda()
    ch[:, 2, 0], ch[:, 2, 1] = 0, 1
    X = torch.linspace(-1, 1, 5).reshape(5, 1).cuda()
    Y = torch.ones(2, 5).cuda()
    r = sr.optimize_ex(X, Y, ops, ch, torch.ones(2, 3).cuda(), raise_errors=False)
    it = r.iters.cpu().tolist()
    assert it[0] == -204 and it[1] >= 0


def test_error_division_by_zero():
    sr = _sr()
    # C / X0 with X0 = 0 at one point
    ops = torch.tensor([[1, 50, 43]], dtype=torch.int64).cuda()
    ch = -torch.ones(1, 3, 2, dtype=torch.int64).cuda()
    ch[0, 2, 0], ch[0, 2, 1] = 0, 1
    X = torch.linspace(-1, 1, 5).reshape(5, 1).cuda()
    Y = torch.ones(1, 5).cuda()
    with pytest.raises(RuntimeError, match=r"Gradient for a/b where b = 0"):
        sr.optimize(X, Y, ops, ch, torch.ones(1, 3).cuda())


def test_validation_error_message():
    sr = _sr()
    ops = torch.tensor([[50, 40]], dtype=torch.int64).cuda()
    ch = -torch.ones(1, 2, 2, dtype=torch.int64).cuda()
    ch[0, 1, 0], ch[0, 1, 1] = 0, 1
    with pytest.raises(RuntimeError, match="Error during input validation: Validation failed: A child's index"):
        sr.optimize(torch.randn(4, 1).cuda(), torch.randn(1, 4).cuda(), ops, ch, torch.zeros(1, 2).cuda())


def test_nan_expression_poisons_every_slot():
    """A NaN gradient ends with all M slots NaN (0*NaN in the vector update), as in the reference."""
    sr = _sr()
    # log(C * X0) with X0 of both signs: NaN loss and NaN gradient
    ops = np.array([[1, 50, 42, 13, 0]], np.int64)
    ch = -np.ones((1, 5, 2), np.int64)
    ch[0, 2] = (0, 1)
    ch[0, 3, 0] = 2
    X = np.linspace(-2, 2, 9, dtype=np.float32).reshape(9, 1)
    Y = np.zeros((1, 9), np.float32)
    C = np.array([[0.7, 0, 0, 0, 0]], np.float32)
    r = sr.optimize_ex(cuda(X), cuda(Y), cuda(ops), cuda(ch), cuda(C), max_iter=5)
    o = oracle.optimize(X, Y, ops, ch, C, max_iter=5, dot_mode=0)
    assert np.isnan(o["C"]).all()
    assert np.isnan(r.C.cpu().numpy()).all()


def test_no_constants_and_determinism():
    from cudasymbolicregression_gb300 import tapes
    sr = _sr()
    rng = np.random.default_rng(3)
    B, M, N = 200, 24, 50
    X = rng.uniform(-3, 3, (N, 2)).astype(np.float32)
    C = rng.standard_normal((B, M)).astype(np.float32)
    kc = rng.integers(0, 4, size=B)
    tb = tapes.generate(B, M, seed=4, lengths=rng.integers(1, M + 1, size=B), const_counts=kc, n_vars=2,
                        X_screen=X, C_screen=C)
    Y = rng.standard_normal((B, N)).astype(np.float32)
    args = (cuda(X), cuda(Y), cuda(tb.ops), cuda(tb.ch), cuda(C))
    r1 = sr.optimize_ex(*args, max_iter=30)
    r2 = sr.optimize_ex(*args, max_iter=30)
    for a, b in ((r1.C, r2.C), (r1.Y, r2.Y), (r1.iters, r2.iters)):
        assert torch.equal(torch.nan_to_num(a, nan=7.0), torch.nan_to_num(b, nan=7.0))
    nc = tb.n_consts == 0
    Cf = r1.C.cpu().numpy()
    np.testing.assert_array_equal(Cf[nc], C[nc])
    assert (r1.iters.cpu().numpy()[nc] == 0).all()
    # a problem's result does not depend on the rest of the batch
    sub = np.where(~nc)[0][:5]
    rs = sr.optimize_ex(cuda(X), cuda(Y[sub]), cuda(tb.ops[sub]), cuda(tb.ch[sub]), cuda(C[sub]), max_iter=30)
    assert torch.equal(torch.nan_to_num(rs.C, nan=7.0), torch.nan_to_num(r1.C[torch.as_tensor(sub).cuda()], nan=7.0))


@pytest.mark.parametrize("ppl,wpb", [(1, 1), (2, 4), (4, 2), (1, 8)])
def test_kernel_shapes_agree(golden, ppl, wpb):
    """Every launch shape the autotuner may pick gives the same answers."""
    sr = _sr()
    g = golden("optimize_readme")
    base = sr.optimize_ex(cuda(g["X"]), cuda(g["Y"]), cuda(g["ops"]), cuda(g["ch"]), cuda(g["C"]), max_iter=20,
                          raise_errors=False)
    r = sr.optimize_ex(cuda(g["X"]), cuda(g["Y"]), cuda(g["ops"]), cuda(g["ch"]), cuda(g["C"]), max_iter=20,
                       points_per_lane=ppl, warps_per_block=wpb, raise_errors=False)
    close = rel_close(mse(r.Y.cpu().numpy(), g["Y"]), mse(base.Y.cpu().numpy(), g["Y"]), 1e-4)
    assert close.mean() >= 0.9


def test_fit_plan_and_cuda_graph_replay(golden):
    """FitPlan: the same results as optimize_ex, and a captured CUDA graph replays the
    fit from new starting constants with identical results to a direct run."""
    sr = _sr()
    g = golden("optimize_ragged")
    X, Y, ops, ch = cuda(g["X"]), cuda(g["Y"]), cuda(g["ops"]), cuda(g["ch"])
    C0 = cuda(g["C"])
    ref = sr.optimize_ex(X, Y, ops, ch, C0, max_iter=25, raise_errors=False)
    plan = sr.FitPlan(X, Y, ops, ch, max_iter=25)
    plan.C_in.copy_(C0)
    plan.run()
    r = plan.result(raise_errors=False)
    for a, b in ((r.C, ref.C), (r.Y, ref.Y), (r.loss, ref.loss)):
        assert torch.equal(torch.nan_to_num(a, nan=9.0), torch.nan_to_num(b, nan=9.0))
    assert torch.equal(r.iters, ref.iters) and torch.equal(r.evals, ref.evals)
    graph = plan.capture()
    C1 = C0 + 0.25
    ref1 = sr.optimize_ex(X, Y, ops, ch, C1, max_iter=25, raise_errors=False)
    plan.C_in.copy_(C1)
    graph.replay()
    r1 = plan.result(raise_errors=False)
    assert torch.equal(torch.nan_to_num(r1.C, nan=9.0), torch.nan_to_num(ref1.C, nan=9.0))
    assert torch.equal(r1.iters, ref1.iters)


def test_autotune_picks_a_shape_and_matches_it(golden):
    sr = _sr()
    from cudasymbolicregression_gb300 import optimization
    g = golden("optimize_ragged")
    X, Y, ops, ch, C = cuda(g["X"]), cuda(g["Y"]), cuda(g["ops"]), cuda(g["ch"]), cuda(g["C"])
    r = sr.optimize_ex(X, Y, ops, ch, C, max_iter=20, raise_errors=False, autotune=True)
    assert len(optimization._TUNED) >= 1
    V, W = list(optimization._TUNED.values())[-1]
    assert (V, W) in optimization._TUNE_CANDIDATES
    r2 = sr.optimize_ex(X, Y, ops, ch, C, max_iter=20, raise_errors=False, points_per_lane=V, warps_per_block=W)
    assert torch.equal(torch.nan_to_num(r.C, nan=9.0), torch.nan_to_num(r2.C, nan=9.0))


def _root_values(sr, X, ops, ch, C):
    with torch.no_grad():
        cache = sr.evaluation.evaluate(X, ops, ch, C)
        root = ((ops != 0).sum(1) - 1).clamp(min=0)
        return cache[torch.arange(ops.shape[0], device=ops.device), root]


def test_large_batch_sine_fit():
    """The reference's large-batch scenario (tests/test_optimization.py:82-169):
    10000 problems y = c1 sin(X0) + c2 with their own true constants, fitted from
    randn constants; the MSE must drop at least tenfold."""
    sr = _sr()
    from cudasymbolicregression_gb300.operators import Operator as Op
    torch.manual_seed(3)
    B, N, M = 10000, 50, 6
    c1, c2 = torch.randn(B, 1).cuda() * 2, torch.randn(B, 1).cuda()
    X = (torch.rand(N, 1) * 4 - 2).cuda()
    Y = c1 * torch.sin(X[:, 0])[None, :] + c2
    row = [int(Op.VAR_START_ID), int(Op.SIN), int(Op.LEARNABLE_CONSTANT), int(Op.MUL), int(Op.LEARNABLE_CONSTANT),
           int(Op.ADD)]
    ops = torch.tensor(row).repeat(B, 1).cuda()
    ch = torch.full((B, M, 2), -1, dtype=torch.int64).cuda()
    ch[:, 1, 0] = 0
    ch[:, 3, 0], ch[:, 3, 1] = 1, 2
    ch[:, 5, 0], ch[:, 5, 1] = 3, 4
    C0 = sr.create_constants(ops)
    _, Yf = sr.optimize(X, Y, ops, ch, C0)
    init = ((_root_values(sr, X, ops, ch, C0) - Y) ** 2).mean()
    final = ((Yf - Y) ** 2).mean()
    assert final < 0.1 * init


def test_large_noisy_fit_recovers_signal():
    """The reference's noisy scenario (tests/test_optimization.py:171-279): 10000
    problems c1 sin(X0 + c2) + c3 log((X1 X2 + c4)^2) + 5% noise, max_iter=300; the
    fit must move towards the noiseless signal.

    With a small c3 the log singularity can fit one noisy point: the fit drives
    X1 X2 + c4 towards 0 at that point until it is exactly 0 in float32 and the loss
    is NaN.  The oracle in the reference's float32 arithmetic ends so on 1 to 3 of
    10000 problems of this kind (which ones depends on rounding), so the MSE is taken
    over the finite fits and at most 0.1% may be non-finite.  From randn starting
    constants many fits end in a local minimum (the sine's phase, the log's shift):
    the oracle's mean MSE against the signal falls from 29.9 to 13.4 on such a batch,
    so the bound is a relative one (the reference test's absolute 0.1 is not met by
    its own float32 algorithm on this data)."""
    sr = _sr()
    from cudasymbolicregression_gb300.operators import Operator as Op
    torch.manual_seed(4)
    B, N, M = 10000, 100, 16
    c1, c2, c3 = torch.randn(B, 1).cuda(), torch.randn(B, 1).cuda(), torch.randn(B, 1).cuda()
    c4 = torch.randn(B, 1).cuda() + 10.0
    X = (torch.randn(N, 4) * 2).cuda()
    Y_true = c1 * torch.sin(X[:, 0][None] + c2) + c3 * torch.log(torch.square(X[:, 1][None] * X[:, 2][None] + c4))
    Y = Y_true + torch.randn_like(Y_true) * 0.05 * Y_true.std()
    V, K = int(Op.VAR_START_ID), int(Op.LEARNABLE_CONSTANT)
    row = [K, V, K, int(Op.ADD), int(Op.SIN), int(Op.MUL), K, V + 1, V + 2, int(Op.MUL), K, int(Op.ADD),
           int(Op.SQUARE), int(Op.LOG), int(Op.MUL), int(Op.ADD)]
    ops = torch.tensor(row).repeat(B, 1).cuda()
    ch = torch.full((B, M, 2), -1, dtype=torch.int64).cuda()
    for k, (a, b) in {3: (1, 2), 4: (3, -1), 5: (0, 4), 9: (7, 8), 11: (9, 10), 12: (11, -1), 13: (12, -1),
                      14: (6, 13), 15: (5, 14)}.items():
        ch[:, k, 0], ch[:, k, 1] = a, b
    C0 = sr.create_constants(ops)
    _, Yf = sr.optimize(X, Y, ops, ch, C0, line_search_fn="strong_wolfe", max_iter=300)
    ok = torch.isfinite(Yf).all(1)
    assert int((~ok).sum()) <= B // 1000
    init = ((_root_values(sr, X, ops, ch, C0)[ok] - Y_true[ok]) ** 2).mean()
    final = ((Yf[ok] - Y_true[ok]) ** 2).mean()
    assert final < 0.6 * init


def test_screen_starts_match_the_first_closure(golden):
    """Multi-start screening (one launch, forward passes only) reports for every
    candidate start the loss the fit's first closure reports from it, NaN where it is
    NaN; the screened start is the candidate with the lowest loss, the plain start on
    ties."""
    from cudasymbolicregression_gb300 import warmstart
    from cudasymbolicregression_gb300.optimization import screen_starts
    sr = _sr()
    g = golden("optimize_ragged")
    X, Y, O, Ch, C = cuda(g["X"]), cuda(g["Y"]), cuda(g["ops"]), cuda(g["ch"]), cuda(g["C"])
    gen = torch.Generator(device="cuda").manual_seed(3)
    Cs = warmstart.candidate_starts(X, Y, O, C, None, 3, generator=gen)
    loss = screen_starts(X, Y, O, Ch, Cs).cpu().numpy()
    for k in range(Cs.shape[0]):
        first = sr.optimize_ex(X, Y, O, Ch, Cs[k], max_iter=0, raise_errors=False, want_y=False).loss.cpu().numpy()
        assert rel_close(loss[:, k], first, 1e-6).all()
    pick = warmstart.screened_start(X, Y, O, Ch, Cs)
    lf = np.where(np.isfinite(loss), loss, np.inf)
    best = np.argmin(lf, axis=1)
    np.testing.assert_array_equal(pick.cpu().numpy(), Cs.cpu().numpy()[best, np.arange(len(best))])
    with pytest.raises(RuntimeError, match="C_sets must be"):
        screen_starts(X, Y, O, Ch, Cs[:, :5])


def test_tape_longer_than_the_launch_is_reported_not_fitted(golden):
    """A C-ABI caller that passes a max_len below a tape's root + 1 (or a max_consts
    below its constants) gets that problem skipped with status 602 and iters -602,
    its C_out = C_init and its loss NaN; the other problems are fitted as usual."""
    import ctypes
    from cudasymbolicregression_gb300 import _lib
    from cudasymbolicregression_gb300.tape import compile_tapes
    g = golden("optimize_ragged")
    X, Y, O, Ch, C = cuda(g["X"]), cuda(g["Y"]), cuda(g["ops"]), cuda(g["ch"]), cuda(g["C"])
    tp = compile_tapes(O, Ch, X.shape[1])
    L = _lib.lib()
    B, M = tp.B, tp.M
    N, nx = X.shape
    roots = tp.meta[:, 1].cpu().numpy() + 1
    kc = tp.meta[:, 2].cpu().numpy()
    for max_len, max_consts in ((tp.max_root - 1, tp.max_consts), (tp.max_root, max(tp.max_consts - 1, 0))):
        opts = _lib.FitOptions(max_iter=10, history_size=10, tolerance_grad=1e-7, line_search=0,
                               line_search_max_iter=10, eps=1e-10, max_operators=0)
        wsb = L.sr_fit_workspace_bytes(B, N, M, tp.max_root, tp.max_consts, ctypes.byref(opts))
        ws = torch.empty(int(wsb), dtype=torch.uint8, device="cuda")
        Cout, Yf = torch.empty(B, M, device="cuda"), torch.empty(B, N, device="cuda")
        it, loss = torch.empty(B, dtype=torch.int32, device="cuda"), torch.empty(B, device="cuda")
        ev, st = torch.empty(B, dtype=torch.int32, device="cuda"), torch.zeros(1, dtype=torch.int32, device="cuda")
        rc = L.sr_fit_lbfgs(_lib.ptr(X), N, nx, _lib.ptr(Y), _lib.ptr(tp.desc), _lib.ptr(tp.meta), B, M, _lib.ptr(C),
                            _lib.ptr(Cout), M, 1, _lib.ptr(Yf), _lib.ptr(it), _lib.ptr(loss), _lib.ptr(ev), None,
                            max_len, max_consts, ctypes.byref(opts), _lib.ptr(ws), ws.numel(), _lib.ptr(st),
                            _lib.stream_ptr(X.device))
        _lib.check(rc, "sr_fit_lbfgs")
        torch.cuda.synchronize()
        over = (roots > max_len) | (kc > max_consts)
        assert over.any() and int(st.item()) == _lib.TAPE_EXCEEDS_LAUNCH
        itn = it.cpu().numpy()
        assert (itn[over] == -_lib.TAPE_EXCEEDS_LAUNCH).all() and (itn[~over] >= -204).all()
        assert (itn[~over] != -_lib.TAPE_EXCEEDS_LAUNCH).all()
        np.testing.assert_array_equal(Cout.cpu().numpy()[over], g["C"][over])
        assert np.isnan(loss.cpu().numpy()[over]).all()


def _live_rows(ops, ch):
    """Restatement of the fit kernel's liveness assignment count for one tape: a row is
    taken at the first parent's sweep (the root's from the start, a node without a
    parent at its own sweep) and freed after the node's own sweep."""
    root = max(int((ops != 0).sum()) - 1, 0)
    isop = lambda k: ops[k] == 0 or 10 <= ops[k] <= 31 or 40 <= ops[k] <= 44  # noqa: E731
    held, cur, best = set(), 0, 0
    if isop(root):
        held.add(root)
        cur = best = 1
    for k in range(root, -1, -1):
        if not isop(k):
            continue
        if k not in held:
            held.add(k)
            cur += 1
            best = max(best, cur)
        cur -= 1
        ar = 1 if 10 <= ops[k] <= 31 else (2 if 40 <= ops[k] <= 44 else 0)
        for c in ch[k][:ar]:
            if isop(c) and c not in held:
                held.add(c)
                cur += 1
                best = max(best, cur)
    return best


def test_live_adjoint_rows_and_their_limit():
    """sr_tape_live_rows counts the rows the fit's liveness assignment needs (here
    against a restatement, with a shared child and an operator node no root uses); the
    fit gives the same bits with rows for every operator node (max_live = 0) as with
    the counted number, and with one row too few the tapes that need them all report
    602 while every other problem is fitted as before."""
    import ctypes
    from cudasymbolicregression_gb300 import _lib, tapes
    from cudasymbolicregression_gb300.tape import compile_tapes
    rng = np.random.default_rng(12)
    B, M, N = 300, 40, 70
    X = rng.uniform(-2, 2, (N, 2)).astype(np.float32)
    C = rng.standard_normal((B, M)).astype(np.float32)
    tb = tapes.generate(B, M, seed=13, lengths=rng.integers(1, M + 1, size=B), const_counts=rng.integers(0, 5, size=B),
                        n_vars=2, X_screen=X, C_screen=C)
    ops, ch = tb.ops.copy(), tb.ch.copy()
    # tape 0: C, sin(C) (no parent: the root does not use it), C, cos(2), cos(3) * cos(3) (a shared child)
    ops[0] = 0
    ch[0] = -1
    ops[0, :6] = [1, 10, 1, 11, 11, 42]
    ch[0, 1, 0], ch[0, 3, 0], ch[0, 4, 0] = 0, 2, 3
    ch[0, 5] = (4, 4)
    Y = rng.standard_normal((B, N)).astype(np.float32)
    X_, Y_, O_, Ch_, C_ = (cuda(a) for a in (X, Y, ops, ch, C))
    tp = compile_tapes(O_, Ch_, 2, live=True)
    want = [_live_rows(ops[b], ch[b]) for b in range(B)]
    assert tp.max_live == max(want)
    L = _lib.lib()

    def fit(max_live):
        o = _lib.FitOptions(max_iter=30, history_size=10, tolerance_grad=1e-7, line_search=0, line_search_max_iter=10,
                            eps=1e-10, max_operators=tp.max_operators, max_live=max_live)
        wsb = L.sr_fit_workspace_bytes(B, N, M, tp.max_root, tp.max_consts, ctypes.byref(o))
        ws = torch.empty(int(wsb), dtype=torch.uint8, device="cuda")
        Co, Yf = torch.empty(B, M, device="cuda"), torch.empty(B, N, device="cuda")
        it, ls, ev = (torch.empty(B, dtype=torch.int32, device="cuda"), torch.empty(B, device="cuda"),
                      torch.empty(B, dtype=torch.int32, device="cuda"))
        st = torch.zeros(1, dtype=torch.int32, device="cuda")
        _lib.check(L.sr_fit_lbfgs(_lib.ptr(X_), N, 2, _lib.ptr(Y_), _lib.ptr(tp.desc), _lib.ptr(tp.meta), B, M,
                                  _lib.ptr(C_), _lib.ptr(Co), M, 1, _lib.ptr(Yf), _lib.ptr(it), _lib.ptr(ls), _lib.ptr(ev),
                                  None, tp.max_root, tp.max_consts, ctypes.byref(o), _lib.ptr(ws), ws.numel(),
                                  _lib.ptr(st), _lib.stream_ptr(X_.device)), "sr_fit_lbfgs")
        torch.cuda.synchronize()
        return [t.cpu().numpy() for t in (Co, Yf, it, ls, ev, st)]

    every = fit(0)
    counted = fit(tp.max_live)
    for a, b in zip(every[:5], counted[:5]):
        np.testing.assert_array_equal(np.nan_to_num(a, nan=7.0), np.nan_to_num(b, nan=7.0))
    short = fit(tp.max_live - 1)
    over = np.array(want) > tp.max_live - 1
    assert over.any() and (~over).any() and short[5][0] == _lib.TAPE_EXCEEDS_LAUNCH
    assert (short[2][over] == -_lib.TAPE_EXCEEDS_LAUNCH).all()
    for a, b in zip(short[:5], counted[:5]):
        np.testing.assert_array_equal(np.nan_to_num(a[~over], nan=7.0), np.nan_to_num(b[~over], nan=7.0))


def test_shards_fitted_with_the_batch_launch_shape_equal_the_whole_fit():
    """sharding.fit_shard, the per-rank part of fit_sharded: each slice of a batch fitted
    alone with the whole batch's launch shape and constant-slot layout gives every
    problem the bits of the whole fit (constants, root values, loss, iterations).  The
    batch is chosen so that a slice left to itself gets another shape: 1200 problems
    at N = 200 run 4 warps each, 600 would run 8, and only the first half has a tape
    with 40 constants (two slot registers per lane)."""
    from cudasymbolicregression_gb300 import sharding, tapes
    from cudasymbolicregression_gb300.operators import Operator as Op
    sr = _sr()
    rng = np.random.default_rng(71)
    B, M, N = 1200, 96, 200
    exact_bin = (int(Op.ADD), int(Op.SUB), int(Op.MUL), int(Op.DIV))
    X = rng.uniform(-3, 3, (N, 2)).astype(np.float32)
    C = rng.standard_normal((B, M)).astype(np.float32)
    consts = rng.integers(0, 5, size=B)
    lens = rng.integers(3, 40, size=B)
    consts[7], lens[7] = 40, 96
    tb = tapes.generate(B, M, seed=72, lengths=lens, const_counts=consts, n_vars=2, binary=exact_bin,
                        unary=(int(Op.SQUARE), int(Op.NEG)), X_screen=X, C_screen=C)
    Y = (np.sin(X[:, 0]) * X[:, 1]).astype(np.float32)[None, :] + 0.1 * rng.standard_normal((B, N)).astype(np.float32)
    Xd, Yd, Od, Chd, Cd = (cuda(a) for a in (X, Y, tb.ops, tb.ch, C))
    kw = dict(max_iter=60, raise_errors=False)
    whole = sr.optimize_ex(Xd, Yd, Od, Chd, Cd, **kw)
    pin = sr.optimization.batch_launch_shape(Xd, Od, Chd)
    assert pin["warps_per_block"] == 4 and pin["consts_floor"] >= 32
    parts, alone = [], []
    for start, stop in (sharding.shard_range(B, r, 2) for r in range(2)):
        parts.append(sharding.fit_shard(Xd, Yd, Od, Chd, Cd, start, stop, **kw))
        alone.append(sr.optimize_ex(Xd, Yd[start:stop], Od[start:stop], Chd[start:stop], Cd[start:stop], **kw))
    Cs = torch.cat([p[0] for p in parts]).cpu().numpy()
    Ys = torch.cat([p[1] for p in parts]).cpu().numpy()

    def bits(a):
        a = np.ascontiguousarray(a, np.float32)
        return np.where(np.isnan(a), np.uint32(0x7fc00000), a.view(np.uint32))
    assert np.array_equal(bits(Cs), bits(whole.C.cpu().numpy()))
    assert np.array_equal(bits(Ys), bits(whole.Y.cpu().numpy()))
    # left to itself the second half runs 8 warps per problem and one slot register
    assert alone[1].shapes[0][2] == 8 and whole.shapes[0][2] == 4
    C_alone = torch.cat([a.C for a in alone]).cpu().numpy()
    assert not np.array_equal(bits(C_alone), bits(whole.C.cpu().numpy()))
