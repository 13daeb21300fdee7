"""GPU parity of evaluate / evaluate_backend and their adjoint.

Checked against (a) the reference's own outputs (tests/golden, written from the
reference's CPU path) and (b) the CPU oracle on seeded tapes.  Criteria
(oracle/parity.py): every node recomputed by the oracle from the device's own
child values agrees bit for bit for IEEE-exact operations and within a few ulps
for transcendental ones, with identical NaN placement; whole-tape values and
gradients are within 1e-5 relative of the reference's float32 result for
>= 99.9% / 99% of the entries and no less accurate against the FP64 oracle
(CUDA's and glibc's transcendentals differ by a few ulps, which cancellation
along a tape can amplify).  Operations one level deep are compared directly
at 1e-5 with identical NaN placement.
"""
import numpy as np
import pytest
import torch

import oracle
from parity import check_accuracy, check_local

pytestmark = pytest.mark.gpu

RTOL = 1e-5


def _sr():
    import cudasymbolicregression_gb300 as sr
    return sr


def assert_close_nan(mine, ref, rtol=RTOL, atol_scale=1e-5):
    mine = np.asarray(mine)
    ref = np.asarray(ref)
    assert mine.shape == ref.shape
    nan_m, nan_r = np.isnan(mine), np.isnan(ref)
    assert np.array_equal(nan_m, nan_r), f"NaN placement differs at {np.argwhere(nan_m != nan_r)[:5]}"
    fin = np.isfinite(ref) & np.isfinite(mine)
    inf_ok = np.array_equal(np.isinf(mine), np.isinf(ref))
    assert inf_ok, "inf placement differs"
    if fin.any():
        d = np.abs(mine[fin].astype(np.float64) - ref[fin].astype(np.float64))
        tol = rtol * np.abs(ref[fin].astype(np.float64)) + atol_scale
        bad = d > tol
        assert not bad.any(), f"max rel err {np.max(d / np.maximum(np.abs(ref[fin]), 1e-30))}, {bad.sum()} entries"


def cuda(a, dtype=None):
    t = torch.as_tensor(np.ascontiguousarray(a))
    if dtype is not None:
        t = t.to(dtype)
    return t.cuda()


@pytest.mark.parametrize("name", ["single_ops", "random_dags", "random_default_ops"])
def test_forward_vs_reference_golden(golden, name):
    """Node by node against the oracle from the device's own children (exact
    operations bit for bit), and no less accurate than the reference's float32
    result against the FP64 oracle."""
    sr = _sr()
    g = golden(name)
    out = sr.evaluation.evaluate(cuda(g["X"]), cuda(g["ops"]), cuda(g["ch"]), cuda(g["C"]))
    assert out.shape == g["cache"].shape
    got = out.cpu().numpy()
    check_local(g["X"], g["ops"], g["ch"], g["C"], got)
    ref64 = oracle.eval_fwd(g["X"], g["ops"], g["ch"], g["C"], dtype=np.float64)
    check_accuracy(got, g["cache"], ref64)
    if name == "single_ops":  # one operation deep: no error amplification
        assert_close_nan(got, g["cache"])


@pytest.mark.parametrize("name", ["single_ops", "random_dags", "random_default_ops"])
def test_backward_vs_reference_golden(golden, name):
    sr = _sr()
    g = golden(name)
    X = cuda(g["X"]).requires_grad_(True)
    C = cuda(g["C"]).requires_grad_(True)
    out = sr.evaluation.evaluate(X, cuda(g["ops"]), cuda(g["ch"]), C)
    out.backward(cuda(g["gout"]))
    gC64, gX64, err = oracle.eval_bwd(g["X"], g["ops"], g["ch"], g["C"], g["gout"], dtype=np.float64)
    check_accuracy(C.grad.cpu().numpy(), g["gC"], gC64, rtol=1e-5, atol=1e-5, min_frac_tight=0.99)
    # gX is an atomic sum over the tapes (in the reference too): where the fixture holds
    # the per-tape contributions, errors are measured against their absolute sum
    scale = np.abs(g["gX_rows"]).sum(0) if "gX_rows" in g.files else None
    check_accuracy(X.grad.cpu().numpy(), g["gX"], gX64, rtol=1e-4, atol=1e-4, min_frac_tight=0.9, abs_scale=scale)
    if name == "single_ops":
        assert_close_nan(C.grad.cpu().numpy(), g["gC"], rtol=1e-5, atol_scale=1e-5)


def test_evaluate_backend_layout(golden):
    """M-first entry point: (M, B) inputs, (M, N, B) output (reference src/symbolic_evaluation.cpp:306)."""
    sr = _sr()
    g = golden("random_dags")
    ops = cuda(g["ops"]).permute(1, 0)
    ch = cuda(g["ch"]).permute(1, 0, 2)
    C = cuda(g["C"]).permute(1, 0)
    out = sr.evaluation.evaluate_backend(cuda(g["X"]), ops, ch, C)
    assert out.shape == (g["ops"].shape[1], g["X"].shape[0], g["ops"].shape[0])
    direct = sr.evaluation.evaluate(cuda(g["X"]), cuda(g["ops"]), cuda(g["ch"]), cuda(g["C"]))
    assert torch.equal(torch.nan_to_num(out.permute(2, 0, 1), nan=3.0), torch.nan_to_num(direct, nan=3.0))


@pytest.mark.parametrize("seed,B,M,N,nx", [(1, 300, 40, 45, 3), (2, 64, 64, 1000, 4), (3, 7, 5, 1, 1),
                                             (4, 33, 17, 129, 2)])
def test_forward_backward_vs_oracle(seed, B, M, N, nx):
    from cudasymbolicregression_gb300 import tapes
    from cudasymbolicregression_gb300.operators import BINARY_OPS, UNARY_OPS
    sr = _sr()
    rng = np.random.default_rng(seed)
    X = rng.uniform(-3, 3, (N, nx)).astype(np.float32)
    C = rng.standard_normal((B, M)).astype(np.float32)
    tb = tapes.generate(B, M, seed=seed, mean_length=M / 3, n_vars=nx, unary=UNARY_OPS, binary=BINARY_OPS,
                        X_screen=X, C_screen=C)
    ref = oracle.eval_fwd(X, tb.ops, tb.ch, C)
    ref64 = oracle.eval_fwd(X, tb.ops, tb.ch, C, dtype=np.float64)
    Xt = cuda(X).requires_grad_(True)
    Ct = cuda(C).requires_grad_(True)
    out = sr.evaluation.evaluate(Xt, cuda(tb.ops), cuda(tb.ch), Ct)
    got = out.detach().cpu().numpy()
    check_local(X, tb.ops, tb.ch, C, got)
    check_accuracy(got, ref, ref64)
    gout = rng.standard_normal(ref.shape).astype(np.float32)
    gout[np.isnan(got) | np.isnan(ref)] = 0.0
    gC, gX, err = oracle.eval_bwd(X, tb.ops, tb.ch, C, gout)
    if err:
        pytest.skip("seeded tapes hit a zero denominator")
    gC64, gX64, _ = oracle.eval_bwd(X, tb.ops, tb.ch, C, gout, dtype=np.float64)
    out.backward(cuda(gout))
    check_accuracy(Ct.grad.cpu().numpy(), gC, gC64, rtol=1e-5, atol=1e-5, min_frac_tight=0.99)
    check_accuracy(Xt.grad.cpu().numpy(), gX, gX64, rtol=1e-4, atol=1e-4, min_frac_tight=0.9)


def test_float64_matches_oracle():
    from cudasymbolicregression_gb300 import tapes
    from cudasymbolicregression_gb300.operators import BINARY_OPS, UNARY_OPS
    sr = _sr()
    rng = np.random.default_rng(9)
    B, M, N, nx = 100, 30, 77, 2
    X = rng.uniform(-3, 3, (N, nx))
    C = rng.standard_normal((B, M))
    tb = tapes.generate(B, M, seed=9, mean_length=10, n_vars=nx, unary=UNARY_OPS, binary=BINARY_OPS)
    ref = oracle.eval_fwd(X, tb.ops, tb.ch, C, dtype=np.float64)
    Ct = cuda(C, torch.float64).requires_grad_(True)
    out = sr.evaluation.evaluate(cuda(X, torch.float64), cuda(tb.ops), cuda(tb.ch), Ct)
    assert out.dtype == torch.float64
    got = out.detach().cpu().numpy()
    assert np.array_equal(np.isnan(got), np.isnan(ref))
    fin = np.isfinite(ref)
    close = np.abs(got[fin] - ref[fin]) <= 1e-9 * np.abs(ref[fin]) + 1e-12
    assert close.mean() >= 0.999
    gout = rng.standard_normal(ref.shape)
    gout[np.isnan(ref)] = 0.0
    gC, _, err = oracle.eval_bwd(X, tb.ops, tb.ch, C, gout, dtype=np.float64)
    if err:
        pytest.skip("seeded tapes hit a zero denominator")
    out.backward(cuda(gout, torch.float64))
    g = Ct.grad.cpu().numpy()
    assert np.array_equal(np.isnan(g), np.isnan(gC))
    fin = np.isfinite(gC)
    assert (np.abs(g[fin] - gC[fin]) <= 1e-8 * np.abs(gC[fin]) + 1e-10).mean() >= 0.995


def test_constants_known_answers():
    """reference tests/test_symbolic_evaluation.py:435-478: C=3.14 -> 4.14, sin(3.14)."""
    sr = _sr()
    X = torch.randn(4, 1).cuda()
    ops = torch.tensor([[1], [2], [40]], dtype=torch.int64).cuda()
    ch = -torch.ones(3, 1, 2, dtype=torch.int64).cuda()
    ch[2, 0, 0] = 0
    ch[2, 0, 1] = 1
    C = torch.zeros(3, 1).cuda()
    C[0, 0] = 3.14
    y = sr.evaluation.evaluate_backend(X, ops, ch, C)
    assert torch.allclose(y[2, :, 0], torch.full((4,), 4.14, device="cuda"), atol=1e-6)
    ops = torch.tensor([[1], [10]], dtype=torch.int64).cuda()
    ch = -torch.ones(2, 1, 2, dtype=torch.int64).cuda()
    ch[1, 0, 0] = 0
    C = torch.zeros(2, 1).cuda()
    C[0, 0] = 3.14
    y = sr.evaluation.evaluate_backend(X, ops, ch, C)
    assert torch.allclose(y[1, :, 0], torch.sin(torch.tensor(3.14)).cuda().expand(4), atol=1e-6)


def test_noop_nan_and_zero_grads():
    """reference tests/test_symbolic_evaluation.py:192-217."""
    sr = _sr()
    X = torch.randn(10, 2).cuda().requires_grad_(True)
    ops = torch.tensor([[0]], dtype=torch.int64).cuda()
    ch = -torch.ones(1, 1, 2, dtype=torch.int64).cuda()
    C = torch.zeros(1, 1).cuda().requires_grad_(True)
    y = sr.evaluation.evaluate_backend(X, ops, ch, C)
    assert torch.isnan(y).all()
    y[-1].backward(torch.zeros(10, 1).cuda())
    assert torch.all(X.grad == 0) and torch.all(C.grad == 0)


def test_validation_errors(golden):
    sr = _sr()
    g = golden("errors")
    for name in ("child_geq", "unary_nochild", "binary_onechild", "leaf_child"):
        ops, ch = cuda(g[name + "__ops"]), cuda(g[name + "__ch"])
        X = cuda(g[name + "__X"])
        C = torch.zeros(ops.shape, device="cuda")
        with pytest.raises(RuntimeError) as e:
            sr.evaluation.evaluate(X, ops, ch, C)
        assert str(e.value) == str(g[name + "__msg"])


def test_backward_errors(golden):
    sr = _sr()
    g = golden("errors")
    for name in ("noop_grad", "div_zero"):
        ops, ch = cuda(g[name + "__ops"]), cuda(g[name + "__ch"])
        X = cuda(g[name + "__X"]).requires_grad_(True)
        C = torch.zeros(ops.shape, device="cuda").requires_grad_(True)
        y = sr.evaluation.evaluate(X, ops, ch, C)
        gout = torch.zeros_like(y)
        gout[:, -1, :] = 1.0
        with pytest.raises(RuntimeError) as e:
            y.backward(gout)
        assert str(g[name + "__msg"]) in str(e.value)


def test_backward_error_precedence():
    """A gradient on a padding (NO_OP) row is reported as 201 even when other tapes of
    the batch meet a zero denominator (204): the padding check and the adjoint run
    concurrently, and 201 takes precedence whichever finds its error first."""
    sr = _sr()
    B, M, N = 4096, 8, 256
    ops = torch.zeros(B, M, dtype=torch.int64)
    ch = -torch.ones(B, M, 2, dtype=torch.int64)
    ops[:, 0], ops[:, 1], ops[:, 2] = 1, 50, 43  # C / X0
    ch[:, 2, 0], ch[:, 2, 1] = 0, 1
    X = torch.linspace(-1, 1, N).reshape(N, 1)
    X[N // 2] = 0.0
    ops, ch, X = ops.cuda(), ch.cuda(), X.cuda()
    for culprit in (0, B // 2, B - 1):
        C = torch.ones(B, M, device="cuda").requires_grad_(True)
        y = sr.evaluation.evaluate(X, ops, ch, C)
        gout = torch.zeros_like(y)
        gout[:, 2, :] = 1.0                      # every tape: a/b with b = 0 at one point
        gout[culprit, M - 1, 3] = 1.0            # one tape: a gradient on a padding row
        with pytest.raises(RuntimeError, match="A non-zero gradient was passed to a NO_OP node"):
            y.backward(gout)
    C = torch.ones(B, M, device="cuda").requires_grad_(True)
    y = sr.evaluation.evaluate(X, ops, ch, C)
    gout = torch.zeros_like(y)
    gout[:, 2, :] = 1.0
    with pytest.raises(RuntimeError, match=r"Gradient for a/b where b = 0"):
        y.backward(gout)


def test_ragged_batch_and_padding_rows():
    """Ragged tapes: rows after the last real node are NaN, NO_OP inside a tape is NaN."""
    sr = _sr()
    V = 50
    ops = torch.tensor([[V, V + 1, 40, 0, 0], [V, 10, 0, 0, 0], [V, 0, 0, 0, 0]], dtype=torch.int64).cuda()
    ch = -torch.ones(3, 5, 2, dtype=torch.int64).cuda()
    ch[0, 2, 0], ch[0, 2, 1], ch[1, 1, 0] = 0, 1, 0
    X = torch.randn(70, 2).cuda()
    y = sr.evaluation.evaluate(X, ops, ch, torch.zeros(3, 5).cuda())
    assert torch.equal(y[0, 2], X[:, 0] + X[:, 1])
    assert torch.equal(y[1, 1], torch.sin(X[:, 0])) or torch.allclose(y[1, 1], torch.sin(X[:, 0]), atol=1e-6)
    assert torch.isnan(y[0, 3:]).all() and torch.isnan(y[1, 2:]).all() and torch.isnan(y[2, 1:]).all()


def test_empty_inputs():
    sr = _sr()
    X = torch.randn(5, 1).cuda()
    y = sr.evaluation.evaluate(X, torch.zeros(0, 3, dtype=torch.int64).cuda(),
                               -torch.ones(0, 3, 2, dtype=torch.int64).cuda(), torch.zeros(0, 3).cuda())
    assert y.shape == (0, 3, 5)
    y = sr.evaluation.evaluate(torch.randn(0, 1).cuda(), torch.full((2, 1), 50, dtype=torch.int64).cuda(),
                               -torch.ones(2, 1, 2, dtype=torch.int64).cuda(), torch.zeros(2, 1).cuda())
    assert y.shape == (2, 1, 0)


def test_create_constants_rng_stream():
    """Same RNG draws as the reference (symbolic_torch/utils.py:7-41) on the same device."""
    sr = _sr()
    ops = torch.tensor([[50, 1, 42, 1, 40], [1, 1, 40, 0, 0], [50, 0, 0, 0, 0]], dtype=torch.int64).cuda()
    for method, kw in (("randn", {"mean": 0.5, "std": 2.0}), ("range", {"lower": -1.0, "upper": 3.0})):
        torch.manual_seed(123)
        mine = sr.create_constants(ops, method=method, **kw)
        torch.manual_seed(123)
        mask = ops == 1
        n = int(mask.sum())
        if method == "randn":
            flat = torch.randn(n, dtype=torch.float32, device="cuda") * kw["std"] + kw["mean"]
        else:
            flat = torch.rand(n, dtype=torch.float32, device="cuda") * (kw["upper"] - kw["lower"]) + kw["lower"]
        ref = torch.zeros(ops.shape, dtype=torch.float32, device="cuda")
        ref[mask] = flat
        assert torch.equal(mine, ref)
    # non-contiguous view: row-major order of the view
    torch.manual_seed(5)
    mine = sr.create_constants(ops.t())
    torch.manual_seed(5)
    m = ops.t() == 1
    ref = torch.zeros(m.shape, device="cuda")
    ref[m] = torch.randn(int(m.sum()), device="cuda")
    assert torch.equal(mine, ref)


@pytest.mark.parametrize("B", [1, 1000, 70001])
def test_create_constants_large(B):
    sr = _sr()
    torch.manual_seed(0)
    ops = torch.randint(0, 3, (B, 33), device="cuda")
    torch.manual_seed(1)
    mine = sr.create_constants(ops)
    torch.manual_seed(1)
    m = ops == 1
    ref = torch.zeros(m.shape, device="cuda")
    ref[m] = torch.randn(int(m.sum()), device="cuda")
    assert torch.equal(mine, ref)


# ---- evaluate_multiple (K constant sets) --------------------------------------------

def test_multiple_vs_reference_golden(golden):
    """evaluate_multiple against the reference's own outputs: every set node by node
    (exact operations bit for bit), gradients per set and the X gradient summed over
    the sets."""
    sr = _sr()
    g = golden("multiple")
    X = cuda(g["X"]).requires_grad_(True)
    C = cuda(g["C"]).requires_grad_(True)
    out = sr.evaluation.evaluate_multiple(X, cuda(g["ops"]), cuda(g["ch"]), C)
    assert out.shape == g["cache"].shape
    got = out.detach().cpu().numpy()
    for k in range(g["C"].shape[2]):
        check_local(g["X"], g["ops"], g["ch"], g["C"][:, :, k], got[..., k])
    ref64 = oracle.eval_fwd_multi(g["X"], g["ops"], g["ch"], g["C"], dtype=np.float64)
    check_accuracy(got, g["cache"], ref64)
    out.backward(cuda(g["gout"]))
    gC64, gX64, err = oracle.eval_bwd_multi(g["X"], g["ops"], g["ch"], g["C"], g["gout"], dtype=np.float64)
    assert err == 0
    check_accuracy(C.grad.cpu().numpy(), g["gC"], gC64, rtol=1e-5, atol=1e-5, min_frac_tight=0.99)
    check_accuracy(X.grad.cpu().numpy(), g["gX"], gX64, rtol=1e-4, atol=1e-4, min_frac_tight=0.9)


@pytest.mark.parametrize("dtype", [torch.float32, torch.float64])
def test_multiple_equals_single_per_set(dtype):
    """Set k of evaluate_multiple is evaluate() with C[..., k], bit for bit, and so are
    the per-set constant gradients; the X gradient is the sum over the sets."""
    sr = _sr()
    from cudasymbolicregression_gb300 import tapes
    rng = np.random.default_rng(21)
    B, M, N, K = 90, 32, 77, 4
    X = rng.uniform(-3, 3, (N, 2))
    tb = tapes.generate(B, M, seed=22, mean_length=12, n_vars=2, p_const_leaf=0.3, X_screen=X.astype(np.float32))
    C = rng.standard_normal((B, M, K))
    Xt = cuda(X, dtype)
    ops, ch = cuda(tb.ops), cuda(tb.ch)
    Cm = cuda(C, dtype).requires_grad_(True)
    Xm = Xt.clone().requires_grad_(True)
    out = sr.evaluation.evaluate_multiple(Xm, ops, ch, Cm)
    root = np.maximum((tb.ops != 0).sum(1) - 1, 0)
    gout = np.zeros(out.shape)
    gout[np.arange(B), root] = rng.standard_normal((B, N, K))
    out.backward(cuda(gout, dtype))
    gx_sum = torch.zeros_like(Xt)
    for k in range(K):
        Ck = cuda(C[:, :, k], dtype).requires_grad_(True)
        Xk = Xt.clone().requires_grad_(True)
        single = sr.evaluation.evaluate(Xk, ops, ch, Ck)
        assert torch.equal(torch.nan_to_num(single, nan=7.0), torch.nan_to_num(out[..., k].detach(), nan=7.0))
        single.backward(cuda(gout[..., k], dtype))
        assert torch.equal(torch.nan_to_num(Ck.grad, nan=7.0), torch.nan_to_num(Cm.grad[..., k], nan=7.0))
        gx_sum += Xk.grad
    torch.testing.assert_close(Xm.grad, gx_sum, rtol=1e-5, atol=1e-5, equal_nan=True)


def test_multiple_backend_layout_and_errors(golden):
    """M-first entry point (M, N, B, K) (reference src/symbolic_evaluation.cpp:171-202),
    its argument checks and the backward error context."""
    sr = _sr()
    g = golden("multiple")
    X, ops, ch, C = cuda(g["X"]), cuda(g["ops"]), cuda(g["ch"]), cuda(g["C"])
    out = sr.evaluation.evaluate_multiple_constant_backend(X, ops.permute(1, 0), ch.permute(1, 0, 2),
                                                           C.permute(1, 0, 2))
    B, M, K = g["C"].shape
    assert out.shape == (M, X.shape[0], B, K)
    direct = sr.evaluation.evaluate_multiple(X, ops, ch, C)
    assert torch.equal(torch.nan_to_num(out.permute(2, 0, 1, 3), nan=3.0), torch.nan_to_num(direct, nan=3.0))
    with pytest.raises(RuntimeError, match="C must be a 3D tensor for multiple constant evaluation"):
        sr.evaluation.evaluate_multiple_constant_backend(X, ops.permute(1, 0), ch.permute(1, 0, 2),
                                                         C[:, :, 0].permute(1, 0))
    with pytest.raises(RuntimeError, match="must have the same batch size"):
        sr.evaluation.evaluate_multiple(X, ops, ch, C[:-1])
    e = golden("errors")
    o, c = cuda(e["noop_grad__ops"]), cuda(e["noop_grad__ch"])
    Xe = cuda(e["noop_grad__X"]).requires_grad_(True)
    Ce = torch.zeros(o.shape + (2,), device="cuda").requires_grad_(True)
    y = sr.evaluation.evaluate_multiple(Xe, o, c, Ce)
    gy = torch.zeros_like(y)
    gy[:, -1] = 1.0
    with pytest.raises(RuntimeError, match="multiple constants"):
        y.backward(gy)


def test_gradients_match_central_finite_differences_fp64():
    """The adjoint in float64 against central finite differences (h = 1e-3) of the
    float64 forward: loss = sum of root outputs, gradient w.r.t. C, tapes over
    {+,-,*,/,sin,cos,exp,log,X0..X3,C} with X ~ U[-3, 3] and C ~ N(0, 1).  The
    differences at h and h/2 give a Richardson estimate and its truncation error,
    which (with the rounding error of the differences) is the tolerance.  Only
    entries where the function is smooth at the scale of h are compared: no division
    by a value below 0.05 at any point, a loss below 1e6, and a change over h no
    larger than ten times the loss (elsewhere the root oscillates or blows up within
    h and the difference quotient is meaningless; the CPU oracle shows the same
    picture there, so those entries say nothing about this kernel)."""
    sr = _sr()
    from cudasymbolicregression_gb300 import tapes
    rng = np.random.default_rng(31)
    B, M, N, nx, h = 2048, 64, 64, 4, 1e-3
    X = rng.uniform(-3, 3, (N, nx))
    C = rng.standard_normal((B, M))
    tb = tapes.generate(B, M, seed=32, mean_length=20, n_vars=nx, p_const_leaf=0.2,
                        X_screen=X.astype(np.float32), C_screen=C.astype(np.float32))
    ops, ch = cuda(tb.ops), cuda(tb.ch)
    Xt = cuda(X, torch.float64)
    root = torch.tensor(np.maximum((tb.ops != 0).sum(1) - 1, 0)).cuda()

    def loss_rows(Cn):
        with torch.no_grad():
            out = sr.evaluation.evaluate(Xt, ops, ch, cuda(Cn, torch.float64))
        return out[torch.arange(B).cuda(), root].sum(1).cpu().numpy()

    Ct = cuda(C, torch.float64).requires_grad_(True)
    out = sr.evaluation.evaluate(Xt, ops, ch, Ct)
    gout = torch.zeros_like(out)
    gout[torch.arange(B).cuda(), root] = 1.0
    out.backward(gout)
    g = Ct.grad.cpu().numpy()
    L0 = loss_rows(C)
    # a difference quotient only means something where the function is smooth at the
    # scale of h: leave out tapes that divide by a value near zero at some point (the
    # root then oscillates or blows up within h) and tapes whose loss is huge
    vals = out.detach().cpu().numpy()
    smooth = np.abs(L0) < 1e6
    from cudasymbolicregression_gb300.operators import Operator
    for b_, k_ in zip(*np.nonzero(tb.ops == int(Operator.DIV))):
        den = np.abs(vals[b_, tb.ch[b_, k_, 1]])
        if (den[np.isfinite(den)] < 0.05).any():
            smooth[b_] = False
    is_c = tb.ops == 1
    rank = np.cumsum(is_c, 1) - 1
    checked = agree = 0
    with np.errstate(invalid="ignore", over="ignore"):
        for j in range(int(is_c.sum(1).max())):
            rows, cols = np.nonzero(is_c & (rank == j))
            fds = []
            for step in (h, h / 2):
                Cp, Cm = C.copy(), C.copy()
                Cp[rows, cols] += step
                Cm[rows, cols] -= step
                fds.append(((loss_rows(Cp) - loss_rows(Cm)) / (2 * step))[rows])
            f1, f2 = fds
            rich = (4 * f2 - f1) / 3
            ad = g[rows, cols]
            ok = smooth[rows] & np.isfinite(L0[rows]) & np.isfinite(f1) & np.isfinite(f2) & np.isfinite(ad)
            ok &= np.abs(ad) * h <= 10 * (np.abs(L0[rows]) + 1)  # changes within h stay small
            tol = 1e-6 * np.maximum(np.abs(ad), 1.0) + 4 * np.abs(f1 - f2) + 1e-12 * np.abs(L0[rows]) / (h / 2)
            checked += int(ok.sum())
            agree += int((np.abs(rich - ad) <= tol)[ok].sum())
    assert checked > 200
    assert agree / checked >= 0.99, (agree, checked)


def test_forward_and_adjoint_replay_in_a_cuda_graph():
    """The forward (length-class grids + the padding fill on the side stream) and the
    adjoint (the padding check on the side stream + length-class grids), called through
    the C ABI inside a CUDA graph capture: the fork/join of the side stream is recorded,
    and a replay gives the direct calls' results bit for bit."""
    sr = _sr()
    from cudasymbolicregression_gb300 import _lib, tapes as tg
    from cudasymbolicregression_gb300.tape import compile_tapes
    rng = np.random.default_rng(31)
    B, M, N, nx = 3000, 64, 256, 3
    # no division: a zero denominator would make both runs report 204, which is not the point here
    tb = tg.generate(B, M, seed=32, mean_length=20.0, n_vars=nx, p_const_leaf=0.3, binary=(40, 41, 42))
    X = cuda(rng.uniform(-2, 2, (N, nx)).astype(np.float32))
    C = cuda(rng.standard_normal((B, M)).astype(np.float32))
    ops, ch = cuda(tb.ops), cuda(tb.ch)
    tp = compile_tapes(ops, ch, nx)
    L = _lib.lib()
    gout = torch.zeros((B, M, N), device="cuda")
    root = torch.tensor(np.maximum((tb.ops != 0).sum(1) - 1, 0), device="cuda")
    gout[torch.arange(B, device="cuda"), root] = 1.0

    def run(cache, gC, status):
        st = _lib.stream_ptr(X.device)
        _lib.check(L.sr_eval_forward_f32(_lib.ptr(X), N, nx, _lib.ptr(tp.desc), _lib.ptr(tp.meta), _lib.ptr(tp.order),
                                         B, M, tp.max_len, _lib.ptr(C), M, 1, _lib.ptr(cache), st), "forward")
        _lib.check(L.sr_eval_backward_f32(_lib.ptr(X), N, nx, _lib.ptr(tp.desc), _lib.ptr(tp.meta), _lib.ptr(tp.order),
                                          B, M, tp.max_len, _lib.ptr(C), M, 1, _lib.ptr(cache), _lib.ptr(gout),
                                          _lib.ptr(gC), None, _lib.ptr(status), st), "backward")

    ref = (torch.empty((B, M, N), device="cuda"), torch.empty((B, M), device="cuda"),
           torch.zeros(1, dtype=torch.int32, device="cuda"))
    run(*ref)
    torch.cuda.synchronize()
    assert int(ref[2].item()) == 0
    out = (torch.full((B, M, N), 7.0, device="cuda"), torch.full((B, M), 7.0, device="cuda"),
           torch.zeros(1, dtype=torch.int32, device="cuda"))
    g = torch.cuda.CUDAGraph()
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(s):
        run(*out)  # warm-up on the capture stream
    torch.cuda.current_stream().wait_stream(s)
    out[0].fill_(7.0)
    out[1].fill_(7.0)
    with torch.cuda.graph(g):
        run(*out)
    g.replay()
    torch.cuda.synchronize()
    assert int(out[2].item()) == 0
    assert torch.equal(torch.nan_to_num(out[0], nan=-9.0), torch.nan_to_num(ref[0], nan=-9.0))
    assert torch.equal(torch.nan_to_num(out[1], nan=-9.0), torch.nan_to_num(ref[1], nan=-9.0))


def test_tape_longer_than_max_len_is_nan_and_reported():
    """A C-ABI caller that passes a max_len below some tape's length: the forward leaves
    no stale rows (that tape's whole block is NaN; the others are evaluated as usual)
    and the adjoint reports status 602 instead of skipping the tape silently."""
    from cudasymbolicregression_gb300 import _lib, tapes as tg
    from cudasymbolicregression_gb300.tape import compile_tapes
    rng = np.random.default_rng(41)
    B, M, N, nx = 200, 48, 64, 2
    tb = tg.generate(B, M, seed=42, lengths=rng.integers(2, M + 1, size=B), n_vars=nx, binary=(40, 41, 42))
    X = cuda(rng.uniform(-2, 2, (N, nx)).astype(np.float32))
    C = cuda(rng.standard_normal((B, M)).astype(np.float32))
    tp = compile_tapes(cuda(tb.ops), cuda(tb.ch), nx)
    L = _lib.lib()
    st = _lib.stream_ptr(X.device)
    max_len = 20
    lens = tp.meta[:, 0].cpu().numpy()
    over = lens > max_len
    assert over.any() and (~over).any()
    cache = torch.full((B, M, N), 7.0, device="cuda")
    _lib.check(L.sr_eval_forward_f32(_lib.ptr(X), N, nx, _lib.ptr(tp.desc), _lib.ptr(tp.meta), None, B, M, max_len,
                                     _lib.ptr(C), M, 1, _lib.ptr(cache), st), "forward")
    full = torch.empty((B, M, N), device="cuda")
    _lib.check(L.sr_eval_forward_f32(_lib.ptr(X), N, nx, _lib.ptr(tp.desc), _lib.ptr(tp.meta), None, B, M, tp.max_len,
                                     _lib.ptr(C), M, 1, _lib.ptr(full), st), "forward")
    torch.cuda.synchronize()
    got, ref = cache.cpu().numpy(), full.cpu().numpy()
    assert np.isnan(got[over]).all()
    np.testing.assert_array_equal(np.nan_to_num(got[~over], nan=-9.0), np.nan_to_num(ref[~over], nan=-9.0))
    gout = torch.zeros((B, M, N), device="cuda")
    gC = torch.zeros((B, M), device="cuda")
    status = torch.zeros(1, dtype=torch.int32, device="cuda")
    _lib.check(L.sr_eval_backward_f32(_lib.ptr(X), N, nx, _lib.ptr(tp.desc), _lib.ptr(tp.meta), None, B, M, max_len,
                                      _lib.ptr(C), M, 1, None, _lib.ptr(gout), _lib.ptr(gC), None, _lib.ptr(status),
                                      st), "backward")
    torch.cuda.synchronize()
    assert int(status.item()) == _lib.TAPE_EXCEEDS_LAUNCH


@pytest.mark.parametrize("dtype,K", [(torch.float32, 0), (torch.float64, 0), (torch.float32, 3), (torch.float64, 2)])
def test_adjoint_from_cache_equals_recomputed(dtype, K):
    """The adjoint reading the node values from the forward's cache (as autograd calls
    it) and the adjoint recomputing them (cache_dev NULL) give the same grad_C bit for
    bit and the same status; grad_X, an atomic sum, agrees to rounding.  K = 0: the
    single-set entry points (16-byte staging when N is a multiple of 4), else
    evaluate_multiple's (strided staging); N = 1001 leaves a ragged last chunk."""
    from cudasymbolicregression_gb300 import _lib, tapes as tg
    from cudasymbolicregression_gb300.tape import compile_tapes
    rng = np.random.default_rng(41 + K)
    B, M, nx = 700, 64, 3
    npdt = np.float32 if dtype == torch.float32 else np.float64
    tb = tg.generate(B, M, seed=42 + K, mean_length=24.0, n_vars=nx, p_const_leaf=0.3, binary=(40, 41, 42))
    tp = compile_tapes(cuda(tb.ops), cuda(tb.ch), nx)
    L = _lib.lib()
    st = _lib.stream_ptr(torch.device("cuda"))
    sfx = "f32" if dtype == torch.float32 else "f64"
    for N in (1000, 1001):
        X = cuda(rng.uniform(-2, 2, (N, nx)).astype(npdt))
        kk = max(K, 1)
        C = cuda(rng.standard_normal((B, M, kk)).astype(npdt))
        cache = torch.empty((B, M, N, kk), dtype=dtype, device="cuda")
        gout = torch.as_tensor(rng.standard_normal((B, M, N, kk)), dtype=dtype).cuda()
        if K == 0:
            _lib.check(getattr(L, "sr_eval_forward_" + sfx)(
                _lib.ptr(X), N, nx, _lib.ptr(tp.desc), _lib.ptr(tp.meta), _lib.ptr(tp.order), B, M, tp.max_len,
                _lib.ptr(C), M, 1, _lib.ptr(cache), st), "forward")
        else:
            _lib.check(getattr(L, "sr_eval_forward_multi_" + sfx)(
                _lib.ptr(X), N, nx, _lib.ptr(tp.desc), _lib.ptr(tp.meta), _lib.ptr(tp.order), B, M, tp.max_len,
                _lib.ptr(C), M * kk, kk, 1, kk, _lib.ptr(cache), st), "forward")
        gout[torch.isnan(cache)] = 0.0  # the padding rows (NaN) and NO_OP values take no gradient
        out = []
        for cp in (cache, None):
            gC = torch.full((B, M, kk), 7.0, dtype=dtype, device="cuda")
            gX = torch.zeros((N, nx), dtype=dtype, device="cuda")
            status = torch.full((1,), -1, dtype=torch.int32, device="cuda")
            cptr = None if cp is None else _lib.ptr(cp)
            if K == 0:
                _lib.check(getattr(L, "sr_eval_backward_" + sfx)(
                    _lib.ptr(X), N, nx, _lib.ptr(tp.desc), _lib.ptr(tp.meta), _lib.ptr(tp.order), B, M, tp.max_len,
                    _lib.ptr(C), M, 1, cptr, _lib.ptr(gout), _lib.ptr(gC), _lib.ptr(gX), _lib.ptr(status), st),
                    "backward")
            else:
                _lib.check(getattr(L, "sr_eval_backward_multi_" + sfx)(
                    _lib.ptr(X), N, nx, _lib.ptr(tp.desc), _lib.ptr(tp.meta), _lib.ptr(tp.order), B, M, tp.max_len,
                    _lib.ptr(C), M * kk, kk, 1, kk, cptr, _lib.ptr(gout), _lib.ptr(gC), _lib.ptr(gX),
                    _lib.ptr(status), st), "backward")
            torch.cuda.synchronize()
            out.append((gC.cpu().numpy(), gX.cpu().numpy(), int(status.item())))
        (gc1, gx1, s1), (gc2, gx2, s2) = out
        assert s1 == s2 == 0
        assert np.array_equal(gc1.view(np.uint64 if dtype == torch.float64 else np.uint32),
                              gc2.view(np.uint64 if dtype == torch.float64 else np.uint32)), f"N={N}"
        fin = np.isfinite(gx2)
        assert np.array_equal(np.isfinite(gx1), fin) and np.array_equal(np.isnan(gx1), np.isnan(gx2))
        assert np.array_equal(gx1[np.isinf(gx2)], gx2[np.isinf(gx2)])
        tol = 1e-4 if dtype == torch.float32 else 1e-10
        if fin.any():
            np.testing.assert_allclose(gx1[fin], gx2[fin], rtol=tol, atol=tol * np.abs(gx2[fin]).max())
