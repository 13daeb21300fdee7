"""GPU tests of the warm-start network's kernels against the numpy oracle
(oracle/mlp_oracle.py), through the C ABI.

Tolerances: a GEMM accumulates bf16 products in fp32 on the tensor cores, so an
fp32 result may differ from the float64 sum of the same operands by the fp32
accumulation error, bounded here by 1e-5 * sum_k |a_k w_k|; a bf16 result is that
value rounded to bfloat16, so it equals the oracle's rounding of the float64 value
except within one bf16 ulp of a rounding boundary.
"""
import ctypes

import numpy as np
import pytest
import torch

import mlp_oracle as mo

pytestmark = pytest.mark.gpu


def _sr():
    import cudasymbolicregression_gb300 as sr
    return sr


def bf(a):
    return torch.tensor(mo.bf16(a)).to(torch.bfloat16).cuda()


def np32(t):
    return t.float().cpu().numpy()


def gemm_call(A, W, rows, k, n, **epi):
    from cudasymbolicregression_gb300 import _lib
    e = _lib.MlpEpilogue()
    for key, val in epi.items():
        if isinstance(val, torch.Tensor):
            setattr(e, key, ctypes.c_void_p(val.data_ptr()))
        else:
            setattr(e, key, val)
    status = torch.zeros(1, dtype=torch.int32, device="cuda")
    rc = _lib.lib().sr_mlp_gemm(ctypes.c_void_p(A.data_ptr()), rows, k, A.shape[1], ctypes.c_void_p(W.data_ptr()),
                                n, W.shape[1], ctypes.byref(e), ctypes.c_void_p(status.data_ptr()),
                                _lib.stream_ptr(torch.device("cuda")))
    _lib.check(rc, "sr_mlp_gemm")
    torch.cuda.synchronize()
    assert int(status.item()) == 0
    return status


def check_f32(dev, ref, A, W):
    bound = acc_bound(A, W) + 1e-30
    err = np.abs(dev.astype(np.float64) - ref)
    assert (err <= bound + 1e-6 * np.abs(ref)).all(), float((err - bound).max())


def acc_bound(A, W):
    """fp32 accumulation error bound of A . W^T."""
    return 1e-5 * (np.abs(A).astype(np.float64) @ np.abs(W).astype(np.float64).T)


def check_bf16(dev, ref_f64, bound=0.0):
    """dev (bf16 values) against the bf16 rounding of the float64 value: equal, or
    within one bf16 ulp plus the fp32 accumulation bound (values next to a rounding
    boundary, or near zero after cancellation)."""
    exp = mo.bf16(ref_f64.astype(np.float32))
    same = dev == exp
    ulp = np.abs(exp) * 2.0 ** -7 + 1e-38
    near = np.abs(dev.astype(np.float64) - ref_f64) <= ulp + bound
    assert (same | near).all(), np.argwhere(~(same | near))[:5]
    assert same.mean() >= 0.99, same.mean()


@pytest.mark.parametrize("rows,k,n", [(128, 64, 64), (300, 128, 256), (1000, 256, 128), (129, 320, 256)])
def test_gemm_f32_and_relu(rows, k, n):
    from cudasymbolicregression_gb300 import _lib
    rng = np.random.default_rng(rows + k + n)
    A = mo.bf16(rng.standard_normal((rows, k)).astype(np.float32))
    W = mo.bf16((rng.standard_normal((n, k)) / np.sqrt(k)).astype(np.float32))
    bias = rng.standard_normal(n).astype(np.float32)
    Ad, Wd = bf(A), bf(W)
    acc = mo.gemm(A, W)
    out = torch.zeros(rows, n, device="cuda")
    gemm_call(Ad, Wd, rows, k, n, epilogue=_lib.MLP_EPI_F32, out_f32=out, ld_out_f32=n,
              bias=torch.tensor(bias).cuda())
    check_f32(np32(out), acc + bias, A, W)
    h = torch.zeros(rows, n + 64, dtype=torch.bfloat16, device="cuda")
    ht = torch.zeros(n + 8, rows + 8, dtype=torch.bfloat16, device="cuda")
    gemm_call(Ad, Wd, rows, k, n, epilogue=_lib.MLP_EPI_RELU, bias=torch.tensor(bias).cuda(), out=h,
              ld_out=n + 64, out_col0=64, out_t=ht, ld_out_t=rows + 8, out_t_row0=8)
    ref = mo.epilogue(acc, 0, bias)
    hn, htn = np32(h), np32(ht)
    check_bf16(hn[:, 64:], ref, acc_bound(A, W))
    assert (hn[:, :64] == 0).all()
    np.testing.assert_array_equal(htn[8:8 + n, :rows], hn[:, 64:].T)
    assert (htn[:8] == 0).all() and (htn[:, rows:] == 0).all()


@pytest.mark.parametrize("n", [64, 256])
def test_gemm_relu_gate_and_linear(n):
    from cudasymbolicregression_gb300 import _lib
    rows, k = 384, 192
    rng = np.random.default_rng(n)
    A = mo.bf16(rng.standard_normal((rows, k)).astype(np.float32))
    W = mo.bf16(rng.standard_normal((n, k)).astype(np.float32) * 0.1)
    gate = mo.bf16(np.maximum(rng.standard_normal((rows, n)), 0).astype(np.float32))
    acc = mo.gemm(A, W)
    out = torch.zeros(rows, n, dtype=torch.bfloat16, device="cuda")
    gemm_call(bf(A), bf(W), rows, k, n, epilogue=_lib.MLP_EPI_RELU_GRAD, gate=bf(gate), ld_gate=n, out=out, ld_out=n)
    check_bf16(np32(out), mo.epilogue(acc, 3, gate=gate), acc_bound(A, W))
    lin_t = torch.zeros(n, rows, dtype=torch.bfloat16, device="cuda")
    gemm_call(bf(A), bf(W), rows, k, n, epilogue=_lib.MLP_EPI_LINEAR, out_t=lin_t, ld_out_t=rows)
    check_bf16(np32(lin_t).T, acc, acc_bound(A, W))


@pytest.mark.parametrize("splits", [1, 3, 8])
def test_gemm_split_reduction(splits):
    """Weight-gradient shape: a long reduction (k = batch) cut into pieces."""
    from cudasymbolicregression_gb300 import _lib
    L = _lib.lib()
    rows, k, n = 256, 64 * 13, 128
    rng = np.random.default_rng(splits)
    A = mo.bf16(rng.standard_normal((rows, k)).astype(np.float32) * 0.05)
    W = mo.bf16(rng.standard_normal((n, k)).astype(np.float32))
    used = L.sr_mlp_gemm_splits_used(k, splits)
    assert 1 <= used <= splits
    part = torch.full((used, rows, n), float("nan"), device="cuda")
    gemm_call(bf(A), bf(W), rows, k, n, epilogue=_lib.MLP_EPI_SPLIT_F32, splits=splits, out_f32=part, ld_out_f32=n,
              split_stride=rows * n)
    out = torch.empty(rows, n, device="cuda")
    _lib.check(L.sr_mlp_reduce_splits(ctypes.c_void_p(part.data_ptr()), used, rows * n, rows * n,
                                      ctypes.c_void_p(out.data_ptr()), None), "reduce")
    torch.cuda.synchronize()
    check_f32(np32(out), mo.gemm(A, W), A, W)


def test_gemm_rejects_bad_shapes():
    from cudasymbolicregression_gb300 import _lib
    A = torch.zeros(128, 96, dtype=torch.bfloat16, device="cuda")
    W = torch.zeros(64, 96, dtype=torch.bfloat16, device="cuda")
    out = torch.zeros(128, 64, device="cuda")
    with pytest.raises(RuntimeError, match="multiple of 64"):
        gemm_call(A, W, 128, 96, 64, epilogue=_lib.MLP_EPI_F32, out_f32=out, ld_out_f32=64)


def test_features_match_oracle():
    sr = _sr()
    from cudasymbolicregression_gb300 import tapes, warmstart
    rng = np.random.default_rng(3)
    B, M, N = 300, 64, 512
    X = rng.uniform(-3, 3, (N, 2)).astype(np.float32)
    tb = tapes.generate(B, M, seed=4, lengths=rng.integers(3, M + 1, B), const_counts=rng.integers(0, 9, B),
                        n_vars=2)
    Y = (rng.standard_normal((B, N)) * rng.uniform(0.1, 10, (B, 1)) + rng.uniform(-5, 5, (B, 1))).astype(np.float32)
    Y[0] = 1.5  # a flat target
    net = warmstart.WarmStartMLP(seed=1)
    ws = net.workspace(B)
    net.features(torch.tensor(tb.ops).cuda(), torch.tensor(X).cuda(), torch.tensor(Y).cuda(), ws)
    torch.cuda.synchronize()
    phi = mo.random_features(X, net.omega.cpu().numpy(), net.beta.cpu().numpy())
    hist, feats = mo.features(tb.ops, Y, phi)
    np.testing.assert_array_equal(np32(ws.hist[:B]), mo.bf16(hist))
    np.testing.assert_array_equal(np32(ws.hist_t[:, :B]).T, mo.bf16(hist))
    f = ws.feats[:B].cpu().numpy()
    np.testing.assert_allclose(f, feats, rtol=2e-3, atol=2e-4)
    x0 = np32(ws.x0[:B])
    np.testing.assert_array_equal(x0[:, 64:96], mo.bf16(f))
    assert (x0[:, 96:] == 0).all()
    del sr


def _random_net(seed):
    from cudasymbolicregression_gb300 import warmstart
    net = warmstart.WarmStartMLP(seed=seed)
    g = torch.Generator().manual_seed(seed + 1)
    for k in net.b:
        net.b[k].copy_(torch.randn(net.b[k].shape, generator=g) * 0.1)
    net._pack()
    return net


def test_forward_backward_layer_local():
    """Every layer of the device forward/backward recomputed by the oracle from the
    device's own inputs to that layer."""
    from cudasymbolicregression_gb300 import tapes
    rng = np.random.default_rng(5)
    B, M, N = 500, 64, 256
    X = rng.uniform(-3, 3, (N, 2)).astype(np.float32)
    tb = tapes.generate(B, M, seed=6, lengths=rng.integers(3, M + 1, B), const_counts=rng.integers(0, 9, B), n_vars=2)
    Y = rng.standard_normal((B, N)).astype(np.float32)
    net = _random_net(2)
    ws = net.workspace(B)
    tgt = torch.tensor(rng.standard_normal((B, 8)).astype(np.float32)).cuda()
    msk = torch.tensor((rng.uniform(size=(B, 8)) < 0.6).astype(np.float32)).cuda()
    ws.target.zero_()
    ws.mask.zero_()
    ws.target[:B] = tgt
    ws.mask[:B] = msk
    net.features(torch.tensor(tb.ops).cuda(), torch.tensor(X).cuda(), torch.tensor(Y).cuda(), ws)
    net.forward_ws(ws, B)
    net.backward_ws(ws, B)
    torch.cuda.synchronize()
    R = ws.R
    w = {k: np32(v) for k, v in net.w_bf.items()}
    b = {k: v.cpu().numpy() for k, v in net.b.items()}
    hist, x0 = np32(ws.hist), np32(ws.x0)
    check_bf16(x0[:, :64], mo.gemm(hist, w["E"]), acc_bound(hist, w["E"]))
    h = {i: np32(ws.h[i][0]) for i in (1, 2, 3)}
    check_bf16(h[1], mo.epilogue(mo.gemm(x0, w["W1"]), 0, b["W1"]), acc_bound(x0, w["W1"]))
    check_bf16(h[2], mo.epilogue(mo.gemm(h[1], w["W2"]), 0, b["W2"]), acc_bound(h[1], w["W2"]))
    check_bf16(h[3], mo.epilogue(mo.gemm(h[2], w["W3"]), 0, b["W3"]), acc_bound(h[2], w["W3"]))
    out = ws.out.cpu().numpy()
    check_f32(out, mo.epilogue(mo.gemm(h[3], w["W4"]), 2, b["W4"]), h[3], w["W4"])
    # loss and output gradient
    tg = np.zeros((R, 8), np.float32)
    mk = np.zeros((R, 8), np.float32)
    tg[:B], mk[:B] = tgt.cpu().numpy(), msk.cpu().numpy()
    row, g = mo.loss(out, tg, mk, 1.0 / B)
    np.testing.assert_allclose(ws.row_loss.cpu().numpy(), row, rtol=1e-5, atol=1e-6)
    d_out = np32(ws.d_out)
    check_bf16(d_out, g)
    # adjoint layers and weight gradients from the device's own inputs
    dz = {i: np32(ws.dz[i][0]) for i in (1, 2, 3)}
    check_bf16(dz[3], mo.epilogue(mo.gemm(d_out, w["W4"].T), 3, gate=h[3]), acc_bound(d_out, w["W4"].T))
    check_bf16(dz[2], mo.epilogue(mo.gemm(dz[3], w["W3"].T), 3, gate=h[2]), acc_bound(dz[3], w["W3"].T))
    check_bf16(dz[1], mo.epilogue(mo.gemm(dz[2], w["W2"].T), 3, gate=h[1]), acc_bound(dz[2], w["W2"].T))
    np.testing.assert_array_equal(np32(ws.dz[2][1]).T, dz[2])
    gw = {k: v.cpu().numpy() for k, v in net.gw.items()}
    gb = {k: v.cpu().numpy() for k, v in net.gb.items()}
    check_f32(gw["W4"], mo.gemm(d_out.T, h[3].T), d_out.T, h[3].T)
    check_f32(gw["W3"], mo.gemm(dz[3].T, h[2].T), dz[3].T, h[2].T)
    check_f32(gw["W1"], mo.gemm(dz[1].T, x0.T), dz[1].T, x0.T)
    np.testing.assert_allclose(gb["W3"], dz[3].astype(np.float64).sum(0), rtol=1e-4, atol=1e-6)
    dx0_t = np32(ws.dx0_t)
    check_bf16(dx0_t.T, mo.gemm(dz[1], w["W1"].T), acc_bound(dz[1], w["W1"].T))
    check_f32(gw["E"], mo.gemm(dx0_t[:64], hist.T), dx0_t[:64], hist.T)


def test_backward_end_to_end_against_oracle():
    """Whole-network gradients against the oracle's forward + backward from the same
    bf16 weights and inputs (aggregate relative error, bf16 rounding points shared)."""
    from cudasymbolicregression_gb300 import tapes
    rng = np.random.default_rng(8)
    B, M, N = 256, 64, 256
    X = rng.uniform(-3, 3, (N, 2)).astype(np.float32)
    tb = tapes.generate(B, M, seed=9, lengths=rng.integers(3, M + 1, B), const_counts=rng.integers(0, 9, B), n_vars=2)
    Y = rng.standard_normal((B, N)).astype(np.float32)
    net = _random_net(3)
    ws = net.workspace(B)
    ws.target.zero_()
    ws.mask.zero_()
    tg = rng.standard_normal((B, 8)).astype(np.float32)
    ws.target[:B] = torch.tensor(tg).cuda()
    ws.mask[:B] = 1.0
    net.features(torch.tensor(tb.ops).cuda(), torch.tensor(X).cuda(), torch.tensor(Y).cuda(), ws)
    net.forward_ws(ws, B)
    net.backward_ws(ws, B)
    torch.cuda.synchronize()
    w = {k: np32(v) for k, v in net.w_bf.items()}
    b = {k: v.cpu().numpy() for k, v in net.b.items()}
    hist = np32(ws.hist)[:B]
    feats = ws.feats[:B].cpu().numpy()
    out, acts = mo.forward(w, b, hist, feats)
    dev_out = ws.out[:B].cpu().numpy()
    assert np.linalg.norm(dev_out - out) <= 1e-2 * np.linalg.norm(out)
    _, g = mo.loss(out, tg, np.ones((B, 8), np.float32), 1.0 / B)
    gw, gbias = mo.backward(w, b, hist, acts, g)
    for k in ("E", "W1", "W2", "W3", "W4"):
        d = net.gw[k].cpu().numpy()
        assert np.linalg.norm(d - gw[k]) <= 3e-2 * np.linalg.norm(gw[k]) + 1e-12, k
    for k in ("W1", "W2", "W3", "W4"):
        d = net.gb[k].cpu().numpy()
        assert np.linalg.norm(d - gbias[k]) <= 3e-2 * np.linalg.norm(gbias[k]) + 1e-12, k


def test_adam_matches_oracle_and_refreshes_bf16_copies():
    from cudasymbolicregression_gb300 import _lib
    L = _lib.lib()
    rng = np.random.default_rng(11)
    rows, cols = 64, 96
    w0 = rng.standard_normal((rows, cols)).astype(np.float32)
    g = rng.standard_normal((rows, cols)).astype(np.float32)
    w, gd = torch.tensor(w0).cuda(), torch.tensor(g).cuda()
    m, v = torch.zeros_like(w), torch.zeros_like(w)
    wb = torch.zeros(rows, cols, dtype=torch.bfloat16, device="cuda")
    wbt = torch.zeros(cols, rows, dtype=torch.bfloat16, device="cuda")
    p = lambda t: ctypes.c_void_p(t.data_ptr())  # noqa: E731
    wr, mr, vr = w0.astype(np.float64), np.zeros((rows, cols)), np.zeros((rows, cols))
    for step in (1, 2, 3):
        _lib.check(L.sr_mlp_adam(p(w), p(gd), p(m), p(v), rows, cols, 1e-2, 0.9, 0.999, 1e-8, 1e-2, step, p(wb),
                                 p(wbt), None), "adam")
        wr, mr, vr = mo.adam(wr, g.astype(np.float64), mr, vr, step, 1e-2, weight_decay=1e-2)
    torch.cuda.synchronize()
    np.testing.assert_allclose(w.cpu().numpy(), wr, rtol=1e-5, atol=1e-6)
    np.testing.assert_array_equal(np32(wb), mo.bf16(w.cpu().numpy()))
    np.testing.assert_array_equal(np32(wbt), mo.bf16(w.cpu().numpy()).T)


def test_training_reduces_loss_on_a_learnable_target():
    """Targets that are a fixed function of the features: the loss must fall."""
    from cudasymbolicregression_gb300 import tapes, warmstart
    rng = np.random.default_rng(12)
    B, M, N = 4096, 64, 256
    X = torch.tensor(rng.uniform(-3, 3, (N, 2)).astype(np.float32)).cuda()
    tb = tapes.generate(B, M, seed=13, lengths=rng.integers(3, M + 1, B), const_counts=rng.integers(0, 9, B),
                        n_vars=2)
    scale = rng.uniform(0.5, 3, (B, 1)).astype(np.float32)
    Y = torch.tensor((rng.standard_normal((B, N)) * scale + 2 * scale).astype(np.float32)).cuda()
    ops = torch.tensor(tb.ops).cuda()
    tgt = torch.tensor(np.repeat(scale, 8, 1)).cuda()
    msk = torch.ones(B, 8, device="cuda")
    net = warmstart.WarmStartMLP(seed=4)
    first = last = None
    for it in range(150):
        s = (it * 1024) % B
        loss = net.train_batch(ops[s:s + 1024], X, Y[s:s + 1024], tgt[s:s + 1024], msk[s:s + 1024], lr=2e-3)
        val = float(loss.mean())
        first = val if first is None else first
        last = val
    net.check_status()
    assert last < 0.1 * first, (first, last)


def test_warm_start_gains_on_the_readme_problem():
    """Ablation: the README problem (one target, expressions from a small grammar).
    Trained on the fits of 2 x 16384 problems (constants of the plain fits, then the
    fit objective), the gated warm start on 8192 held-out problems must need fewer
    closures than plain randn starts, with a median final MSE no worse (within 0.5%:
    problems that stop at max_iter end at slightly different points)."""
    sr = _sr()
    from cudasymbolicregression_gb300 import warmstart, workloads
    T = lambda a: torch.tensor(a).cuda()  # noqa: E731
    probs, data = [], warmstart.TrainingSet([], [], [], [], [])
    for s in (10, 12):
        tr = workloads.readme_fit(B=16384, seed=s)
        X, Y, O, Ch, C = T(tr.X), T(tr.Y), T(tr.ops), T(tr.ch), T(tr.C)
        tgt, msk, _ = warmstart.fitted_examples(X, Y, O, Ch, C, max_iter=100)
        probs.append((X, Y, O, Ch, C))
        for lst, v in zip((data.X, data.Y, data.ops, data.target, data.mask), (X, Y, O, tgt, msk)):
            lst.append(v)
    net = warmstart.WarmStartMLP(seed=0, n_vars=1)
    warmstart.train(net, data, epochs=12, batch=2048, lr=2e-3)
    warmstart.train_fit_objective(net, probs, epochs=12, batch=2048, lr=5e-4)
    te = workloads.readme_fit(B=8192, seed=11)
    X, Y, O, Ch, C = T(te.X), T(te.Y), T(te.ops), T(te.ch), T(te.C)
    plain = sr.optimize_ex(X, Y, O, Ch, C, max_iter=100, raise_errors=False)
    Cg = warmstart.gated_warm_start(net, X, Y, O, Ch, C)
    warm = sr.optimize_ex(X, Y, O, Ch, Cg, max_iter=100, raise_errors=False)
    ep, ew = plain.evals.float().mean().item(), warm.evals.float().mean().item()
    lp, lw = plain.loss.cpu().numpy(), warm.loss.cpu().numpy()
    fin = np.isfinite(lp)
    mp, mw = np.median(lp[fin]), np.median(np.where(np.isfinite(lw), lw, np.inf)[fin])
    print(f"mean closures plain {ep:.2f} warm {ew:.2f}; median MSE plain {mp:.5g} warm {mw:.5g}")
    assert ew < 0.95 * ep
    assert mw <= mp * 1.005 + 1e-9
