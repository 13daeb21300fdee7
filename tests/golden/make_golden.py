"""Writes the golden fixtures in tests/golden/ by running the reference itself.

Run in the development container, where the reference checkout exists:

    python tests/golden/make_golden.py

The reference extension is compiled from its own sources by
``oracle/build_ref.py`` into ``oracle/_ref`` and imported as ``symbolic_torch``.
Every fixture stores its inputs next to the reference's outputs, so the tests
can replay them on a machine without the reference.  Inputs are seeded.
"""
from __future__ import annotations

import os
import sys

import numpy as np
import torch

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, ROOT)

import build_ref  # noqa: E402
from grammars import BAD_GRAMMARS, NOTATION_GRAMMAR, README_GRAMMAR, SAMPLING_GRAMMAR  # noqa: E402
from inputs import EVAL_INPUT_CASES, MULTI_INPUT_CASES, eval_input_case  # noqa: E402

from cudasymbolicregression_gb300 import tapes  # noqa: E402
from cudasymbolicregression_gb300.operators import BINARY_OPS, UNARY_OPS, Operator  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))
ALL_UNARY = UNARY_OPS
ALL_BINARY = BINARY_OPS


def ref_eval(st, X, ops, ch, C, gout=None):
    """Reference forward (B,M,N) and, with gout, gradients w.r.t. C and X."""
    Xt = torch.tensor(X, requires_grad=True)
    Ct = torch.tensor(C, requires_grad=True)
    out = st.evaluation.evaluate(Xt, torch.tensor(ops), torch.tensor(ch), Ct)
    cache = out.detach().numpy().copy()
    if gout is None:
        return cache, None, None
    out.backward(torch.tensor(gout))
    return cache, Ct.grad.numpy().copy(), Xt.grad.numpy().copy()


def edge_inputs():
    """X rows that hit every domain policy (zero, +-1, negatives, large, tiny)."""
    vals = np.array([-3.0, -2.0, -1.0, -0.5, -1e-30, 0.0, 1e-30, 0.5, 1.0, 2.0, 3.0, 40.0, 100.0,
                     -100.0, 0.25, 7.5], np.float32)
    a = np.repeat(vals, len(vals))
    b = np.tile(vals, len(vals))
    return np.stack([a, b], 1).astype(np.float32)


def case_single_ops(st, rng):
    """Every unary/binary operator applied to X0 (and X1) at the edge inputs."""
    X = edge_inputs()
    ops_list = list(ALL_UNARY) + list(ALL_BINARY)
    B, M = len(ops_list), 3
    ops = np.zeros((B, M), np.int64)
    ch = np.full((B, M, 2), -1, np.int64)
    for b, op in enumerate(ops_list):
        ops[b, 0] = int(Operator.VAR_START_ID)
        ops[b, 1] = int(Operator.VAR_START_ID) + 1
        ops[b, 2] = op
        ch[b, 2, 0] = 0
        if op in ALL_BINARY:
            ch[b, 2, 1] = 1
    C = np.zeros((B, M), np.float32)
    cache, _, _ = ref_eval(st, X, ops, ch, C)
    # gradient through the root only; the reference raises 204 for a/0 with g != 0,
    # so the DIV row gets zero gradient where its denominator is 0.
    gout = np.zeros_like(cache)
    gout[:, 2, :] = rng.standard_normal((B, X.shape[0])).astype(np.float32)
    div_row = ops_list.index(int(Operator.DIV))
    gout[div_row, 2, X[:, 1] == 0] = 0.0
    _, gC, gX = ref_eval(st, X, ops, ch, C, gout)
    # per-row X gradients: run each row alone so gX is not summed over the batch
    gX_rows = np.zeros((B,) + X.shape, np.float32)
    for b in range(B):
        _, _, gx = ref_eval(st, X, ops[b:b + 1], ch[b:b + 1], C[b:b + 1], gout[b:b + 1])
        gX_rows[b] = gx
    np.savez_compressed(os.path.join(OUT, "single_ops.npz"), X=X, ops=ops, ch=ch, C=C, cache=cache,
                        gout=gout, gC=gC, gX=gX, gX_rows=gX_rows)


def case_random_dags(st, rng, name, B, M, N, n_vars, seed, unary, binary, mean_length, dense=True):
    X = rng.uniform(-3, 3, (N, n_vars)).astype(np.float32)
    C = rng.standard_normal((B, M)).astype(np.float32)
    tb = tapes.generate(B, M, seed=seed, mean_length=mean_length, n_vars=n_vars, unary=unary,
                        binary=binary, p_const_leaf=0.3)
    ops, ch = tb.ops, tb.ch
    # sprinkle a few hard constants so CONST_1..E are covered
    consts = np.array([2, 3, 4, 5, 6, 7, 8], np.int64)
    hard = (ops == int(Operator.LEARNABLE_CONSTANT)) & (rng.random(ops.shape) < 0.25)
    ops[hard] = consts[rng.integers(0, len(consts), size=int(hard.sum()))]
    cache, _, _ = ref_eval(st, X, ops, ch, C)
    if dense:
        gout = rng.standard_normal(cache.shape).astype(np.float32)
    else:
        gout = np.zeros_like(cache)
        root = np.maximum((ops != 0).sum(1) - 1, 0)
        gout[np.arange(B), root, :] = rng.standard_normal((B, N)).astype(np.float32)
    gout[np.isnan(cache)] = 0.0
    # drop gradients that would reach a zero denominator (the reference raises 204)
    for _ in range(4):
        try:
            _, gC, gX = ref_eval(st, X, ops, ch, C, gout)
            break
        except RuntimeError:
            # zero the gradient of tapes that contain a DIV with a zero denominator
            zero_den = np.zeros(B, bool)
            for b in range(B):
                for k in range(M):
                    if ops[b, k] == int(Operator.DIV) and (cache[b, ch[b, k, 1]] == 0).any():
                        zero_den[b] = True
            gout[zero_den] = 0.0
    np.savez_compressed(os.path.join(OUT, name + ".npz"), X=X, ops=ops, ch=ch, C=C, cache=cache,
                        gout=gout, gC=gC, gX=gX)


def case_errors(st):
    """Validation / backward error messages, as the reference raises them."""
    rows = []
    VAR = int(Operator.VAR_START_ID)
    X = np.ones((3, 2), np.float32)
    # child index >= parent
    rows.append(("child_geq", [[VAR, int(Operator.ADD)]], [[[-1, -1], [0, 2]]], "fwd"))
    # unary with no child / binary with one child / leaf with a child
    rows.append(("unary_nochild", [[int(Operator.SIN)]], [[[-1, -1]]], "fwd"))
    rows.append(("binary_onechild", [[VAR, int(Operator.MUL)]], [[[-1, -1], [0, -1]]], "fwd"))
    rows.append(("leaf_child", [[VAR, VAR]], [[[-1, -1], [0, -1]]], "fwd"))
    # backward: grad on NO_OP, and 1/0
    rows.append(("noop_grad", [[0]], [[[-1, -1]]], "bwd"))
    rows.append(("div_zero", [[int(Operator.CONST_1), VAR, int(Operator.DIV)]],
                 [[[-1, -1], [-1, -1], [0, 1]]], "bwd_x0zero"))
    out = {}
    for name, ops, ch, kind in rows:
        ops = np.array(ops, np.int64)
        ch = np.array(ch, np.int64)
        C = np.zeros(ops.shape, np.float32)
        Xc = X.copy()
        if kind == "bwd_x0zero":
            Xc[:, 0] = 0.0
        msg = ""
        try:
            cache, _, _ = ref_eval(st, Xc, ops, ch, C)
            if kind.startswith("bwd"):
                gout = np.zeros_like(cache)
                gout[:, -1, :] = 1.0
                ref_eval(st, Xc, ops, ch, C, gout)
        except RuntimeError as e:
            msg = str(e).splitlines()[0]
        out[name + "__ops"] = ops
        out[name + "__ch"] = ch
        out[name + "__X"] = Xc
        out[name + "__msg"] = np.array(msg)
    np.savez_compressed(os.path.join(OUT, "errors.npz"), **out)


def case_optimize_linear(st):
    """tests/test_optimization.py:10-80 known answer: y = c1*X0 + c2."""
    torch.manual_seed(1234)
    B, N, M = 2, 100, 5
    X = torch.randn(N, 1)
    c1 = torch.tensor([2.5, -1.5]).view(B, 1)
    c2 = torch.tensor([0.5, 3.0]).view(B, 1)
    Y = c1 * X[:, 0].T + c2
    Ops = torch.full((B, M), 0, dtype=torch.int64)
    Ops[:, 0] = int(Operator.VAR_START_ID)
    Ops[:, 1] = 1
    Ops[:, 2] = int(Operator.MUL)
    Ops[:, 3] = 1
    Ops[:, 4] = int(Operator.ADD)
    Ch = torch.full((B, M, 2), -1, dtype=torch.int64)
    Ch[:, 2, 0] = 0
    Ch[:, 2, 1] = 1
    Ch[:, 4, 0] = 2
    Ch[:, 4, 1] = 3
    C = st.create_constants(Ops, method="randn", mean=0.0, std=1.0)
    Cf, Yf = st.optimize(X, Y, Ops, Ch, C)
    np.savez_compressed(os.path.join(OUT, "optimize_linear.npz"), X=X.numpy(), Y=Y.numpy(), ops=Ops.numpy(),
                        ch=Ch.numpy(), C=C.numpy(), C_final=Cf.numpy(), Y_final=Yf.numpy())




def case_optimize_readme(st, B=128, max_iter=100):
    """The README grammar workload (plain method, small): PCFG-sampled postfix
    tapes, X = 2 randn, Y = 2.5 cos(X0) - 1.5, randn constants."""
    torch.manual_seed(0)
    pcfg = st.ProbabilisticContextFreeGrammar(README_GRAMMAR, "E", 32, 1, torch.device("cpu"))
    infix = pcfg.sample_infix(B)
    ops = pcfg.infix_to_postfix(infix)
    ch = pcfg.get_postfix_children(ops)
    X = 2 * torch.randn(100, 1)
    Y = (2.5 * torch.cos(X[:, 0]) - 1.5).unsqueeze(0).repeat(B, 1)
    C = st.create_constants(ops)
    Cf, Yf = st.optimize(X, Y, ops, ch, C, max_iter=max_iter, tolerance_grad=1e-7,
                         line_search_fn="strong_wolfe")
    infix_out = pcfg.postfix_to_infix(ops, 64)
    np.savez_compressed(os.path.join(OUT, "optimize_readme.npz"), X=X.numpy(), Y=Y.numpy(), ops=ops.numpy(),
                        ch=ch.numpy(), C=C.numpy(), C_final=Cf.numpy(), Y_final=Yf.numpy(),
                        infix=infix.numpy(), infix_from_postfix=infix_out.numpy(),
                        max_iter=np.array(max_iter))


def case_optimize_ragged(st, B=96, N=64, M=32, max_iter=40, line_search="strong_wolfe", name="optimize_ragged"):
    """Ragged tapes (lengths 3..M, 0..8 constants, 2 variables), noisy hidden targets."""
    rng = np.random.default_rng(77)
    X = rng.uniform(-3, 3, (N, 2)).astype(np.float32)
    lengths = rng.integers(3, M + 1, size=B)
    kc = rng.integers(0, 9, size=B)
    Cs = rng.standard_normal((B, M)).astype(np.float32)
    tb = tapes.generate(B, M, seed=5, lengths=lengths, const_counts=kc, n_vars=2, X_screen=X, C_screen=Cs)
    hid = tapes.generate(B, M, seed=6, lengths=rng.integers(3, 16, size=B), const_counts=rng.integers(0, 4, size=B),
                         n_vars=2, X_screen=X, C_screen=Cs)
    Ch_hidden = rng.standard_normal((B, M)).astype(np.float32)
    yh, _, _ = ref_eval(st, X, hid.ops, hid.ch, Ch_hidden)
    root = np.maximum((hid.ops != 0).sum(1) - 1, 0)
    Y = yh[np.arange(B), root] + 0.01 * rng.standard_normal((B, N)).astype(np.float32)
    Y = np.where(np.isfinite(Y), Y, 0.0).astype(np.float32)
    C = Cs.copy()
    Cf, Yf = st.optimize(torch.tensor(X), torch.tensor(Y), torch.tensor(tb.ops), torch.tensor(tb.ch),
                         torch.tensor(C), max_iter=max_iter, line_search_fn=line_search)
    np.savez_compressed(os.path.join(OUT, name + ".npz"), X=X, Y=Y, ops=tb.ops, ch=tb.ch, C=C,
                        C_final=Cf.numpy(), Y_final=Yf.numpy(), max_iter=np.array(max_iter))


def case_rosenbrock(st):
    """tests/test_lbfgs_batch.py:38-75: batched Rosenbrock from fixed starts."""
    from symbolic_torch.lbfgs_batch import LBFGS_batch
    torch.manual_seed(7)
    x0 = torch.randn(2, 10)
    res = {}
    for ls in ("strong_wolfe", "backtracking"):
        x = x0.clone().requires_grad_(True)
        opt = LBFGS_batch([x], max_iter=250, history_size=15, tolerance_grad=1e-7, line_search_fn=ls)

        def closure():
            opt.zero_grad(set_to_none=True)
            f = (1.0 - x[0]) ** 2 + 100.0 * (x[1] - x[0] ** 2) ** 2
            f.sum().backward()
            return f

        opt.step(closure)
        res[ls] = x.detach().numpy().copy()
    np.savez_compressed(os.path.join(OUT, "rosenbrock.npz"), x0=x0.numpy(), x_wolfe=res["strong_wolfe"],
                        x_backtracking=res["backtracking"])




def case_notation(st):
    """get_postfix_children / postfix_to_infix / to_string on PCFG samples and on
    generated tapes over every operator, plus the error messages of malformed rows."""
    torch.manual_seed(3)
    pcfg = st.ProbabilisticContextFreeGrammar(NOTATION_GRAMMAR, "E", 64, 2, torch.device("cpu"))
    infix = pcfg.sample_infix(400)
    post = pcfg.infix_to_postfix(infix)
    ch = pcfg.get_postfix_children(post)
    inf = pcfg.postfix_to_infix(post, 100)
    strings = pcfg.to_string(inf)
    tb = tapes.generate(300, 40, seed=21, mean_length=14, n_vars=2, unary=ALL_UNARY, binary=ALL_BINARY,
                        p_const_leaf=0.3)
    ops_all = tb.ops.copy()
    consts = np.array([2, 3, 4, 5, 6, 7, 8], np.int64)
    rng = np.random.default_rng(5)
    hard = (ops_all == 1) & (rng.random(ops_all.shape) < 0.3)
    ops_all[hard] = consts[rng.integers(0, 7, size=int(hard.sum()))]
    ch_all = pcfg.get_postfix_children(torch.tensor(ops_all))
    inf_all = pcfg.postfix_to_infix(torch.tensor(ops_all), 200)
    strings_all = pcfg.to_string(inf_all)
    V = int(Operator.VAR_START_ID)
    bad_rows = {
        "unary_missing": [10, V, 40, 0],
        "binary_missing": [V, 40, 0, 0],
        "noop_inside": [V, 0, V, 40],
        "too_many": [V, V, V, 40],
        "empty": [0, 0, 0, 0],
        "negative": [V, -3, 40, 0],
        "too_large": [V, V + 2, 40, 0],
    }
    out = {}
    for name, row in bad_rows.items():
        x = torch.tensor([row], dtype=torch.int64)
        for fn, kw in (("children", {}), ("infix", {"max_infix_len": 10})):
            try:
                if fn == "children":
                    r = pcfg.get_postfix_children(x)
                else:
                    r = pcfg.postfix_to_infix(x, 10)
                out[f"{name}__{fn}"] = r.numpy()
                out[f"{name}__{fn}_msg"] = np.array("")
            except RuntimeError as e:
                out[f"{name}__{fn}_msg"] = np.array(str(e))
        out[f"{name}__row"] = np.array([row], np.int64)
    # output exactly as long as the infix, and one token shorter
    x = torch.tensor([[V, V + 1, 40, 10]], dtype=torch.int64)
    full = pcfg.postfix_to_infix(x, 20)
    n = int((full != 0).sum())
    out["exact_len"] = pcfg.postfix_to_infix(x, n).numpy()
    try:
        pcfg.postfix_to_infix(x, n - 1)
        out["short_msg"] = np.array("")
    except RuntimeError as e:
        out["short_msg"] = np.array(str(e))
    out["exact_row"] = x.numpy()
    np.savez_compressed(os.path.join(OUT, "notation.npz"), post=post.numpy(), ch=ch.numpy(), infix=inf.numpy(),
                        strings=np.array(strings), ops_all=ops_all, ch_all=ch_all.numpy(), infix_all=inf_all.numpy(),
                        strings_all=np.array(strings_all), **out)


def case_multiple(st):
    """evaluate_multiple: K=3 constant sets, dense output gradient on every node
    (reference tests/test_evaluation_multiple_constants.py pattern)."""
    rng = np.random.default_rng(77)
    B, M, N, n_vars, K = 64, 24, 33, 3, 3
    X = rng.uniform(-3, 3, (N, n_vars)).astype(np.float32)
    tb = tapes.generate(B, M, seed=78, mean_length=10, n_vars=n_vars, p_const_leaf=0.35)
    ops, ch = tb.ops, tb.ch
    C = rng.standard_normal((B, M, K)).astype(np.float32)
    Xt = torch.tensor(X, requires_grad=True)
    Ct = torch.tensor(C, requires_grad=True)
    out = st.evaluation.evaluate_multiple(Xt, torch.tensor(ops), torch.tensor(ch), Ct)
    cache = out.detach().numpy().copy()
    gout = rng.standard_normal(cache.shape).astype(np.float32)
    gout[np.isnan(cache)] = 0.0
    for b in range(B):  # no gradient into tapes whose DIV denominators hit exact zeros
        for k in range(M):
            if ops[b, k] == int(Operator.DIV) and (cache[b, ch[b, k, 1]] == 0).any():
                gout[b] = 0.0
    out.backward(torch.tensor(gout))
    np.savez_compressed(os.path.join(OUT, "multiple.npz"), X=X, ops=ops, ch=ch, C=C, cache=cache, gout=gout,
                        gC=Ct.grad.numpy().copy(), gX=Xt.grad.numpy().copy())





def case_pcfg(st):
    """Grammar object: symbol ids, arities, valid ops and operator names for some
    grammars, the constructor's error messages, infix -> postfix / prefix of sampled
    and hand-made rows (with the error reports), and sampling frequencies of the
    reference's own sampler (src/pcfg.cpp, src/pcfg_cpu.cpp)."""
    out = {}
    names = sorted({n for n in ["NO_OP", "C", "1", "5", "pi", "PI", "e", "E", "sin", "Sin", "ln", "LN", "Ln", "log",
                                "log10", "^2", "square", "u-", "minus", "^-1", "inv", "^5", "+", "-", "*", "/", "^",
                                "X_0", "X_1", "X_2", "(", ")", "T", "F", "V", "R", "P", "asin", "atan", "floor"]})
    out["names"] = np.array(names)
    for tag, (g, start, nv) in {"readme": (README_GRAMMAR, "E", 1), "sampling": (SAMPLING_GRAMMAR, "E", 1),
                                "notation": (NOTATION_GRAMMAR, "E", 2), "wide": ("S -> 1 [1.0]", "S", 5)}.items():
        pcfg = st.ProbabilisticContextFreeGrammar(g, start, 32, nv, torch.device("cpu"))
        ids = []
        for n in names:
            try:
                ids.append(pcfg.get_symbol_id(n))
            except RuntimeError:
                ids.append(-999)
        out[f"{tag}__ids"] = np.array(ids, np.int64)
        out[f"{tag}__n_operators"] = np.array(pcfg.n_operators)
        out[f"{tag}__arities"] = pcfg.get_arities().numpy()
        out[f"{tag}__valid"] = pcfg.valid_ops().numpy()
        out[f"{tag}__available"] = np.array(sorted(pcfg.available_operators()))
    for tag, g in BAD_GRAMMARS.items():
        try:
            st.ProbabilisticContextFreeGrammar(g, "E", 16, 1, torch.device("cpu"))
            out[f"bad_{tag}__msg"] = np.array("")
        except (ValueError, RuntimeError) as e:
            out[f"bad_{tag}__msg"] = np.array(str(e))
    try:
        st.ProbabilisticContextFreeGrammar("S -> 1 [1.0]", "S", 129, 0, torch.device("cpu"))
        out["too_long__msg"] = np.array("")
    except (ValueError, RuntimeError) as e:
        out["too_long__msg"] = np.array(str(e))
    # parsing: sampled rows of the notation grammar and hand-made ones
    torch.manual_seed(17)
    pcfg = st.ProbabilisticContextFreeGrammar(NOTATION_GRAMMAR, "E", 64, 2, torch.device("cpu"))
    infix = pcfg.sample_infix(500)
    out["parse_infix"] = infix.numpy()
    out["parse_postfix"] = pcfg.infix_to_postfix(infix).numpy()
    out["parse_prefix"] = pcfg.infix_to_prefix(infix).numpy()
    V, LP, RP = 50, 52, 53
    hand = {
        "precedence": [2, 40, 2, 42, 2],
        "paren": [LP, 2, 40, 2, RP, 42, 2],
        "assoc_add": [2, 40, 2, 40, 2, 40, 2],
        "assoc_pow": [2, 44, 2, 44, 2],
        "assoc_sin": [10, 10, 10, 10, 2],
        "mixed": [10, LP, 2, RP, 40, 2],
        "all_ops": [10, LP, V, RP, 40, 2, 42, LP, 13, LP, V, RP, 41, 2, RP],
        "sub_div": [V, 41, V + 1, 43, 2, 41, 3],
        "unary_pow": [V, 44, 14, 44, 3],
        "mismatch_close": [2, RP],
        "mismatch_open": [LP, 2, 40, 2],
        "after_end": [2, 0, 2],
        "unary_missing": [10],
        "binary_missing": [2, 40],
        "too_many": [2, 2],
        "empty": [0, 0],
        "negative": [2, -4, 2],
        "too_large": [2, 40, RP + 1],
    }
    for tag, row in hand.items():
        x = torch.tensor([row + [0] * (16 - len(row))], dtype=torch.int64)
        out[f"hand_{tag}__row"] = x.numpy()
        for fn in ("postfix", "prefix"):
            try:
                r = getattr(pcfg, f"infix_to_{fn}")(x)
                out[f"hand_{tag}__{fn}"] = r.numpy()
                out[f"hand_{tag}__{fn}_msg"] = np.array("")
            except (RuntimeError, ValueError) as e:
                out[f"hand_{tag}__{fn}_msg"] = np.array(str(e))
    # a batch with several errors, and the verbose report's first lines
    batch = torch.tensor([[2, RP, 0, 0], [10, 0, 0, 0], [2, 40, 2, 0], [2, RP, 0, 0]], dtype=torch.int64)
    for verbosity in (0, 1):
        try:
            pcfg.infix_to_postfix(batch, verbosity)
        except RuntimeError as e:
            out[f"batch_v{verbosity}_msg"] = np.array(str(e))
    out["batch_rows"] = batch.numpy()
    # generation failure and frequencies of the reference sampler
    try:
        st.ProbabilisticContextFreeGrammar("S -> 1 S [1.0]", "S", 5, 0, torch.device("cpu"), max_tries=10).sample_infix(3)
    except RuntimeError as e:
        out["max_tries_msg"] = np.array(str(e))
    torch.manual_seed(23)
    sp = st.ProbabilisticContextFreeGrammar(SAMPLING_GRAMMAR, "E", 128, 1, torch.device("cpu"))
    strings = sp.to_string(sp.sample_infix(200000))
    counts = {}
    for s_ in strings:
        counts[s_] = counts.get(s_, 0) + 1
    top = sorted(counts.items(), key=lambda kv: -kv[1])[:40]
    out["freq_strings"] = np.array([k for k, _ in top])
    out["freq_counts"] = np.array([v for _, v in top], np.int64)
    out["freq_total"] = np.array(len(strings))
    lengths = np.array([len(s_.split()) for s_ in strings])
    out["freq_length_hist"] = np.bincount(lengths, minlength=129)
    torch.manual_seed(29)
    rp = st.ProbabilisticContextFreeGrammar(README_GRAMMAR, "E", 32, 1, torch.device("cpu"))
    rs = rp.to_string(rp.sample_infix(200000))
    rc = {}
    for s_ in rs:
        rc[s_] = rc.get(s_, 0) + 1
    rtop = sorted(rc.items(), key=lambda kv: -kv[1])[:40]
    out["readme_strings"] = np.array([k for k, _ in rtop])
    out["readme_counts"] = np.array([v for _, v in rtop], np.int64)
    out["readme_length_hist"] = np.bincount(np.array([len(s_.split()) for s_ in rs]), minlength=129)
    np.savez_compressed(os.path.join(OUT, "pcfg.npz"), **out)


def case_prefix(st):
    """prefix_to_postfix, prefix_to_infix and get_prefix_parent of the reference
    (src/pcfg_cpu.cpp:637-1064) on sampled expressions and on malformed rows, with the
    error reports (postfix_to_prefix is not bound by the reference's module)."""
    torch.manual_seed(19)
    pcfg = st.ProbabilisticContextFreeGrammar(NOTATION_GRAMMAR, "E", 48, 2, torch.device("cpu"))
    infix = pcfg.sample_infix(600)
    post = pcfg.infix_to_postfix(infix)
    pre = pcfg.infix_to_prefix(infix)
    out = {"post": post.numpy(), "pre": pre.numpy(),
           "pre_to_post": pcfg.prefix_to_postfix(pre).numpy(),
           "pre_to_infix": pcfg.prefix_to_infix(pre, 160).numpy(),
           "pre_parent": pcfg.get_prefix_parent(pre).numpy()}
    V = int(Operator.VAR_START_ID)
    rows = {
        "binary_missing": [40, V, 0, 0],
        "unary_missing": [10, 0, 0, 0],
        "after_end": [40, V, V, 0, V],
        "too_many": [40, V, V, V],
        "two_leaves": [V, V, 0, 0],
        "empty": [0, 0, 0, 0],
        "negative": [40, -2, V, 0],
        "too_large": [40, V, V + 2, 0],
        "unary_chain": [10, 11, 14, V],
        "nested": [42, 40, V, 2, 41, V + 1, 28],
    }
    for name, row in rows.items():
        x = torch.tensor([row], dtype=torch.int64)
        out[f"{name}__row"] = x.numpy()
        for fn, call in (("to_post", lambda t: pcfg.prefix_to_postfix(t)), ("to_infix", lambda t: pcfg.prefix_to_infix(t, 12)),
                         ("parent", lambda t: pcfg.get_prefix_parent(t))):
            try:
                out[f"{name}__{fn}"] = call(x).numpy()
                out[f"{name}__{fn}_msg"] = np.array("")
            except RuntimeError as e:
                out[f"{name}__{fn}_msg"] = np.array(str(e))
    np.savez_compressed(os.path.join(OUT, "prefix.npz"), **out)


def case_operators(st):
    """get_arity and is_valid_op of the reference for ids -3..199 and 0..5 variables,
    and the Operator enum's names and values."""
    C = sys.modules["symbolic_torch._C"]
    ids = np.arange(-3, 200)
    arity = np.array([C.get_arity(int(o)) for o in ids])
    valid = np.array([[bool(C.is_valid_op(int(o), nv)) for nv in range(6)] for o in ids])
    names = sorted(n for n, v in C.Operator.__members__.items())
    values = np.array([int(C.Operator.__members__[n]) for n in names])
    np.savez_compressed(os.path.join(OUT, "operators.npz"), ids=ids, arity=arity, valid=valid,
                        names=np.array(names), values=values)


def case_pcfg_verbose(st):
    """The grammar constructor's verbose report (std::cout, so captured from a child
    process) for the fixture grammars; max_tries 7, tolerance 1e-5 and lengths 32/48."""
    import subprocess
    out = {}
    for tag, (gram, nv, length) in {"readme": (README_GRAMMAR, 1, 32), "sampling": (SAMPLING_GRAMMAR, 1, 48),
                                    "notation": (NOTATION_GRAMMAR, 2, 32)}.items():
        code = ("import sys, torch\n"
                f"sys.path.insert(0, {os.path.join(ROOT, 'oracle')!r})\n"
                "import build_ref\n"
                "st = build_ref.load_reference()\n"
                f"st.ProbabilisticContextFreeGrammar({gram!r}, 'E', {length}, {nv}, torch.device('cpu'), "
                "max_tries=7, tolerance=1e-5, verbose=True)\n")
        lines = subprocess.run([sys.executable, "-c", code], check=True, capture_output=True,
                               text=True).stdout.splitlines()
        out[tag] = np.array(lines)
    np.savez_compressed(os.path.join(OUT, "pcfg_verbose.npz"), **out)


def case_pcfg_input_errors(st):
    """Exception type and first message line of every token-row method of the grammar
    object for inputs of the wrong rank or dtype."""
    g = st.ProbabilisticContextFreeGrammar(README_GRAMMAR, "E", 32, 1, torch.device("cpu"))
    inputs = {"0d": torch.tensor(8), "1d": torch.tensor([8, 40, 8]), "3d": torch.tensor([[[8, 40, 8]]]),
              "float": torch.tensor([[8.0, 40.0, 8.0]]), "int32": torch.tensor([[8, 40, 8]], dtype=torch.int32),
              "bool": torch.tensor([[True, False]]), "1d_float": torch.tensor([8.0, 40.0])}
    calls = {"to_string": lambda x: g.to_string(x), "infix_to_postfix": lambda x: g.infix_to_postfix(x),
             "infix_to_prefix": lambda x: g.infix_to_prefix(x), "postfix_to_infix": lambda x: g.postfix_to_infix(x, 10),
             "prefix_to_infix": lambda x: g.prefix_to_infix(x, 10), "prefix_to_postfix": lambda x: g.prefix_to_postfix(x),
             "get_prefix_parent": lambda x: g.get_prefix_parent(x),
             "get_postfix_children": lambda x: g.get_postfix_children(x)}
    rows = []
    for m, f in calls.items():
        for k, x in inputs.items():
            try:
                f(x)
                rows.append((m, k, "ok", ""))
            except Exception as e:  # the exception is the fixture
                rows.append((m, k, type(e).__name__, str(e).splitlines()[0]))
    np.savez_compressed(os.path.join(OUT, "pcfg_input_errors.npz"), rows=np.array(rows))


def case_eval_input_errors(st):
    """Exception type and first message line of evaluate and evaluate_multiple for
    malformed inputs (wrong ranks, shapes and dtypes)."""
    rows = []
    for fn, names, multiple in ((st.evaluation.evaluate, EVAL_INPUT_CASES, False),
                                (st.evaluation.evaluate_multiple, MULTI_INPUT_CASES, True)):
        for name in names:
            try:
                fn(*eval_input_case(name, multiple))
                rows.append((str(multiple), name, "ok", ""))
            except Exception as e:  # the exception is the fixture
                rows.append((str(multiple), name, type(e).__name__, str(e).splitlines()[0]))
    np.savez_compressed(os.path.join(OUT, "eval_input_errors.npz"), rows=np.array(rows))


def case_error_messages(st=None):
    """getErrorMessage of the reference (include/error_codes.h) for every code of its
    enum, the gaps between them and out-of-range values, with and without a context,
    printed by a helper compiled against the reference's header."""
    import subprocess
    exe = build_ref.build_error_messages()
    rows = [ln.split("\t") for ln in subprocess.run([exe], check=True, capture_output=True,
                                                      text=True).stdout.splitlines()]
    np.savez_compressed(os.path.join(OUT, "error_messages.npz"), code=np.array([int(r[0]) for r in rows]),
                        context=np.array([r[1] for r in rows]), message=np.array([r[2] for r in rows]))


def main():
    st = build_ref.load_reference()
    torch.set_num_threads(1)
    if len(sys.argv) > 1:  # selected cases only, e.g. `make_golden.py multiple`
        for name in sys.argv[1:]:
            globals()["case_" + name](st)
        return
    rng = np.random.default_rng(2024)
    case_single_ops(st, rng)
    case_random_dags(st, rng, "random_dags", B=160, M=24, N=37, n_vars=3, seed=11,
                     unary=ALL_UNARY, binary=ALL_BINARY, mean_length=10)
    case_random_dags(st, rng, "random_default_ops", B=128, M=64, N=70, n_vars=4, seed=12,
                     unary=tapes.UN_DEFAULT, binary=tapes.BIN_DEFAULT, mean_length=20, dense=False)
    case_errors(st)
    case_optimize_linear(st)
    case_optimize_readme(st)
    case_optimize_ragged(st)
    case_optimize_ragged(st, B=48, max_iter=30, line_search="backtracking", name="optimize_ragged_bt")
    case_rosenbrock(st)
    case_notation(st)
    case_multiple(st)
    case_pcfg(st)
    case_prefix(st)
    case_error_messages(st)
    case_operators(st)
    case_pcfg_verbose(st)
    case_pcfg_input_errors(st)
    case_eval_input_errors(st)
    for f in sorted(os.listdir(OUT)):
        if f.endswith(".npz"):
            print(f, os.path.getsize(os.path.join(OUT, f)))


if __name__ == "__main__":
    main()
