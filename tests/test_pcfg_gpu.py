"""Grammar sampling and infix parsing on the GPU, through the C ABI, against the
oracle (token for token) and the reference's own outputs (tests/golden/pcfg.npz)."""
import os
import sys

import numpy as np
import pytest
import torch

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "..", "oracle"))
sys.path.insert(0, os.path.join(HERE, "golden"))

import oracle  # noqa: E402
from grammars import NOTATION_GRAMMAR, README_GRAMMAR, SAMPLING_GRAMMAR  # noqa: E402

pytestmark = pytest.mark.gpu


def _pcfg(grammar, start, nv, length, **kw):
    from cudasymbolicregression_gb300.pcfg import ProbabilisticContextFreeGrammar
    return ProbabilisticContextFreeGrammar(grammar, start, length, nv, torch.device("cuda"), **kw)


@pytest.fixture(scope="module")
def g():
    return np.load(os.path.join(HERE, "golden", "pcfg.npz"))


def _seed_of(torch_seed):
    """The 64-bit seed sample_infix draws after torch.manual_seed(torch_seed)."""
    torch.manual_seed(torch_seed)
    return int(torch.randint(0, 2 ** 63 - 1, (1,), dtype=torch.int64).item())


@pytest.mark.parametrize("grammar,start,nv,length,B", [
    (SAMPLING_GRAMMAR, "E", 1, 128, 20000), (README_GRAMMAR, "E", 1, 32, 50000),
    (NOTATION_GRAMMAR, "E", 2, 64, 30000), (README_GRAMMAR, "E", 1, 7, 3000), (SAMPLING_GRAMMAR, "E", 1, 5, 1000)])
def test_sampler_matches_oracle_token_for_token(grammar, start, nv, length, B):
    p = _pcfg(grammar, start, nv, length, max_tries=64)
    seed = _seed_of(11)
    torch.manual_seed(11)
    try:
        got = p.sample_infix(B).cpu().numpy()
        failed = None
    except RuntimeError as e:
        got, failed = None, str(e)
    want, err = oracle.pcfg_sample(p._tables_np, p.get_symbol_id(start), B, length, 64, seed)
    if err.any():
        assert failed is not None and "max_tries" in failed
    else:
        assert failed is None
        np.testing.assert_array_equal(got, want)


def test_sampler_batch_edges():
    """B = 1, a partial last CTA, and B = 0."""
    p = _pcfg(README_GRAMMAR, "E", 1, 32)
    for B in (1, 129, 0):
        seed = _seed_of(3)
        torch.manual_seed(3)
        got = p.sample_infix(B).cpu().numpy()
        want, _ = oracle.pcfg_sample(p._tables_np, p.get_symbol_id("E"), B, 32, 64, seed)
        assert got.shape == (B, 32)
        np.testing.assert_array_equal(got, want)


@pytest.mark.parametrize("length,max_tries,B", [(7, 3, 5000), (7, 0, 777), (32, 64, 33), (12, 2, 100003),
                                                 (5, 1, 4097)])
def test_sampler_rows_and_error_codes_through_the_c_abi(length, max_tries, B):
    """Every row and every error word of the C ABI equal the oracle's, failed expressions
    included (rows of NO_OP, 303 after max_tries failed tries, 303 at once for
    max_tries = 0): the sampler's lanes take the expressions of their warp's range one
    after another, so batch sizes that leave ragged ranges are covered too."""
    from cudasymbolicregression_gb300 import _lib
    p = _pcfg(README_GRAMMAR, "E", 1, length, max_tries=max(max_tries, 1))
    nt, cum, rp, rc = p._tables
    start = p.get_symbol_id("E")
    seed = 0x5EED1234ABCDEF
    out = torch.full((B, length), 77, dtype=torch.int64, device="cuda")
    err = torch.full((B,), 77, dtype=torch.int64, device="cuda")
    L = _lib.lib()
    _lib.check(L.sr_pcfg_sample_infix(_lib.ptr(nt), _lib.ptr(cum), _lib.ptr(rp), _lib.ptr(rc), int(nt.numel() - 1),
                                      start, B, length, max_tries, seed, _lib.ptr(out), _lib.ptr(err),
                                      _lib.stream_ptr(torch.device("cuda"))), "sr_pcfg_sample_infix")
    want, want_err = oracle.pcfg_sample(p._tables_np, start, B, length, max_tries, seed)
    got_err = err.cpu().numpy()
    np.testing.assert_array_equal(got_err, want_err)
    np.testing.assert_array_equal(out.cpu().numpy(), want)
    if max_tries == 0:
        assert (got_err == 303).all()
    elif length == 7:
        assert 0 < (got_err == 303).sum() < B  # some expressions fail, most do not


def test_reference_sampling_patterns(g):
    """tests/test_sampling.py of the reference: one-rule grammars, 50/50 rules, and
    the max_tries error."""
    for gram, nv, tok, text in (("S -> 1 [1.0]", 0, 2, "1"), ("S -> C [1.0]", 0, 1, "C"),
                                ("S -> X_4 [1.0]", 10, 54, "X_4")):
        p = _pcfg(gram, "S", nv, 1)
        s = p.sample_infix(10)
        assert s.shape == (10, 1) and (s == tok).all()
        assert set(p.to_string(s)) == {text}
    for op, code in (("exp", 12), ("sin", 10), ("cos", 11)):
        p = _pcfg(f"S -> {op} ( 1 ) [0.5]\nS -> 1 [0.5]", "S", 0, 5)
        s = p.sample_infix(1000)
        assert (s == code).sum() > 400 and (s == 2).sum() > 400
        assert all(op in t or t == "1" for t in p.to_string(s))
    for sym, code in (("+", 40), ("-", 41), ("*", 42), ("/", 43), ("^", 44)):
        p = _pcfg(f"S -> 1 {sym} 1 [0.5]\nS -> 1 [0.5]", "S", 0, 3)
        s = p.sample_infix(1000)
        assert torch.any(s == code, dim=1).sum() > 400 and (s == 2).sum() > 1400
    p = _pcfg("S -> 1 S [1.0]", "S", 0, 5, max_tries=10)
    with pytest.raises(RuntimeError) as e:
        p.sample_infix(3)
    assert str(e.value) == str(g["max_tries_msg"])


def test_sampling_frequencies_match_reference(g):
    """200000 device samples against the reference's own sampler: the 20 most
    frequent expressions within 5 standard deviations, length histograms within
    0.01 in total variation."""
    p = _pcfg(SAMPLING_GRAMMAR, "E", 1, 128)
    torch.manual_seed(41)
    strings = p.to_string(p.sample_infix(200000))
    n, n_ref = len(strings), int(g["freq_total"])
    counts = {}
    for s in strings:
        counts[s] = counts.get(s, 0) + 1
    for s, c in list(zip(g["freq_strings"], g["freq_counts"]))[:20]:
        pr, po = c / n_ref, counts.get(str(s), 0) / n
        assert abs(po - pr) < 5 * np.sqrt(pr * (1 - pr) * (1 / n + 1 / n_ref)), str(s)
    ours = np.bincount(np.array([len(s.split()) for s in strings]), minlength=129)[:129] / n
    ref = g["freq_length_hist"][:129] / g["freq_length_hist"].sum()
    assert 0.5 * np.abs(ours - ref).sum() < 0.01


def test_parser_matches_reference(g):
    p = _pcfg(NOTATION_GRAMMAR, "E", 2, 64)
    infix = torch.tensor(g["parse_infix"]).cuda()
    np.testing.assert_array_equal(p.infix_to_postfix(infix).cpu().numpy(), g["parse_postfix"])
    np.testing.assert_array_equal(p.infix_to_prefix(infix).cpu().numpy(), g["parse_prefix"])
    tags = sorted({k.split("__")[0][5:] for k in g.files if k.startswith("hand_")})
    for tag in tags:
        row = torch.tensor(g[f"hand_{tag}__row"]).cuda()
        for fn in ("postfix", "prefix"):
            want = str(g[f"hand_{tag}__{fn}_msg"])
            try:
                out = getattr(p, f"infix_to_{fn}")(row)
                assert want == "", (tag, fn)
                np.testing.assert_array_equal(out.cpu().numpy(), g[f"hand_{tag}__{fn}"], err_msg=f"{tag} {fn}")
            except RuntimeError as e:
                assert str(e) == want, (tag, fn)
    with pytest.raises(RuntimeError) as e:
        p.infix_to_postfix(torch.tensor(g["batch_rows"]).cuda())
    assert str(e.value) == str(g["batch_v0_msg"])
    with pytest.raises(ValueError, match="HARD_MAX_LENGTH"):
        p.infix_to_postfix(torch.zeros(2, 129, dtype=torch.int64, device="cuda"))


def test_parser_matches_oracle_on_large_batches():
    """Every sampled row of a large batch, both directions, plus rows damaged at
    random positions (the error codes and NO_OP rows must agree too)."""
    p = _pcfg(NOTATION_GRAMMAR, "E", 2, 64)
    torch.manual_seed(5)
    infix = p.sample_infix(40000)
    rng = np.random.default_rng(0)
    x = infix.cpu().numpy()
    bad = rng.random(x.shape[0]) < 0.2
    pos = rng.integers(0, 8, x.shape[0])
    x[bad, pos[bad]] = rng.choice([10, 40, 52, 53, 0, 2], size=int(bad.sum()))
    xd = torch.tensor(x).cuda()
    lib = __import__("cudasymbolicregression_gb300._lib", fromlist=["lib"])
    for prefix in (False, True):
        out = torch.empty_like(xd)
        err = torch.empty(x.shape[0], dtype=torch.int64, device="cuda")
        fn = lib.lib().sr_infix_to_prefix if prefix else lib.lib().sr_infix_to_postfix
        assert fn(lib.ptr(xd), x.shape[0], x.shape[1], 2, lib.ptr(out), lib.ptr(err), lib.stream_ptr(xd.device)) == 0
        want, werr = oracle.infix_parse(x, 2, prefix=prefix)
        np.testing.assert_array_equal(err.cpu().numpy(), werr)
        np.testing.assert_array_equal(out.cpu().numpy(), want)
        assert (werr != 0).any() and (werr == 0).any()


def test_sample_pipeline_feeds_the_fit():
    """sample(B): postfix Ops and the child table on the device, equal to the
    separate steps; the batch then evaluates and fits."""
    import cudasymbolicregression_gb300 as sr
    p = _pcfg(README_GRAMMAR, "E", 1, 32)
    torch.manual_seed(9)
    ops, ch = p.sample(4096)
    torch.manual_seed(9)
    infix = p.sample_infix(4096)
    post = p.infix_to_postfix(infix)
    assert torch.equal(ops, post)
    assert torch.equal(ch, p.get_postfix_children(post))
    assert ops.device.type == "cuda" and ch.shape == (4096, 32, 2)
    X = torch.linspace(-2, 2, 100, device="cuda").reshape(100, 1)
    Y = (2.5 * torch.cos(X[:, 0]) - 1.5).expand(4096, 100).contiguous()
    C0 = sr.create_constants(ops)
    r = sr.optimize_ex(X, Y, ops, ch, C0, max_iter=50, raise_errors=False)
    best = torch.nan_to_num(r.loss, nan=float("inf")).min()
    assert float(best) < 1e-6  # the batch holds C * cos(X_0) + C-like forms


def test_postfix_infix_round_trip():
    """postfix -> infix (with the renderer's parentheses) -> postfix is the identity
    (32-token expressions render to at most 96 tokens)."""
    p = _pcfg(NOTATION_GRAMMAR, "E", 2, 32)
    torch.manual_seed(13)
    post, _ = p.sample(5000)
    inf = p.postfix_to_infix(post, 128)
    back = p.infix_to_postfix(inf)
    assert torch.equal(back[:, :32], post)
    assert (back[:, 32:] == 0).all()


def test_prefix_conversions_match_reference():
    """prefix_to_postfix, prefix_to_infix and get_prefix_parent against the
    reference's outputs (tests/golden/prefix.npz), with its error reports;
    postfix_to_prefix (not bound by the reference's module) must invert them."""
    gp = np.load(os.path.join(HERE, "golden", "prefix.npz"))
    p = _pcfg(NOTATION_GRAMMAR, "E", 2, 48)
    pre = torch.tensor(gp["pre"]).cuda()
    post = torch.tensor(gp["post"]).cuda()
    np.testing.assert_array_equal(p.prefix_to_postfix(pre).cpu().numpy(), gp["pre_to_post"])
    np.testing.assert_array_equal(p.prefix_to_infix(pre, 160).cpu().numpy(), gp["pre_to_infix"])
    np.testing.assert_array_equal(p.get_prefix_parent(pre).cpu().numpy(), gp["pre_parent"])
    np.testing.assert_array_equal(p.postfix_to_prefix(post).cpu().numpy(), gp["pre"])
    calls = {"to_post": lambda t: p.prefix_to_postfix(t), "to_infix": lambda t: p.prefix_to_infix(t, 12),
             "parent": lambda t: p.get_prefix_parent(t)}
    tags = sorted({k.split("__")[0] for k in gp.files if k.endswith("__row")})
    for tag in tags:
        row = torch.tensor(gp[f"{tag}__row"]).cuda()
        for fn, call in calls.items():
            want = str(gp[f"{tag}__{fn}_msg"])
            try:
                out = call(row)
                assert want == "", (tag, fn)
                np.testing.assert_array_equal(out.cpu().numpy(), gp[f"{tag}__{fn}"], err_msg=f"{tag} {fn}")
            except RuntimeError as e:
                assert str(e) == want, (tag, fn)


def test_prefix_round_trips_on_large_batches():
    p = _pcfg(NOTATION_GRAMMAR, "E", 2, 64)
    torch.manual_seed(21)
    infix = p.sample_infix(30000)
    post = p.infix_to_postfix(infix)
    pre = p.infix_to_prefix(infix)
    assert torch.equal(p.postfix_to_prefix(post), pre)
    assert torch.equal(p.prefix_to_postfix(pre), post)
    assert torch.equal(p.prefix_to_infix(pre, 200), p.postfix_to_infix(post, 200))
    par = p.get_prefix_parent(pre)
    # every non-root node's parent precedes it; exactly one root per expression
    idx = torch.arange(pre.shape[1], device="cuda").expand_as(pre)
    real = pre != 0
    assert ((par < idx) | ~real).all()
    assert (((par == -1) & real).sum(1) == 1).all()


def test_infix_rendering_length_limits():
    """The reference's length cases (tests/test_to_infix.py:258-340): nested logs
    rendered exactly at the output length in both notations, one token short raising
    501, and 30 nested logs from the 128-token grammar."""
    p = _pcfg(NOTATION_GRAMMAR, "E", 2, 64)
    X0, LOG, LP, RP = 50, 13, 52, 53
    for depth, width in ((3, 10), (5, 16)):
        want = [LOG, LP] * depth + [X0] + [RP] * depth
        for fn, row in (("postfix_to_infix", [X0] + [LOG] * depth), ("prefix_to_infix", [LOG] * depth + [X0])):
            x = torch.tensor([row], device="cuda")
            assert getattr(p, fn)(x, width)[0].tolist() == want, fn
            with pytest.raises(RuntimeError, match="longer than the maximum allowed length"):
                getattr(p, fn)(x, width - 1)
    p128 = _pcfg(NOTATION_GRAMMAR, "E", 2, 128)
    out = p128.postfix_to_infix(torch.tensor([[X0] + [LOG] * 30], device="cuda"), 91)
    assert out[0].tolist() == [LOG, LP] * 30 + [X0] + [RP] * 30


def test_notation_kernels_match_oracle_on_random_rows():
    """Every conversion kernel against the oracle's restatement on 20000 random tapes
    over every operator, a fifth of them damaged at a random position: error codes on
    every row, outputs on the rows without an error."""
    from cudasymbolicregression_gb300 import _lib, tapes
    from cudasymbolicregression_gb300.operators import BINARY_OPS, UNARY_OPS
    tb = tapes.generate(20000, 48, seed=43, mean_length=16, n_vars=2, unary=UNARY_OPS, binary=BINARY_OPS,
                        p_const_leaf=0.3)
    rng = np.random.default_rng(44)
    post = tb.ops.copy()
    bad = rng.random(post.shape[0]) < 0.2
    pos = rng.integers(0, 20, post.shape[0])
    post[bad, pos[bad]] = rng.choice([0, 10, 40, 50, 2, -3, 60], size=int(bad.sum()))
    pre, _ = oracle.reorder(tb.ops, 2, False)
    pre[bad, pos[bad]] = post[bad, pos[bad]]
    L = _lib.lib()
    B, M = post.shape

    def device(fn, x, width=None, last=2):
        xd = torch.tensor(x).cuda()
        shape = (B, M, 2) if last == 3 else (B, width if width is not None else M)
        out = torch.empty(shape, dtype=torch.int64, device="cuda")
        err = torch.empty(B, dtype=torch.int64, device="cuda")
        args = [_lib.ptr(xd), B, M, 2, _lib.ptr(out)] + ([width] if width is not None else [])
        assert getattr(L, fn)(*args, _lib.ptr(err), _lib.stream_ptr(xd.device)) == 0
        return out.cpu().numpy(), err.cpu().numpy()

    cases = [
        (device("sr_postfix_to_infix", post, 160), oracle.to_infix(post, 2, 160)),
        (device("sr_prefix_to_infix", pre, 160), oracle.to_infix(pre, 2, 160, prefix=True)),
        (device("sr_prefix_to_postfix", pre), oracle.reorder(pre, 2, True)),
        (device("sr_postfix_to_prefix", post), oracle.reorder(post, 2, False)),
        (device("sr_prefix_parent", pre), oracle.prefix_parent(pre, 2)),
    ]
    for i, ((got, gerr), (want, werr)) in enumerate(cases):
        np.testing.assert_array_equal(gerr, werr, err_msg=f"case {i}")
        ok = werr == 0
        assert ok.any() and (~ok).any()
        np.testing.assert_array_equal(got[ok], want[ok], err_msg=f"case {i}")
    got, gerr = device("sr_postfix_children", post, last=3)
    want, werr = oracle.postfix_children(post)
    sym = np.array([-1 if (r < 0).any() else (-2 if (r >= 52).any() else 0) for r in post])
    np.testing.assert_array_equal(gerr, np.where(sym != 0, sym, werr))
    ok = gerr == 0
    np.testing.assert_array_equal(got[ok], want[ok])
