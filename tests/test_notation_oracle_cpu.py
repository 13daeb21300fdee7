"""The oracle's restatements of the notation conversions (postfix -> infix, prefix ->
infix, prefix <-> postfix, prefix parents, child tables) against the reference's own
outputs (tests/golden/notation.npz and prefix.npz), error rows and their messages
included.  The messages are built by the package's host-side reporting from the
oracle's error codes, as they are from the device's.  No GPU needed."""
import os
import sys

import numpy as np
import pytest
import torch

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "..", "oracle"))
sys.path.insert(0, os.path.join(HERE, "golden"))

import oracle  # noqa: E402
from grammars import NOTATION_GRAMMAR  # noqa: E402

from cudasymbolicregression_gb300 import notation  # noqa: E402
from cudasymbolicregression_gb300.pcfg import ProbabilisticContextFreeGrammar  # noqa: E402


@pytest.fixture(scope="module")
def gn():
    return np.load(os.path.join(HERE, "golden", "notation.npz"))


@pytest.fixture(scope="module")
def gp():
    return np.load(os.path.join(HERE, "golden", "prefix.npz"))


def _msg(fn):
    try:
        fn()
    except RuntimeError as e:
        return str(e)
    return ""


def test_postfix_conversions_match_reference(gn):
    for key_in, key_ch, key_inf, width in (("post", "ch", "infix", 100), ("ops_all", "ch_all", "infix_all", 200)):
        inf, e1 = oracle.to_infix(gn[key_in], 2, width)
        ch, e2 = oracle.postfix_children(gn[key_in])
        assert not e1.any() and not e2.any()
        np.testing.assert_array_equal(inf, gn[key_inf])
        np.testing.assert_array_equal(ch, gn[key_ch])


def test_postfix_error_rows_match_reference(gn):
    names = sorted({k.split("__")[0] for k in gn.files if k.endswith("__row")})
    for name in names:
        row = gn[f"{name}__row"]
        ch, e_ch = oracle.postfix_children(row)
        inf, e_inf = oracle.to_infix(row, 2, 10)
        # the children restatement reports only its own codes: the symbol check of the
        # reference's wrapper (src/pcfg.cpp:644-657) comes first, as in the package
        e_sym = np.array([-1 if (r < 0).any() else (-2 if (r >= 52).any() else 0) for r in row])
        e_ch = np.where(e_sym != 0, e_sym, e_ch)
        got_ch = _msg(lambda: notation._raise_for(torch.tensor(e_ch), "get postfix children", "postfix_ops"))
        got_inf = _msg(lambda: notation._raise_for(torch.tensor(e_inf), "postfix to infix conversion", "prefix_ops"))
        assert got_ch == str(gn[f"{name}__children_msg"]), name
        assert got_inf == str(gn[f"{name}__infix_msg"]), name
        if not got_ch:
            np.testing.assert_array_equal(ch, gn[f"{name}__children"])
        if not got_inf:
            np.testing.assert_array_equal(inf, gn[f"{name}__infix"])
    # output exactly as long as the rendering, and one token shorter
    x = gn["exact_row"]
    n = int(gn["exact_len"].shape[1])
    inf, e = oracle.to_infix(x, 2, n)
    assert not e.any()
    np.testing.assert_array_equal(inf, gn["exact_len"])
    _, e = oracle.to_infix(x, 2, n - 1)
    assert _msg(lambda: notation._raise_for(torch.tensor(e), "postfix to infix conversion", "prefix_ops")) == \
        str(gn["short_msg"])


def test_prefix_conversions_match_reference(gp):
    for got, want in ((oracle.reorder(gp["pre"], 2, True), gp["pre_to_post"]),
                      (oracle.reorder(gp["post"], 2, False), gp["pre"]),
                      (oracle.to_infix(gp["pre"], 2, 160, prefix=True), gp["pre_to_infix"]),
                      (oracle.prefix_parent(gp["pre"], 2), gp["pre_parent"])):
        assert not got[1].any()
        np.testing.assert_array_equal(got[0], want)


def test_prefix_error_rows_match_reference(gp):
    p = ProbabilisticContextFreeGrammar(NOTATION_GRAMMAR, "E", 48, 2, torch.device("cpu"))
    calls = {
        "to_post": (lambda r: oracle.reorder(r, 2, True), "prefix to postfix parent conversion"),
        "to_infix": (lambda r: oracle.to_infix(r, 2, 12, prefix=True), "prefix to infix conversion"),
        "parent": (lambda r: oracle.prefix_parent(r, 2), "get prefix parent"),
    }
    tags = sorted({k.split("__")[0] for k in gp.files if k.endswith("__row")})
    for tag in tags:
        row = gp[f"{tag}__row"]
        for fn, (call, context) in calls.items():
            out, err = call(row)
            got = _msg(lambda: p._parsing_error(torch.tensor(err), torch.tensor(row), context, 0, "prefix_ops"))
            assert got == str(gp[f"{tag}__{fn}_msg"]), (tag, fn)
            if not got:
                np.testing.assert_array_equal(out, gp[f"{tag}__{fn}"], err_msg=f"{tag} {fn}")


def test_round_trips_on_random_tapes():
    """postfix -> prefix -> postfix and the two infix renderings agree on random tapes
    over every operator (the generator's tapes), with the parents consistent."""
    from cudasymbolicregression_gb300 import tapes
    from cudasymbolicregression_gb300.operators import BINARY_OPS, UNARY_OPS
    tb = tapes.generate(2000, 48, seed=41, mean_length=16, n_vars=2, unary=UNARY_OPS, binary=BINARY_OPS,
                        p_const_leaf=0.3)
    pre, e1 = oracle.reorder(tb.ops, 2, False)
    back, e2 = oracle.reorder(pre, 2, True)
    assert not e1.any() and not e2.any()
    np.testing.assert_array_equal(back, tb.ops)
    inf_post, e3 = oracle.to_infix(tb.ops, 2, 160)
    inf_pre, e4 = oracle.to_infix(pre, 2, 160, prefix=True)
    assert not e3.any() and not e4.any()
    np.testing.assert_array_equal(inf_post, inf_pre)
    par, e5 = oracle.prefix_parent(pre, 2)
    assert not e5.any()
    real = pre != 0
    assert (((par == -1) & real).sum(1) == 1).all()
    assert ((par < np.arange(pre.shape[1])) | ~real).all()


@pytest.mark.parametrize("M,n_vars", [(1, 1), (2, 1), (7, 3), (64, 1), (128, 2)])
def test_round_trips_at_edge_sizes(M, n_vars):
    """Tapes of every length 1..M (single leaves, full-width rows) over every operator:
    the child table equals the generator's, postfix -> prefix -> postfix is the
    identity, both infix renderings agree and fit in 3M tokens (each operator adds at
    most two parentheses), and every prefix node but the root has an earlier parent."""
    from cudasymbolicregression_gb300 import tapes
    from cudasymbolicregression_gb300.operators import BINARY_OPS, UNARY_OPS
    B = 400
    lengths = np.arange(B) % M + 1
    tb = tapes.generate(B, M, seed=M, lengths=lengths, n_vars=n_vars, unary=UNARY_OPS, binary=BINARY_OPS,
                        p_const_leaf=0.3)
    ch, e0 = oracle.postfix_children(tb.ops)
    assert not e0.any()
    np.testing.assert_array_equal(ch, tb.ch)
    pre, e1 = oracle.reorder(tb.ops, n_vars, False)
    back, e2 = oracle.reorder(pre, n_vars, True)
    assert not e1.any() and not e2.any()
    np.testing.assert_array_equal(back, tb.ops)
    np.testing.assert_array_equal((pre != 0).sum(1), lengths)
    inf_post, e3 = oracle.to_infix(tb.ops, n_vars, 3 * M)
    inf_pre, e4 = oracle.to_infix(pre, n_vars, 3 * M, prefix=True)
    assert not e3.any() and not e4.any()
    np.testing.assert_array_equal(inf_post, inf_pre)
    # one token short of a rendering is reported (501, too long), not truncated
    lens = (inf_post != 0).sum(1)
    _, e5 = oracle.to_infix(tb.ops, n_vars, int(lens.max()) - 1)
    np.testing.assert_array_equal(e5, np.where(lens == lens.max(), 501, 0))
    par, e6 = oracle.prefix_parent(pre, n_vars)
    assert not e6.any()
    real = pre != 0
    assert (((par == -1) & real).sum(1) == 1).all()
    assert ((par < np.arange(M)) | ~real).all()


def test_to_string_matches_reference(gn):
    """notation.to_string (host code) renders the reference's infix rows as the
    reference's own to_string does (tests/golden/notation.npz)."""
    for key_inf, key_str in (("infix", "strings"), ("infix_all", "strings_all")):
        assert notation.to_string(torch.tensor(gn[key_inf]), 2) == [str(s) for s in gn[key_str]]
