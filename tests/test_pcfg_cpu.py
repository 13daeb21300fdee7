"""Grammar object on the host and the oracle's sampler and parser, against the
reference's own outputs (tests/golden/pcfg.npz, written by make_golden.py from the
reference's CPU path).  No GPU needed."""
import os
import sys

import numpy as np
import pytest
import torch

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "..", "oracle"))
sys.path.insert(0, os.path.join(HERE, "golden"))

import oracle  # noqa: E402
from grammars import BAD_GRAMMARS, NOTATION_GRAMMAR, README_GRAMMAR, SAMPLING_GRAMMAR  # noqa: E402

from cudasymbolicregression_gb300.pcfg import ProbabilisticContextFreeGrammar  # noqa: E402

GRAMMARS = {"readme": (README_GRAMMAR, "E", 1), "sampling": (SAMPLING_GRAMMAR, "E", 1),
            "notation": (NOTATION_GRAMMAR, "E", 2), "wide": ("S -> 1 [1.0]", "S", 5)}


@pytest.fixture(scope="module")
def g():
    return np.load(os.path.join(HERE, "golden", "pcfg.npz"))


def _pcfg(grammar, start, nv, length=32, **kw):
    return ProbabilisticContextFreeGrammar(grammar, start, length, nv, torch.device("cpu"), **kw)


def test_symbol_tables_match_reference(g):
    names = [str(n) for n in g["names"]]
    for tag, (gram, start, nv) in GRAMMARS.items():
        p = _pcfg(gram, start, nv)
        ids = []
        for n in names:
            try:
                ids.append(p.get_symbol_id(n))
            except RuntimeError:
                ids.append(-999)
        np.testing.assert_array_equal(ids, g[f"{tag}__ids"], err_msg=tag)
        assert p.n_operators == int(g[f"{tag}__n_operators"])
        np.testing.assert_array_equal(p.get_arities().numpy(), g[f"{tag}__arities"])
        np.testing.assert_array_equal(p.valid_ops().numpy(), g[f"{tag}__valid"])
        assert sorted(p.available_operators()) == [str(s) for s in g[f"{tag}__available"]]


def test_grammar_errors_match_reference(g):
    for tag, gram in BAD_GRAMMARS.items():
        with pytest.raises(ValueError) as e:
            _pcfg(gram, "E", 1, 16)
        assert str(e.value) == str(g[f"bad_{tag}__msg"]), tag
    with pytest.raises(ValueError) as e:
        _pcfg("S -> 1 [1.0]", "S", 0, 129)
    assert str(e.value) == str(g["too_long__msg"])
    with pytest.raises(RuntimeError, match="Symbol not found: nothing"):
        _pcfg("S -> 1 [1.0]", "S", 0).get_symbol_id("nothing")


def test_properties_are_read_only():
    p = _pcfg("S -> 1 [1.0]", "S", 5, 32, max_tries=99, tolerance=1e-5, verbose=False)
    assert (p.start_symbol, p.padded_maximum_length, p.n_variables, p.max_tries) == ("S", 32, 5, 99)
    assert abs(p.tolerance - 1e-5) < 1e-9 and p.verbose is False and p.device == torch.device("cpu")
    for name, value in (("start_symbol", "E"), ("padded_maximum_length", 64), ("n_variables", 1),
                        ("max_tries", 3), ("tolerance", 0.1), ("verbose", True), ("device", "cuda")):
        with pytest.raises(AttributeError):
            setattr(p, name, value)


def test_oracle_parser_matches_reference(g):
    infix = g["parse_infix"]
    post, e1 = oracle.infix_parse(infix, 2)
    pre, e2 = oracle.infix_parse(infix, 2, prefix=True)
    assert not e1.any() and not e2.any()
    np.testing.assert_array_equal(post, g["parse_postfix"])
    np.testing.assert_array_equal(pre, g["parse_prefix"])


def _message_for(p, err, rows, fn, verbosity=0):
    try:
        p._parsing_error(torch.tensor(err), torch.tensor(rows), f"{fn} parsing", verbosity, "infix_ops")
    except RuntimeError as e:
        return str(e)
    return ""


def test_oracle_hand_rows_and_messages(g):
    p = _pcfg(NOTATION_GRAMMAR, "E", 2, 64)
    tags = sorted({k.split("__")[0][5:] for k in g.files if k.startswith("hand_")})
    for tag in tags:
        row = g[f"hand_{tag}__row"]
        for fn in ("postfix", "prefix"):
            out, err = oracle.infix_parse(row, 2, prefix=fn == "prefix")
            msg = _message_for(p, err, row, fn)
            assert msg == str(g[f"hand_{tag}__{fn}_msg"]), (tag, fn)
            if not msg:
                np.testing.assert_array_equal(out, g[f"hand_{tag}__{fn}"], err_msg=f"{tag} {fn}")


def test_batch_error_report(g):
    p = _pcfg(NOTATION_GRAMMAR, "E", 2, 64)
    rows = g["batch_rows"]
    _, err = oracle.infix_parse(rows, 2)
    assert _message_for(p, err, rows, "postfix") == str(g["batch_v0_msg"])
    # the verbose report: the same lines up to each tensor print (whose layout is the host library's)
    ours = _message_for(p, err, rows, "postfix", verbosity=1).split("\n")
    ref = str(g["batch_v1_msg"]).split("\n")
    keep = lambda lines: [ln for ln in lines if ln and not ln.startswith("  Expression Tensor") and not ln.startswith("[")]
    assert keep(ours) == keep(ref)


def _tables(p):
    return p._tables_np


def _frequencies(p, strings):
    c = {}
    for s in strings:
        c[s] = c.get(s, 0) + 1
    return c


@pytest.mark.parametrize("tag,grammar,seed", [("freq", SAMPLING_GRAMMAR, 5), ("readme", README_GRAMMAR, 6)])
def test_oracle_sampler_distribution_matches_reference(g, tag, grammar, seed):
    """The restated sampler over this library's tables draws the reference's
    distribution: the 20 most frequent expressions within 5 standard deviations of
    the reference's frequencies over 200000 samples, and the length histograms
    within 0.01 in total variation."""
    length = 128 if tag == "freq" else 32
    p = _pcfg(grammar, "E", 1, length)
    n = 200000
    rows, err = oracle.pcfg_sample(_tables(p), p.get_symbol_id("E"), n, length, 64, seed)
    assert not err.any()
    strings = p.to_string(torch.tensor(rows))
    ours = _frequencies(p, strings)
    key_s, key_c = ("freq_strings", "freq_counts") if tag == "freq" else ("readme_strings", "readme_counts")
    n_ref = int(g["freq_total"])
    for s, c in list(zip(g[key_s], g[key_c]))[:20]:
        pr, po = c / n_ref, ours.get(str(s), 0) / n
        sd = np.sqrt(pr * (1 - pr) / n + pr * (1 - pr) / n_ref)
        assert abs(po - pr) < 5 * sd + 1e-12, (str(s), po, pr)
    hist_key = "freq_length_hist" if tag == "freq" else "readme_length_hist"
    ours_h = np.bincount(np.array([len(s.split()) for s in strings]), minlength=129)[:129] / n
    ref_h = g[hist_key][:129] / g[hist_key].sum()
    assert 0.5 * np.abs(ours_h - ref_h).sum() < 0.01


def test_oracle_sampler_max_tries(g):
    p = _pcfg("S -> 1 S [1.0]", "S", 0, 5, max_tries=10)
    rows, err = oracle.pcfg_sample(_tables(p), p.get_symbol_id("S"), 3, 5, 10, 1)
    assert (err == 303).all() and (rows == 0).all()
    with pytest.raises(RuntimeError) as e:
        p._generation_error(torch.tensor(err))
    assert str(e.value) == str(g["max_tries_msg"])


def test_oracle_sampler_fixed_grammars():
    """The reference's one-rule grammars (tests/test_sampling.py:46-84)."""
    for gram, nv, tok in (("S -> 1 [1.0]", 0, 2), ("S -> C [1.0]", 0, 1), ("S -> X_3 [1.0]", 10, 53)):
        p = _pcfg(gram, "S", nv, 1)
        rows, err = oracle.pcfg_sample(_tables(p), p.get_symbol_id("S"), 10, 1, 64, 3)
        assert not err.any() and (rows == tok).all()
        assert set(p.to_string(torch.tensor(rows))) == {gram.split()[2]}


def test_gpu_entry_points_have_no_cpu_path():
    p = _pcfg("S -> 1 [1.0]", "S", 0, 1)
    with pytest.raises(RuntimeError):
        p.sample_infix(4)
    with pytest.raises(RuntimeError):
        p.infix_to_postfix(torch.zeros(2, 3, dtype=torch.int64))


def test_oracle_postfix_children_matches_reference():
    """The oracle's child table (the CPU baseline of the sampling workload) against the
    reference's get_postfix_children on its own fixtures."""
    gn = np.load(os.path.join(HERE, "golden", "notation.npz"))
    for key_in, key_out in (("post", "ch"), ("ops_all", "ch_all")):
        ch, err = oracle.postfix_children(gn[key_in])
        assert not err.any()
        np.testing.assert_array_equal(ch, gn[key_out])


@pytest.mark.parametrize("tag,length", [("readme", 32), ("sampling", 48), ("notation", 32)])
def test_verbose_report_matches_reference(tag, length, capsys):
    """The constructor's verbose report against the reference's own output
    (tests/golden/pcfg_verbose.npz): the same header lines in the same order; the same
    symbol lines, which the reference lists in its hash map's order and this class by
    id; the same rules under each left-hand side, in the same order where the grammar
    has at most 16 rules (beyond that the reference's unstable sort may reorder rules
    with equal left-hand sides, and this class keeps the grammar's order)."""
    want = [str(s) for s in np.load(os.path.join(HERE, "golden", "pcfg_verbose.npz"))[tag]]
    gram, start, nv = GRAMMARS[tag]
    ProbabilisticContextFreeGrammar(gram, start, length, nv, torch.device("cpu"), max_tries=7, tolerance=1e-5,
                                    verbose=True)
    got = capsys.readouterr().out.splitlines()

    def split(lines):
        sym = [ln for ln in lines if ln.startswith("\tSymbol: ")]
        rules = [ln.split(": ", 1)[1] for ln in lines if ln.startswith("\tRule ")]
        rest = [ln for ln in lines if not ln.startswith(("\tSymbol: ", "\tRule "))]
        return rest, sym, rules
    (g_rest, g_sym, g_rules), (w_rest, w_sym, w_rules) = split(got), split(want)
    assert g_rest == w_rest
    assert sorted(g_sym) == sorted(w_sym)
    ids = [int(ln.rsplit("ID: ", 1)[1]) for ln in g_sym]
    assert ids == sorted(ids)
    assert [r.split(" -> ")[0] for r in g_rules] == [r.split(" -> ")[0] for r in w_rules]
    assert sorted(g_rules) == sorted(w_rules)
    if len(w_rules) <= 16:
        assert g_rules == w_rules


def test_token_row_input_errors_match_reference():
    """Every token-row method rejects inputs of the wrong rank or dtype with the
    reference's exception type and message (tests/golden/pcfg_input_errors.npz), before
    any device work, so the check runs here on CPU tensors."""
    rows = np.load(os.path.join(HERE, "golden", "pcfg_input_errors.npz"))["rows"]
    g = ProbabilisticContextFreeGrammar(README_GRAMMAR, "E", 32, 1, torch.device("cpu"))
    inputs = {"0d": torch.tensor(8), "1d": torch.tensor([8, 40, 8]), "3d": torch.tensor([[[8, 40, 8]]]),
              "float": torch.tensor([[8.0, 40.0, 8.0]]), "int32": torch.tensor([[8, 40, 8]], dtype=torch.int32),
              "bool": torch.tensor([[True, False]]), "1d_float": torch.tensor([8.0, 40.0])}
    calls = {"to_string": lambda x: g.to_string(x), "infix_to_postfix": lambda x: g.infix_to_postfix(x),
             "infix_to_prefix": lambda x: g.infix_to_prefix(x), "postfix_to_infix": lambda x: g.postfix_to_infix(x, 10),
             "prefix_to_infix": lambda x: g.prefix_to_infix(x, 10), "prefix_to_postfix": lambda x: g.prefix_to_postfix(x),
             "get_prefix_parent": lambda x: g.get_prefix_parent(x),
             "get_postfix_children": lambda x: g.get_postfix_children(x)}
    assert len(rows) == len(calls) * len(inputs)
    for method, kind, etype, msg in rows:
        assert etype != "ok", (method, kind)
        with pytest.raises(Exception) as e:
            calls[str(method)](inputs[str(kind)])
        assert (type(e.value).__name__, str(e.value)) == (str(etype), str(msg)), (str(method), str(kind))
