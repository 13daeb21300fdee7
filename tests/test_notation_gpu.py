"""GPU parity of the integer conversions (bit-exact) against the reference's own
outputs: get_postfix_children, postfix_to_infix, to_string and their errors."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _nt():
    from cudasymbolicregression_gb300 import notation
    return notation


def test_children_bit_exact(golden):
    nt = _nt()
    g = golden("notation")
    for ops, ref in ((g["post"], g["ch"]), (g["ops_all"], g["ch_all"])):
        got = nt.get_postfix_children(torch.tensor(ops).cuda(), 2).cpu().numpy()
        np.testing.assert_array_equal(got, ref)


def test_postfix_to_infix_bit_exact(golden):
    nt = _nt()
    g = golden("notation")
    for ops, ref, strings, width in ((g["post"], g["infix"], g["strings"], 100),
                                     (g["ops_all"], g["infix_all"], g["strings_all"], 200)):
        got = nt.postfix_to_infix(torch.tensor(ops).cuda(), width, 2)
        np.testing.assert_array_equal(got.cpu().numpy(), ref)
        assert nt.to_string(got, 2) == [str(s) for s in strings]


def test_readme_workload_infix(golden):
    """The optimize fixture's PCFG-sampled tapes (one variable)."""
    nt = _nt()
    g = golden("optimize_readme")
    got = nt.postfix_to_infix(torch.tensor(g["ops"]).cuda(), 64, 1).cpu().numpy()
    np.testing.assert_array_equal(got, g["infix_from_postfix"])
    ch = nt.get_postfix_children(torch.tensor(g["ops"]).cuda(), 1).cpu().numpy()
    np.testing.assert_array_equal(ch, g["ch"])


@pytest.mark.parametrize("name", ["unary_missing", "binary_missing", "noop_inside", "too_many", "empty",
                                  "negative", "too_large"])
def test_error_behaviour(golden, name):
    nt = _nt()
    g = golden("notation")
    row = torch.tensor(g[name + "__row"]).cuda()
    for fn in ("children", "infix"):
        msg = str(g[f"{name}__{fn}_msg"])
        call = (lambda: nt.get_postfix_children(row, 2)) if fn == "children" else \
            (lambda: nt.postfix_to_infix(row, 10, 2))
        if name == "empty" and fn == "children":
            # the reference's CUDA kernel reports an all-NO_OP row as malformed (407);
            # its CPU path (where the fixture comes from) returns an empty child table
            with pytest.raises(RuntimeError, match="Malformed expression"):
                call()
            continue
        if msg:
            with pytest.raises(RuntimeError) as e:
                call()
            assert str(e.value) == msg
        else:
            np.testing.assert_array_equal(call().cpu().numpy(), g[f"{name}__{fn}"])


def test_output_length_limits(golden):
    nt = _nt()
    g = golden("notation")
    row = torch.tensor(g["exact_row"]).cuda()
    n = g["exact_len"].shape[1]
    np.testing.assert_array_equal(nt.postfix_to_infix(row, n, 2).cpu().numpy(), g["exact_len"])
    with pytest.raises(RuntimeError) as e:
        nt.postfix_to_infix(row, n - 1, 2)
    assert str(e.value) == str(g["short_msg"])


def test_children_full_size_matches_generator():
    """262144 generated tapes of length <= 64: the child table equals the one the
    generator built with its own operand stack."""
    from cudasymbolicregression_gb300 import tapes
    nt = _nt()
    rng = np.random.default_rng(0)
    B = 262144
    tb = tapes.generate(B, 64, seed=2, lengths=rng.integers(1, 65, size=B), n_vars=3)
    got = nt.get_postfix_children(torch.tensor(tb.ops).cuda(), 3).cpu().numpy()
    np.testing.assert_array_equal(got, tb.ch)
    inf = nt.postfix_to_infix(torch.tensor(tb.ops[:4096]).cuda(), 3 * 128, 3).cpu().numpy()
    # parentheses balance and one token per non-parenthesis node
    lp, rp = nt.paren_ids(3)
    assert ((inf == lp).sum(1) == (inf == rp).sum(1)).all()
    assert (((inf != 0) & (inf != lp) & (inf != rp)).sum(1) == tb.lengths[:4096]).all()


def test_generation_to_evaluation_pipeline():
    """Sample -> child table -> evaluate (the reference's end-to-end smoke,
    tests/test_generation_evaluation.py): expressions of the README grammar, their
    child table rebuilt on the device, evaluated to a (B, M, N) cache."""
    import cudasymbolicregression_gb300 as sr
    from cudasymbolicregression_gb300 import workloads
    wl = workloads.readme_fit(B=512, seed=5)
    ops = torch.tensor(wl.ops).cuda()
    ch = sr.notation.get_postfix_children(ops, n_variables=1)
    assert torch.equal(ch.cpu(), torch.tensor(wl.ch))
    out = sr.evaluation.evaluate(torch.tensor(wl.X).cuda(), ops, ch, torch.tensor(wl.C).cuda())
    assert out.shape == (512, wl.ops.shape[1], wl.X.shape[0])
