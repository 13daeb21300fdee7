"""Host-side checks that need no GPU: the C-ABI library loads and exports every
entry point include/sr_gb300.h declares, the argument checks raise the
reference's messages, and the tape generator emits valid postfix tapes."""
import os
import re

import numpy as np
import pytest
import torch

import oracle

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_functions():
    txt = open(os.path.join(ROOT, "include", "sr_gb300.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(sr_[a-z0-9_]+)\s*\(", txt)))


def test_library_exports_every_declared_symbol():
    from cudasymbolicregression_gb300 import _lib
    lib = _lib.load()
    names = header_functions()
    assert len(names) >= 10
    for n in names:
        assert hasattr(lib, n), n
    assert set(names) == set(_lib.exported_symbols())
    assert b"sm_103a" in lib.sr_version()


def test_operator_table_matches_reference():
    import cudasymbolicregression_gb300 as sr
    O = sr.Operator
    assert (int(O.NO_OP), int(O.LEARNABLE_CONSTANT), int(O.SIN), int(O.FIFTH), int(O.ADD), int(O.POW),
            int(O.VAR_START_ID)) == (0, 1, 10, 31, 40, 44, 50)
    for op in range(0, 70):
        exp = 1 if 10 <= op <= 31 else 2 if 40 <= op <= 44 else 0
        assert sr.get_arity(op) == exp
    assert not sr.is_valid_op(0, 2)
    assert sr.is_valid_op(51, 2) and not sr.is_valid_op(52, 2)
    assert not sr.is_valid_op(9, 2) and not sr.is_valid_op(35, 2)


def test_error_messages():
    from cudasymbolicregression_gb300.operators import error_message
    assert error_message(101, "input validation") == (
        "Error during input validation: Validation failed: A child's index is greater than or equal to its parent's.")
    assert error_message(204, "symbolic evaluation backward pass").endswith("Gradient for a/b where b = 0.")
    assert error_message(504) == "Unknown error code: 504"


def test_dtype_errors_before_any_kernel():
    """reference tests/test_symbolic_evaluation.py:326-340 (messages), on CPU tensors."""
    from cudasymbolicregression_gb300.evaluation import evaluate_backend
    X = torch.randn(10, 2)
    ops = torch.tensor([[50]], dtype=torch.int64)
    ch = -torch.ones(1, 1, 2, dtype=torch.int64)
    C = torch.zeros(1, 1)
    with pytest.raises(RuntimeError, match="X must be a floating-point tensor"):
        evaluate_backend(X.to(torch.int32), ops, ch, C)
    with pytest.raises(RuntimeError, match="must be a Long tensor"):
        evaluate_backend(X, ops.float(), ch, C)
    with pytest.raises(RuntimeError, match="must be a Long tensor"):
        evaluate_backend(X, ops, ch.float(), C)
    with pytest.raises(RuntimeError, match="C must be a floating-point tensor"):
        evaluate_backend(X, ops, ch, C.to(torch.int32))
    with pytest.raises(RuntimeError, match="Ch must have MaxArity"):
        evaluate_backend(X, ops, -torch.ones(1, 1, 3, dtype=torch.int64), C)
    # valid CPU inputs: there is no CPU path, the call says so
    with pytest.raises(RuntimeError, match="CUDA tensors only"):
        evaluate_backend(X, ops, ch, C)


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_tape_generator_valid_postfix(seed):
    from cudasymbolicregression_gb300 import tapes
    rng = np.random.default_rng(seed)
    B, M = 500, 64
    lengths = rng.integers(1, M + 1, size=B)
    kc = rng.integers(0, 9, size=B)
    tb = tapes.generate(B, M, seed=seed, lengths=lengths, const_counts=kc, n_vars=3)
    assert oracle.validate(tb.ops, tb.ch) == 0
    real = tb.ops != 0
    L = real.sum(1)
    np.testing.assert_array_equal(L, lengths)
    # left-packed: every real node precedes every NO_OP
    assert all(real[b, :L[b]].all() and not real[b, L[b]:].any() for b in range(B))
    # postfix stack discipline: each node is the child of exactly one later node, except the root
    for b in range(0, B, 37):
        used = np.zeros(M, int)
        for k in range(L[b]):
            for c in tb.ch[b, k]:
                if c >= 0:
                    used[c] += 1
        assert (used[:L[b] - 1] == 1).all() and used[L[b] - 1] == 0
    np.testing.assert_array_equal(tb.n_consts, np.minimum(kc, (tb.ops == 1).sum(1)))


def test_tape_generator_screens_zero_denominators():
    from cudasymbolicregression_gb300 import tapes
    rng = np.random.default_rng(0)
    X = rng.uniform(-3, 3, (16, 1)).astype(np.float32)
    C = rng.standard_normal((400, 16)).astype(np.float32)
    tb = tapes.generate(400, 16, seed=3, mean_length=9, n_vars=1, X_screen=X, C_screen=C)
    cache = oracle.eval_fwd(X, tb.ops, tb.ch, C)
    for b in range(400):
        for k in range(16):
            if tb.ops[b, k] == 43:
                assert not (cache[b, tb.ch[b, k, 1]] == 0).any()
