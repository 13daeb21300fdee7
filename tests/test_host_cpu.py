"""Host-side checks that need no GPU: the C-ABI library loads and exports every
entry point include/sr_gb300.h declares, the ctypes signatures and struct mirrors
match the header's declarations, the argument checks raise the
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


def _c_kind(decl: str) -> str:
    """Kind of one C parameter or field declaration: pointer, integer width or float width."""
    d = re.sub(r"\b(const|struct)\b", " ", decl).strip()
    if "*" in d:
        return "p"
    return {"int64_t": "i64", "int32_t": "i32", "int": "i32", "uint64_t": "u64", "double": "f64",
            "float": "f32"}[d.split()[0]]


def _ctypes_kind(t) -> str:
    import ctypes
    if t in (ctypes.c_void_p, ctypes.c_char_p) or isinstance(getattr(t, "_type_", None), type):
        return "p"  # untyped pointers, strings and ctypes.POINTER(...)
    return {ctypes.c_int64: "i64", ctypes.c_int32: "i32", ctypes.c_uint64: "u64", ctypes.c_double: "f64",
            ctypes.c_float: "f32"}[t]


def _header_text():
    txt = open(os.path.join(ROOT, "include", "sr_gb300.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return re.sub(r"//[^\n]*", "", txt)


def test_ctypes_signatures_match_header():
    """Every prototype of include/sr_gb300.h against the ctypes table the package binds
    with: parameter count, and for each parameter and the result its kind (pointer,
    int32, int64, uint64, float, double), so that no argument is passed at the wrong
    width."""
    from cudasymbolicregression_gb300 import _lib
    protos = re.findall(r"([A-Za-z_][A-Za-z0-9_ ]*?[\s*]+)(sr_[a-z0-9_]+)\s*\(([^)]*)\)\s*;", _header_text())
    assert {name for _, name, _ in protos} == set(_lib._SIGS)
    for ret, name, params in protos:
        args, res = _lib._SIGS[name]
        kinds = [] if params.strip() in ("", "void") else [_c_kind(p) for p in params.split(",")]
        assert kinds == [_ctypes_kind(a) for a in args], name
        assert _c_kind(ret) == _ctypes_kind(res), name


def test_ctypes_structs_match_header():
    """sr_fit_options and sr_mlp_epilogue: field names (the header's device pointers
    carry a ``_dev`` suffix), order and kinds of the ctypes mirrors equal the header's."""
    from cudasymbolicregression_gb300 import _lib
    txt = _header_text()
    for cname, mirror in (("sr_fit_options", _lib.FitOptions), ("sr_mlp_epilogue", _lib.MlpEpilogue)):
        body = re.search(r"typedef struct[^{]*\{([^}]*)\}\s*" + cname + r"\s*;", txt).group(1)
        fields = []
        for decl in filter(None, (d.strip() for d in body.split(";"))):
            # a base type, then declarators whose own stars make them pointers
            m = re.match(r"((?:const\s+)?[A-Za-z_][A-Za-z0-9_]*)\s*(.*)$", decl)
            for d in (x.strip() for x in m.group(2).split(",")):
                kind = "p" if d.startswith("*") else _c_kind(m.group(1))
                fields.append((re.sub(r"_dev$", "", d.lstrip("* ")), kind))
        assert fields == [(n, _ctypes_kind(t)) for n, t in mirror._fields_], cname


def test_ragged_chunks_prefix_property():
    """The first chunks of a large ragged batch are the same problems as a smaller batch
    (what lets a bounded CPU sample stand for the benchmark's batch problem by problem),
    and the batch has the documented shapes: lengths 3..64, at most 8 constants."""
    from cudasymbolicregression_gb300 import workloads

    def roots(X, ops, ch, C):
        cache = oracle.eval_fwd(X, ops, ch, C)
        root = np.maximum((ops != 0).sum(1) - 1, 0)
        return cache[np.arange(ops.shape[0]), root]
    big = workloads.ragged_fit_chunks(B=1024, N=64, chunk=512, seed=3, root_eval=roots)
    small = workloads.ragged_fit_chunks(B=512, N=64, chunk=512, seed=3, root_eval=roots)
    for k in ("ops", "ch", "C", "Y"):
        np.testing.assert_array_equal(getattr(big, k)[:512], getattr(small, k), err_msg=k)
    np.testing.assert_array_equal(big.X, small.X)
    L = (big.ops != 0).sum(1)
    assert L.min() >= 3 and L.max() <= 64
    assert ((big.ops == 1).sum(1) <= 8).all()
    assert oracle.validate(big.ops, big.ch) == 0
    assert np.isfinite(big.Y).all()


def test_error_messages_match_reference_table():
    """operators.error_message for every code of the reference's ErrorCode enum, the
    gaps between them and out-of-range values, with and without a context, against
    the reference's own getErrorMessage (tests/golden/error_messages.npz, printed by a
    helper compiled against include/error_codes.h)."""
    from cudasymbolicregression_gb300.operators import error_message
    g = np.load(os.path.join(ROOT, "tests", "golden", "error_messages.npz"))
    assert len(g["code"]) > 150
    for code, ctx, msg in zip(g["code"], g["context"], g["message"]):
        assert error_message(int(code), str(ctx)) == str(msg), (int(code), str(ctx))


def test_operator_table_matches_reference_fixture():
    """get_arity and is_valid_op for ids -3..199 with 0..5 variables, and every name
    and value of the Operator enum, against the reference's own functions
    (tests/golden/operators.npz)."""
    import cudasymbolicregression_gb300 as sr
    g = np.load(os.path.join(ROOT, "tests", "golden", "operators.npz"))
    np.testing.assert_array_equal([sr.get_arity(int(o)) for o in g["ids"]], g["arity"])
    np.testing.assert_array_equal([[sr.is_valid_op(int(o), nv) for nv in range(6)] for o in g["ids"]], g["valid"])
    for name, value in zip(g["names"], g["values"]):
        assert int(getattr(sr.Operator, str(name))) == int(value), name


def test_evaluation_input_errors_match_reference():
    """evaluate and evaluate_multiple reject malformed inputs (wrong ranks, shapes,
    dtypes, mixed float types) with the reference's exception type and message
    (tests/golden/eval_input_errors.npz), before any device work."""
    import sys
    sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))
    from inputs import eval_input_case
    import cudasymbolicregression_gb300 as sr
    rows = np.load(os.path.join(ROOT, "tests", "golden", "eval_input_errors.npz"))["rows"]
    assert len(rows) > 20
    for multiple, name, etype, msg in rows:
        multiple = str(multiple) == "True"
        fn = sr.evaluation.evaluate_multiple if multiple else sr.evaluation.evaluate
        assert str(etype) != "ok"
        with pytest.raises(Exception) as e:
            fn(*eval_input_case(str(name), multiple))
        assert (type(e.value).__name__, str(e.value).splitlines()[0]) == (str(etype), str(msg)), (multiple, str(name))


def test_fit_targets_broadcast_like_the_reference():
    """optimize's targets: the reference's loss broadcasts Y against the (B, N)
    predictions, so a row (N,) or (1, N), a column (B, 1) and a scalar serve every
    expression; shapes that do not broadcast to (B, N) are rejected before any kernel
    (the fit kernel reads B x N targets)."""
    from cudasymbolicregression_gb300.optimization import _targets
    B, N = 3, 5
    full = torch.arange(B * N, dtype=torch.float64).reshape(B, N)
    for Y in (full, full[:1], full[0], full[:, :1], torch.tensor(2.0)):
        got = _targets(Y, B, N, torch.device("cpu"))
        assert got.shape == (B, N) and got.dtype == torch.float32 and got.is_contiguous()
        torch.testing.assert_close(got, torch.broadcast_to(Y, (B, N)).float())
    for Y in (full[:2], torch.zeros(N + 1), torch.zeros(B, N, 1), torch.zeros(B + 1, 1)):
        with pytest.raises(RuntimeError, match="Y must broadcast to"):
            _targets(Y, B, N, torch.device("cpu"))


def test_optimize_argument_errors_in_reference_order():
    """optimize's errors before any kernel, as the reference raises them: Ops' shape is
    unpacked first, C_init is permuted, then the line search name and the evaluation's
    checks (reference symbolic_torch/optimization.py:44-63)."""
    import cudasymbolicregression_gb300 as sr
    X, Y = torch.randn(10, 1), torch.randn(1, 10)
    ops = torch.tensor([[50, 1, 40]])
    ch = torch.tensor([[[-1, -1], [-1, -1], [0, 1]]])
    C = torch.zeros(1, 3)
    with pytest.raises(ValueError, match="not enough values to unpack"):
        sr.optimize(X, Y, ops[0], ch, C, line_search_fn="nope")
    with pytest.raises(RuntimeError, match="permute"):
        sr.optimize(X, Y, ops, ch, C[0], line_search_fn="nope")
    with pytest.raises(ValueError, match="Invalid line_search_fn"):
        sr.optimize(X, Y, ops, ch[0], C, line_search_fn="nope")
    with pytest.raises(RuntimeError, match="permute"):
        sr.optimize(X, Y, ops, ch[0], C)
    with pytest.raises(RuntimeError, match="expected scalar type Float but found Double"):
        sr.optimize(X, Y, ops, ch, C.double())
