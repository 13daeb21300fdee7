"""Operator vocabulary of the postfix tape and the reference's error vocabulary.

The integer codes are the reference's ``enum Operator`` (include/operators.h:10-59);
``Ops`` tensors built for the reference evaluate unchanged here.  Arity follows
``get_arity`` (include/operators.h:118-125): codes 10..31 are unary, 40..44 binary,
everything else (leaves, NO_OP, unknown codes) has arity 0.  Variables are
``VAR_START_ID + i``.
"""
from __future__ import annotations

import enum


class Operator(enum.IntEnum):
    NO_OP = 0
    LEARNABLE_CONSTANT = 1
    CONST_1 = 2
    CONST_2 = 3
    CONST_3 = 4
    CONST_4 = 5
    CONST_5 = 6
    PI = 7
    E = 8
    SIN = 10
    COS = 11
    EXP = 12
    LOG = 13
    SQUARE = 14
    SQRT = 15
    TAN = 16
    ARCSIN = 17
    ARCCOS = 18
    ARCTAN = 19
    SINH = 20
    COSH = 21
    TANH = 22
    FLOOR = 23
    CEIL = 24
    LN = 25
    LOG10 = 26
    NEG = 27
    INV = 28
    CUBE = 29
    FOURTH = 30
    FIFTH = 31
    ADD = 40
    SUB = 41
    MUL = 42
    DIV = 43
    POW = 44
    VAR_START_ID = 50


MAX_ARITY = 2
NULL_CHILD = -1

UNARY_OPS = tuple(int(o) for o in Operator if 10 <= int(o) <= 31)
BINARY_OPS = tuple(int(o) for o in Operator if 40 <= int(o) <= 44)


def get_arity(op: int) -> int:
    """Number of children of ``op`` (reference: operators.h:118-125)."""
    op = int(op)
    if int(Operator.SIN) <= op <= int(Operator.FIFTH):
        return 1
    if int(Operator.ADD) <= op <= int(Operator.POW):
        return 2
    return 0


def is_valid_op(op: int, n_variables: int) -> bool:
    """True for every defined operator and for variables below ``n_variables``
    (reference: operators.h:66-116).  NO_OP is not a valid operator."""
    op = int(op)
    if op == int(Operator.NO_OP):
        return False
    if op in _DEFINED:
        return True
    v = int(Operator.VAR_START_ID)
    return v <= op < v + int(n_variables)


_DEFINED = frozenset(int(o) for o in Operator if o not in (Operator.NO_OP, Operator.VAR_START_ID))


class ErrorCode(enum.IntEnum):
    """Numeric status codes shared with the C-ABI (reference: include/error_codes.h:14-63)."""
    NO_ERROR = 0
    VALIDATION_CHILD_INDEX_GEQ_PARENT = 101
    VALIDATION_ARITY_MISMATCH = 102
    EVAL_BACKWARD_GRAD_ON_NO_OP = 201
    EVAL_BACKWARD_DIV_BY_ZERO = 204
    PARSING_TREE_UNARY_OP_MISSING_OPERAND = 404
    PARSING_TREE_BINARY_OP_MISSING_OPERANDS = 405
    PARSING_TREE_CHILD_STACK_OVERFLOW = 406
    PARSING_TREE_MALFORMED_EXPRESSION = 407
    PARSING_UNEXPECTED_TOKEN = 408
    CONVERSION_RESULTING_INFIX_TOO_LONG = 501
    CONVERSION_INTERNAL_STACK_OVERFLOW = 504
    CONVERSION_UNARY_OP_MISSING_OPERAND = 505
    CONVERSION_BINARY_OP_MISSING_OPERANDS = 506
    CONVERSION_MALFORMED_EXPRESSION = 507
    CONVERSION_MULTIPLE_ROOTS = 508
    CONVERSION_UNEXPECTED_TOKEN = 509
    INTERNAL_ERROR = 1000


# Message texts are part of the drop-in contract: the reference's tests match them
# (reference: include/error_codes.h:72-195).
_MESSAGES = {
    0: "No error.",
    101: "Validation failed: A child's index is greater than or equal to its parent's.",
    102: "Validation failed: Operator arity does not match the number of children.",
    201: "Backward pass error: A non-zero gradient was passed to a NO_OP node.",
    204: "Backward pass error: Gradient for a/b where b = 0.",
    301: "Generation failed: Internal stack exceeded capacity.",
    302: "Generation failed: Produced expression exceeded maximum length.",
    303: "Generation failed: Could not produce a valid expression within the max_tries limit.",
    304: "Generation failed: No valid production rule found during sampling.",
    401: "Parsing failed: Output queue overflowed (expression likely too complex).",
    402: "Parsing failed: Operator stack overflowed (expression likely too complex).",
    403: "Parsing failed: Mismatched or unbalanced parentheses.",
    404: "Parsing failed: Unary operator is missing an operand during tree construction.",
    405: "Parsing failed: Binary operator is missing one or both operands during tree construction.",
    406: "Parsing failed: Child stack overflowed during tree construction.",
    407: "Parsing failed: Malformed expression (e.g., too many operands).",
    408: "Parsing failed: Unexpected token encountered during parsing.",
    501: "Conversion failed: Resulting infix expression is longer than the maximum allowed length.",
    502: "Conversion failed: Resulting postfix expression is longer than the maximum allowed length.",
    503: "Conversion failed: Resulting prefix expression is longer than the maximum allowed length.",
    505: "Conversion failed: Malformed input, unary operator is missing an operand.",
    506: "Conversion failed: Malformed input, binary operator is missing one or both operands.",
    507: "Conversion failed: Malformed input (e.g., too many operands).",
    508: "Conversion failed: Resulting infix expression has multiple roots, which is not allowed.",
    509: "Conversion failed: Unexpected token encountered (e.g., an operator without operands).",
    1000: "An internal error occurred that does not fit into the above categories.",
}


# torch's names of its scalar types, as its "expected scalar type" errors print them
_SCALAR_NAMES = {"torch.float32": "Float", "torch.float64": "Double", "torch.float16": "Half",
                 "torch.bfloat16": "BFloat16", "torch.int64": "Long", "torch.int32": "Int", "torch.int16": "Short",
                 "torch.int8": "Char", "torch.uint8": "Byte", "torch.bool": "Bool",
                 "torch.complex64": "ComplexFloat", "torch.complex128": "ComplexDouble"}


def scalar_type_name(dtype) -> str:
    """The name torch's C++ type checks print for a torch dtype ("Float", "Long", ...)."""
    return _SCALAR_NAMES.get(str(dtype), str(dtype))


def error_message(code: int, context: str = "") -> str:
    """Human-readable text for a status code, optionally prefixed with
    ``"Error during <context>: "`` as the reference's getErrorMessage does."""
    code = int(code)
    base = _MESSAGES.get(code, f"Unknown error code: {code}")
    return f"Error during {context}: {base}" if context else base
