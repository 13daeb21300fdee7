"""Integer tape conversions around the fitting path, on the GPU.

Mirrors the two methods of the reference's grammar object that the fitting path
uses (src/pcfg.cpp:790-826 and 957-986): ``get_postfix_children`` builds the
``Ch`` table of postfix ``Ops``, ``postfix_to_infix`` renders postfix tapes as
infix token ids with parentheses for display, and ``to_string`` turns those ids
into text with the reference's symbol names.  Only the number of variables of the
grammar matters to them (it fixes the ids of "(" and ")" and the valid range), so
they take ``n_variables`` instead of a grammar.  Errors are raised with the
reference's messages.
"""
from __future__ import annotations

from collections import Counter

import torch

from . import _lib
from .operators import Operator, error_message

# Display names: for every id the first name the reference's symbol table registers.
_NAMES = {
    0: "NO_OP", 1: "C", 2: "1", 3: "2", 4: "3", 5: "4", 6: "5", 7: "pi", 8: "e",
    10: "sin", 11: "cos", 12: "exp", 13: "log", 14: "^2", 15: "sqrt", 16: "tan", 17: "arcsin", 18: "arccos",
    19: "arctan", 20: "sinh", 21: "cosh", 22: "tanh", 23: "floor", 24: "ceil", 25: "ln", 26: "log10", 27: "u-",
    28: "^-1", 29: "^3", 30: "^4", 31: "^5", 40: "+", 41: "-", 42: "*", 43: "/", 44: "^",
}


def paren_ids(n_variables: int):
    """Ids of "(" and ")" for a grammar with n_variables variables."""
    lp = int(Operator.VAR_START_ID) + int(n_variables)
    return lp, lp + 1


def symbol_name(token: int, n_variables: int):
    token = int(token)
    if token in _NAMES:
        return _NAMES[token]
    v = token - int(Operator.VAR_START_ID)
    if 0 <= v < n_variables:
        return f"X_{v}"
    lp, rp = paren_ids(n_variables)
    if token == lp:
        return "("
    if token == rp:
        return ")"
    return None


def _raise_for(err: torch.Tensor, context: str, check_kind: str):
    e = err.cpu()
    if (e == -1).any():
        raise RuntimeError(f"All symbols in the {check_kind} must be non-negative integers.")
    if (e == -2).any():
        raise RuntimeError(f"All symbols in the {check_kind} must be valid operator IDs.")
    if (e != 0).any():
        counts = Counter(int(c) for c in e.tolist() if c != 0)
        msg = f"Failed to parse expressions during {context} for some batch items.\nError Summary:\n"
        for code in sorted(counts):
            msg += f"  {error_message(code)}: {counts[code]} occurrences.\n"
        raise RuntimeError(msg)


def get_postfix_children(postfix_ops: torch.Tensor, n_variables: int) -> torch.Tensor:
    """(B, M) int64 left-packed postfix tapes -> (B, M, 2) int64 child table."""
    dev = _lib.require_cuda(postfix_ops)
    ops = postfix_ops.to(torch.int64).contiguous()
    B, M = ops.shape
    ch = torch.empty((B, M, 2), dtype=torch.int64, device=dev)
    err = torch.empty(B, dtype=torch.int64, device=dev)
    rc = _lib.lib().sr_postfix_children(_lib.ptr(ops), B, M, int(n_variables), _lib.ptr(ch), _lib.ptr(err),
                                        _lib.stream_ptr(dev))
    _lib.check(rc, "sr_postfix_children")
    _raise_for(err, "get postfix children", "postfix_ops")
    return ch


def postfix_to_infix(postfix_ops: torch.Tensor, max_infix_len: int, n_variables: int) -> torch.Tensor:
    """(B, M) postfix tapes -> (B, max_infix_len) infix token ids, NO_OP padded."""
    dev = _lib.require_cuda(postfix_ops)
    ops = postfix_ops.to(torch.int64).contiguous()
    B, M = ops.shape
    out = torch.empty((B, int(max_infix_len)), dtype=torch.int64, device=dev)
    err = torch.empty(B, dtype=torch.int64, device=dev)
    rc = _lib.lib().sr_postfix_to_infix(_lib.ptr(ops), B, M, int(n_variables), _lib.ptr(out), int(max_infix_len),
                                        _lib.ptr(err), _lib.stream_ptr(dev))
    _lib.check(rc, "sr_postfix_to_infix")
    _raise_for(err, "postfix to infix conversion", "prefix_ops")
    return out


def to_string(expressions: torch.Tensor, n_variables: int) -> list[str]:
    """Token ids -> text, space separated, up to the first NO_OP (unknown ids skipped)."""
    out = []
    for row in expressions.cpu().tolist():
        toks = []
        for t in row:
            if t == 0:
                break
            nm = symbol_name(t, n_variables)
            if nm is not None:
                toks.append(nm)
        out.append(" ".join(toks))
    return out
