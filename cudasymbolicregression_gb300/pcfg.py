"""The reference's grammar object, ``ProbabilisticContextFreeGrammar``, with its
sampling and parsing on the GPU.

Mirrors the class of the reference (src/pcfg.cpp, include/pcfg.h; bound in
src/pcfg.cpp:1006-1061): the constructor parses the grammar text on the host with
the reference's symbol table, rules and error messages and builds its CSR tables
(rules sorted by left-hand side, cumulative probabilities per non-terminal, the
concatenated right-hand sides), which then live on the device.  ``sample_infix``
draws expressions on the device, each lane deriving one expression at a time
(``sr_pcfg_sample_infix``);
``infix_to_postfix`` / ``infix_to_prefix`` run the shunting-yard on the device
(``sr_infix_to_postfix`` / ``sr_infix_to_prefix``); ``get_postfix_children`` and
``postfix_to_infix`` are the kernels of :mod:`.notation`.  ``sample(B)`` chains
sampling, parsing and the child table on the device with one host
synchronisation at the end (a two-number summary of the error words per kernel; the
words themselves are copied only to report an error), which is what a search loop
feeds to the fit.

Random numbers: one SplitMix64 stream per expression from a 64-bit seed drawn
from torch's default generator, so ``torch.manual_seed`` fixes the samples (the
reference seeds curand the same way, from ``torch.randint``).  The streams
differ from curand's, so samples equal the reference's in distribution, not
token for token.

There is no CPU path: the grammar can be built for any device, but sampling and
parsing need a CUDA device.
"""
from __future__ import annotations

from collections import Counter

import numpy as np
import torch

from . import _lib, notation
from .operators import Operator, error_message, get_arity, is_valid_op, scalar_type_name

HARD_MAX_LENGTH = 128  # include/pcfg_kernels.h:4
DEFAULT_TOLERANCE = 1e-6  # include/pcfg.h:25


def _check_token_rows(x: torch.Tensor, accessor_only: bool = False) -> None:
    """The reference's checks of a (B, M) int64 token tensor, in its order and with its
    exceptions: the methods read ``size(0)`` and ``size(1)`` first (IndexError below two
    dimensions), then take a two-dimensional int64 accessor; ``to_string`` takes the
    accessor only (src/pcfg.cpp:660-986)."""
    if not accessor_only and x.dim() == 0:
        raise IndexError("Dimension specified as 0 but tensor has no dimensions")
    if not accessor_only and x.dim() == 1:
        raise IndexError("Dimension out of range (expected to be in range of [-1, 0], but got 1)")
    if x.dim() != 2:
        raise RuntimeError(f"TensorAccessor expected 2 dims but tensor has {x.dim()}")
    if x.dtype != torch.int64:
        raise RuntimeError(f"expected scalar type Long but found {scalar_type_name(x.dtype)}")


def _terminal_symbols(n_variables: int):
    """(name, id) pairs in the order the reference registers them
    (src/pcfg.cpp:44-181); a later name overrides an earlier one for lookup, the
    first name of an id is its display name."""
    O = Operator
    pairs = [("NO_OP", O.NO_OP), ("C", O.LEARNABLE_CONSTANT), ("1", O.CONST_1), ("2", O.CONST_2),
             ("3", O.CONST_3), ("4", O.CONST_4), ("5", O.CONST_5), ("pi", O.PI), ("PI", O.PI), ("e", O.E),
             ("E", O.E)]
    for names, op in ((("sin", "SIN", "Sin"), O.SIN), (("cos", "COS", "Cos"), O.COS),
                      (("exp", "EXP", "Exp"), O.EXP), (("log", "LOG", "Log", "ln", "LN", "Ln"), O.LOG),
                      (("^2", "square", "SQUARE", "Square"), O.SQUARE), (("sqrt", "SQRT", "Sqrt"), O.SQRT),
                      (("tan", "TAN", "Tan"), O.TAN), (("arcsin", "ARCSIN", "asin", "ASIN"), O.ARCSIN),
                      (("arccos", "ARCCOS", "acos", "ACOS"), O.ARCCOS),
                      (("arctan", "ARCTAN", "atan", "ATAN"), O.ARCTAN), (("sinh", "SINH", "Sinh"), O.SINH),
                      (("cosh", "COSH", "Cosh"), O.COSH), (("tanh", "TANH", "Tanh"), O.TANH),
                      (("floor", "FLOOR", "Floor"), O.FLOOR), (("ceil", "CEIL", "Ceil"), O.CEIL),
                      (("ln", "LN"), O.LN), (("log10", "LOG10"), O.LOG10),
                      (("u-", "neg", "NEG", "minus"), O.NEG), (("^-1", "inv", "INV"), O.INV),
                      (("^3", "cube", "CUBE", "Cube"), O.CUBE), (("^4", "fourth", "FOURTH", "Fourth"), O.FOURTH),
                      (("^5", "fifth", "FIFTH", "Fifth"), O.FIFTH), (("+",), O.ADD), (("-",), O.SUB),
                      (("*",), O.MUL), (("/",), O.DIV), (("^",), O.POW)):
        pairs += [(n, op) for n in names]
    v = int(O.VAR_START_ID)
    pairs += [(f"X_{i}", v + i) for i in range(n_variables)]
    pairs += [("(", v + n_variables), (")", v + n_variables + 1)]
    return [(n, int(i)) for n, i in pairs]


class ProbabilisticContextFreeGrammar:
    """A probabilistic context-free grammar over the reference's operator tokens.

    ``grammar`` has one rule per line, ``LHS -> RHS tokens [probability]``; tokens
    are separated by spaces; every non-terminal's probabilities sum to 1 within
    ``tolerance``.  Expressions are at most ``padded_maximum_length`` infix tokens
    (<= 128).  Errors in the grammar raise ValueError with the reference's messages
    (src/pcfg.cpp:274-470).
    """

    def __init__(self, grammar: str, start_symbol: str, padded_maximum_length: int, n_variables: int,
                 device, max_tries: int = 64, tolerance: float = DEFAULT_TOLERANCE, verbose: bool = False):
        if padded_maximum_length > HARD_MAX_LENGTH:
            raise ValueError(f"padded_maximum_length must be less than or equal to HARD_MAX_LENGTH "
                             f"({HARD_MAX_LENGTH})")
        self._device = torch.device(device)
        self._start_symbol = str(start_symbol)
        self._padded_maximum_length = int(padded_maximum_length)
        self._n_variables = int(n_variables)
        self._max_tries = int(max_tries)
        self._tolerance = float(np.float32(tolerance))
        self._verbose = bool(verbose)
        self._symbol_to_id: dict[str, int] = {}
        self._id_to_symbol: dict[int, str] = {}
        for name, i in _terminal_symbols(self._n_variables):
            self._add_symbol(name, i)
        v = int(Operator.VAR_START_ID)
        self._n_operators = v + self._n_variables
        self._terminal_limit = v + self._n_variables + 2
        self._next_id = self._terminal_limit

        lhs_ids, rhss, probs = [], [], []
        for raw in grammar.split("\n"):
            line = raw.strip()
            if not line:
                continue
            arrow = line.find("->")
            if arrow < 0:
                raise ValueError("Invalid grammar rule: " + line)
            lhs = line[:arrow].strip()
            if not lhs:
                raise ValueError("LHS cannot be empty in rule: " + line)
            rest = line[arrow + 2:].strip()
            if "->" in rest:
                raise ValueError("Invalid grammar rule with multiple '->': " + line)
            bracket = rest.find("[")
            if bracket < 0:
                raise ValueError("Invalid grammar rule without probability: " + line)
            rhs = rest[:bracket].strip()
            prob_str = rest[bracket + 1:]
            if not prob_str.endswith("]"):
                raise ValueError("Invalid grammar rule with missing ']': " + line)
            if prob_str.count("]") > 1:
                raise ValueError("Invalid grammar rule with multiple ']' characters: " + line)
            prob = float(np.float32(float(prob_str[:-1].strip())))
            lhs_tokens = [self._token_id(t) for t in lhs.split()]
            if len(lhs_tokens) != 1:
                raise ValueError("LHS must contain exactly one non-terminal: " + lhs)
            rhs_tokens = [self._token_id(t) for t in rhs.split()]
            if not rhs_tokens:
                raise ValueError("RHS cannot be empty: " + rhs)
            lhs_ids.append(lhs_tokens[0])
            rhss.append(rhs_tokens)
            probs.append(prob)

        # CSR tables (src/pcfg.cpp:362-451): rules sorted by left-hand side
        order = sorted(range(len(lhs_ids)), key=lambda i: lhs_ids[i])
        lhs_sorted = [lhs_ids[i] for i in order]
        rhs_sorted = [rhss[i] for i in order]
        prob_sorted = [probs[i] for i in order]
        if not lhs_sorted:
            raise ValueError("No rules found in the grammar.")
        n_sym = self._next_id
        nt_ptr = np.searchsorted(np.asarray(lhs_sorted, np.int64), np.arange(n_sym + 1), side="left").astype(np.int32)
        cum = np.zeros(len(lhs_sorted), np.float32)
        for s in range(n_sym):
            a, b = int(nt_ptr[s]), int(nt_ptr[s + 1])
            if a == b:
                continue
            total = 0.0
            for j in range(a, b):
                total += prob_sorted[j]
            if abs(total - 1.0) > self._tolerance:
                raise ValueError(f"Non-terminal '{self._id_to_symbol[s]}' does not sum to 1.0. "
                                 f"Total probability: {total:.6f}.")
            acc = 0.0
            for j in range(a, b):
                acc += prob_sorted[j]
                cum[j] = acc
            cum[b - 1] = 1.0
        for s in range(self._terminal_limit, n_sym):
            if nt_ptr[s] == nt_ptr[s + 1]:
                raise ValueError(f"Symbol {self._id_to_symbol[s]} with ID {s} has no rules and is not a terminal.")
        rhs_ptr = np.zeros(len(rhs_sorted) + 1, np.int32)
        rhs_ptr[1:] = np.cumsum([len(r) for r in rhs_sorted])
        rhs_concat = np.asarray([t for r in rhs_sorted for t in r], np.int32)
        self._tables_np = (nt_ptr, cum, rhs_ptr, rhs_concat)
        self._tables = tuple(torch.tensor(a, device=self._device) for a in self._tables_np)
        self._rules = (lhs_sorted, rhs_sorted, prob_sorted)
        if self._verbose:
            self._describe()

    # ---- symbol table ----------------------------------------------------------------
    def _add_symbol(self, name: str, i: int) -> None:
        self._symbol_to_id[name] = i
        self._id_to_symbol.setdefault(i, name)

    def _token_id(self, name: str) -> int:
        if not name:
            raise ValueError("Symbol cannot be empty.")
        if name not in self._symbol_to_id:
            self._add_symbol(name, self._next_id)
            self._next_id += 1
        return self._symbol_to_id[name]

    def _describe(self) -> None:
        """The constructor's verbose report (src/pcfg.cpp:473-499).  Numbers print as a
        C++ stream prints a float (six significant digits); the symbol lines come in id
        order, where the reference lists its hash map in that map's own order."""
        lhs, rhs, prob = self._rules
        print(f"ProbabilisticContextFreeGrammar initialized with {len(lhs)} rules.")
        print(f"\tStart symbol: {self._start_symbol}, ID: {self._symbol_to_id.get(self._start_symbol)}")
        print(f"\tMaximum length: {self._padded_maximum_length}")
        print(f"\tNumber of variables: {self._n_variables}")
        print(f"\tDevice: {self._device}")
        print(f"\tMax tries: {self._max_tries}")
        print(f"\tTolerance: {self._tolerance:g}")
        for name, i in sorted(self._symbol_to_id.items(), key=lambda kv: (kv[1], kv[0])):
            print(f"\tSymbol: {name}, ID: {i}")
        print("Processed grammar rules:")
        for k in range(len(lhs)):
            body = "".join(self._id_to_symbol[t] + " " for t in rhs[k])
            print(f"\tRule {k + 1}: {self._id_to_symbol[lhs[k]]} -> {body}[{prob[k]:g}]")

    # ---- read-only attributes (include/pcfg.h; bound read-only in src/pcfg.cpp:1045-1057)
    device = property(lambda self: self._device)
    start_symbol = property(lambda self: self._start_symbol)
    padded_maximum_length = property(lambda self: self._padded_maximum_length)
    n_variables = property(lambda self: self._n_variables)
    max_tries = property(lambda self: self._max_tries)
    tolerance = property(lambda self: self._tolerance)
    verbose = property(lambda self: self._verbose)
    n_operators = property(lambda self: self._n_operators)

    def get_symbol_id(self, symbol: str) -> int:
        """Id of a symbol; RuntimeError("Symbol not found: ...") otherwise."""
        if symbol not in self._symbol_to_id:
            raise RuntimeError("Symbol not found: " + symbol)
        return self._symbol_to_id[symbol]

    def get_arities(self) -> torch.Tensor:
        """(n_operators,) int64 arity of every operator id (include/pcfg.h:74-82)."""
        return torch.tensor([get_arity(i) for i in range(self._n_operators)], dtype=torch.int64, device=self._device)

    def valid_ops(self) -> torch.Tensor:
        """(n_operators,) bool: which ids are operators for this number of variables."""
        return torch.tensor([is_valid_op(i, self._n_variables) for i in range(self._n_operators)], dtype=torch.bool,
                            device=self._device)

    def available_operators(self) -> list[str]:
        """Every symbol name whose id is an operator id (src/pcfg.cpp:988-1000)."""
        return [n for n, i in self._symbol_to_id.items() if i < self._n_operators]

    def to_string(self, expressions: torch.Tensor) -> list[str]:
        """Token rows -> text, space separated, up to the first NO_OP; ids without a
        name are skipped (src/pcfg.cpp:760-788)."""
        _check_token_rows(expressions, accessor_only=True)
        out = []
        for row in expressions.cpu().tolist():
            toks = []
            for t in row:
                if t == int(Operator.NO_OP):
                    break
                nm = self._id_to_symbol.get(int(t))
                if nm is not None:
                    toks.append(nm)
            out.append(" ".join(toks))
        return out

    # ---- sampling ----------------------------------------------------------------------
    def _start_id(self) -> int:
        if self._start_symbol not in self._symbol_to_id:
            raise ValueError(f"Start symbol '{self._start_symbol}' does not occur in the grammar.")
        return self._symbol_to_id[self._start_symbol]

    def _launch_sample(self, B: int, out: torch.Tensor, err: torch.Tensor) -> None:
        dev = _lib.require_cuda(out)
        nt, cum, rp, rc = self._tables
        seed = int(torch.randint(0, 2 ** 63 - 1, (1,), dtype=torch.int64).item())
        rc_ = _lib.lib().sr_pcfg_sample_infix(_lib.ptr(nt), _lib.ptr(cum), _lib.ptr(rp), _lib.ptr(rc), int(nt.numel() - 1),
                                              self._start_id(), int(B), self._padded_maximum_length, self._max_tries,
                                              seed, _lib.ptr(out), _lib.ptr(err), _lib.stream_ptr(dev))
        _lib.check(rc_, "sr_pcfg_sample_infix")

    @staticmethod
    def _generation_error(err_cpu: torch.Tensor) -> None:
        if (err_cpu != 0).any():
            counts = Counter(int(c) for c in err_cpu.tolist() if c != 0)
            msg = "Failed to generate expressions for some batch items. Error counts:\n"
            for code in sorted(counts):
                msg += f"  {error_message(code)}: {counts[code]} occurrences.\n"
            raise RuntimeError(msg)

    @staticmethod
    def _any_error(errs: torch.Tensor) -> bool:
        """Whether any per-row error word is nonzero, from the smallest and largest word of
        each row of errs (one small device-to-host copy instead of all B words)."""
        lo, hi = torch.aminmax(errs, dim=-1)
        return bool(torch.stack((lo, hi)).ne(0).any().cpu())

    def sample_infix(self, B: int) -> torch.Tensor:
        """(B, padded_maximum_length) int64 infix token rows, NO_OP padded."""
        B = int(B)
        out = torch.empty((B, self._padded_maximum_length), dtype=torch.int64, device=self._device)
        err = torch.empty(B, dtype=torch.int64, device=self._device)
        if B:
            self._launch_sample(B, out, err)
            if self._any_error(err):  # the full words only to report them
                self._generation_error(err.cpu())
        return out

    def sample(self, B: int):
        """Sample B expressions and return them as the fit takes them: postfix Ops
        (B, padded_maximum_length) int64 and their child table Ch (B, L, 2), all on
        the device with one host synchronisation (the error check) at the end."""
        B, L = int(B), self._padded_maximum_length
        dev = self._device
        infix = torch.empty((B, L), dtype=torch.int64, device=dev)
        post = torch.empty((B, L), dtype=torch.int64, device=dev)
        ch = torch.empty((B, L, 2), dtype=torch.int64, device=dev)
        errs = torch.zeros((3, B), dtype=torch.int64, device=dev)
        if B == 0:
            return post, ch
        self._launch_sample(B, infix, errs[0])
        st = _lib.stream_ptr(dev)
        lib = _lib.lib()
        _lib.check(lib.sr_infix_to_postfix(_lib.ptr(infix), B, L, self._n_variables, _lib.ptr(post),
                                           _lib.ptr(errs[1]), st), "sr_infix_to_postfix")
        _lib.check(lib.sr_postfix_children(_lib.ptr(post), B, L, self._n_variables, _lib.ptr(ch), _lib.ptr(errs[2]),
                                           st), "sr_postfix_children")
        if self._any_error(errs):  # the full words only to report them
            e = errs.cpu()
            self._generation_error(e[0])
            self._parsing_error(e[1], infix, "postfix parsing", 0, "infix_ops")
            self._parsing_error(e[2], post, "get postfix children", 0, "postfix_ops")
        return post, ch

    # ---- parsing and conversions -------------------------------------------------------
    def _parsing_error(self, err_cpu: torch.Tensor, expressions: torch.Tensor, context: str, verbosity: int,
                       check_kind: str) -> None:
        """The reference's checks and error report (src/pcfg.cpp:504-566, 630-657)."""
        if (err_cpu == -1).any():
            raise RuntimeError(f"All symbols in the {check_kind} must be non-negative integers.")
        if (err_cpu == -2).any():
            what = ("terminal symbols (less than terminal_limit)" if check_kind == "infix_ops"
                    else "valid operator IDs")
            raise RuntimeError(f"All symbols in the {check_kind} must be {what}.")
        if not (err_cpu != 0).any():
            return
        counts = Counter(int(c) for c in err_cpu.tolist() if c != 0)
        msg = f"Failed to parse expressions during {context} for some batch items.\nError Summary:\n"
        for code in sorted(counts):
            msg += f"  {error_message(code)}: {counts[code]} occurrences.\n"
        if verbosity > 0:
            bad = torch.nonzero(err_cpu).flatten().tolist()
            limit = min(5, len(bad)) if verbosity == 1 else len(bad)
            msg += f"\nDisplaying {limit} out of {len(bad)} problematic expressions:\n"
            rows = expressions.cpu()
            for i in bad[:limit]:
                msg += "----------------------------------------\n"
                msg += f"Problem at Index: {i}\n"
                msg += f"  Error: {error_message(int(err_cpu[i]))}\n"
                msg += f"  Input Expression: '{self.to_string(rows[i:i + 1])[0]}'\n"
                msg += f"  Expression Tensor: {rows[i:i + 1]}\n"
            if len(bad) > limit:
                msg += "----------------------------------------\n"
                msg += f"... and {len(bad) - limit} more.\n"
        raise RuntimeError(msg)

    def _parse(self, expressions: torch.Tensor, prefix: bool, verbosity: int) -> torch.Tensor:
        _check_token_rows(expressions)
        dev = _lib.require_cuda(expressions)
        x = expressions.to(torch.int64).contiguous()
        B, M = x.shape
        if M > HARD_MAX_LENGTH:
            raise ValueError(f"M must be less than or equal to HARD_MAX_LENGTH, but got {M} > {HARD_MAX_LENGTH}.")
        out = torch.empty((B, M), dtype=torch.int64, device=dev)
        err = torch.zeros(B, dtype=torch.int64, device=dev)
        fn = _lib.lib().sr_infix_to_prefix if prefix else _lib.lib().sr_infix_to_postfix
        _lib.check(fn(_lib.ptr(x), B, M, self._n_variables, _lib.ptr(out), _lib.ptr(err), _lib.stream_ptr(dev)),
                   "sr_infix_to_prefix" if prefix else "sr_infix_to_postfix")
        self._parsing_error(err.cpu(), x, "prefix parsing" if prefix else "postfix parsing", verbosity, "infix_ops")
        return out

    def infix_to_postfix(self, expressions: torch.Tensor, verbosity: int = 0) -> torch.Tensor:
        """(B, M) infix token rows -> (B, M) postfix, NO_OP padded."""
        return self._parse(expressions, False, verbosity)

    def infix_to_prefix(self, expressions: torch.Tensor, verbosity: int = 0) -> torch.Tensor:
        """(B, M) infix token rows -> (B, M) prefix, NO_OP padded."""
        return self._parse(expressions, True, verbosity)

    def postfix_to_infix(self, expressions: torch.Tensor, max_infix_len: int, verbosity: int = 0) -> torch.Tensor:
        """(B, M) postfix -> (B, max_infix_len) infix token rows with parentheses."""
        _check_token_rows(expressions)
        return notation.postfix_to_infix(expressions, max_infix_len, self._n_variables)

    def _convert(self, fn: str, expressions: torch.Tensor, context: str, check_kind: str, verbosity: int,
                 width=None, fill=int(Operator.NO_OP)) -> torch.Tensor:
        _check_token_rows(expressions)
        dev = _lib.require_cuda(expressions)
        x = expressions.to(torch.int64).contiguous()
        B, M = x.shape
        out = torch.full((B, M if width is None else int(width)), fill, dtype=torch.int64, device=dev)
        err = torch.zeros(B, dtype=torch.int64, device=dev)
        args = [_lib.ptr(x), B, M, self._n_variables, _lib.ptr(out)]
        if width is not None:
            args.append(int(width))
        _lib.check(getattr(_lib.lib(), fn)(*args, _lib.ptr(err), _lib.stream_ptr(dev)), fn)
        self._parsing_error(err.cpu(), x, context, verbosity, check_kind)
        return out

    def prefix_to_infix(self, expressions: torch.Tensor, max_infix_len: int, verbosity: int = 0) -> torch.Tensor:
        """(B, M) prefix -> (B, max_infix_len) infix token rows with parentheses."""
        return self._convert("sr_prefix_to_infix", expressions, "prefix to infix conversion", "prefix_ops",
                             verbosity, width=max_infix_len)

    def prefix_to_postfix(self, expressions: torch.Tensor, verbosity: int = 0) -> torch.Tensor:
        """(B, M) prefix -> (B, M) postfix."""
        return self._convert("sr_prefix_to_postfix", expressions, "prefix to postfix parent conversion",
                             "prefix_ops", verbosity)

    def postfix_to_prefix(self, expressions: torch.Tensor, verbosity: int = 0) -> torch.Tensor:
        """(B, M) postfix -> (B, M) prefix."""
        return self._convert("sr_postfix_to_prefix", expressions, "postfix to prefix parent conversion",
                             "postfix_ops", verbosity)

    def get_prefix_parent(self, prefix_ops: torch.Tensor, verbosity: int = 0) -> torch.Tensor:
        """(B, M) prefix -> (B, M) index of every node's parent (-1: root or padding)."""
        return self._convert("sr_prefix_parent", prefix_ops, "get prefix parent", "prefix_ops", verbosity, fill=-1)

    def get_postfix_children(self, postfix_ops: torch.Tensor, verbosity: int = 0) -> torch.Tensor:
        """(B, M) postfix -> (B, M, 2) child table (NULL_CHILD = -1)."""
        _check_token_rows(postfix_ops)
        return notation.get_postfix_children(postfix_ops, self._n_variables)
