"""Validation and staging of (Ops, Ch) tapes for the kernels.

One launch of ``sr_tape_compile`` checks every node the way the reference's
``validate_inputs`` does (src/symbolic_evaluation.cpp:7-37) and writes the compact
node table the interpreter kernels read; the host then reads a 4-word summary
once (status, longest tape, longest root prefix, most constants), as the
reference reads its error flag once per call.
"""
from __future__ import annotations

from dataclasses import dataclass

import torch

from . import _lib
from .operators import error_message


@dataclass
class CompiledTapes:
    desc: torch.Tensor  # (B, M) int32 node words (uint32 bit patterns)
    meta: torch.Tensor  # (B, 4) int32: L_eff, root, constants up to the root, constants
    B: int
    M: int
    max_len: int        # largest L_eff
    max_root: int       # largest root + 1
    max_consts: int     # largest number of constants up to the root
    max_operators: int  # largest number of operator nodes (arity >= 1 or NO_OP) up to the root
    max_live: int = 0   # most operator-node adjoints live at once in a reverse sweep (0: not measured)
    _order: torch.Tensor | None = None

    @property
    def order(self) -> torch.Tensor:
        """Tape indices, longest first (work order for the persistent kernels)."""
        if self._order is None:
            self._order = torch.argsort(self.meta[:, 0], descending=True, stable=True).to(torch.int32)
        return self._order


def compile_tapes(ops_bm: torch.Tensor, ch_bm: torch.Tensor, n_vars: int, validate_only: bool = False,
                  live: bool = False):
    """Validate (and stage) tapes given as (B, M) / (B, M, 2) int64 CUDA views; live
    also measures the fit kernel's live adjoint rows (``sr_tape_live_rows``), read with
    the same single host synchronisation.

    Raises RuntimeError("Error during input validation: ...") on an invalid tape.
    """
    dev = ops_bm.device
    B, M = ops_bm.shape
    L = _lib.lib()
    st = _lib.stream_ptr(dev)
    stats = torch.zeros(8, dtype=torch.int32, device=dev)
    sb, sm = ops_bm.stride()
    cb, cm, ci = ch_bm.stride()
    if validate_only:
        rc = L.sr_validate(_lib.ptr(ops_bm), _lib.ptr(ch_bm), B, M, sb, sm, cb, cm, ci, _lib.ptr(stats), st)
        _lib.check(rc, "sr_validate")
        code = int(stats[0].item())
        if code:
            raise RuntimeError(error_message(code, "input validation"))
        return None
    desc = torch.empty((B, M), dtype=torch.int32, device=dev)
    meta = torch.empty((B, 4), dtype=torch.int32, device=dev)
    rc = L.sr_tape_compile(_lib.ptr(ops_bm), _lib.ptr(ch_bm), B, M, sb, sm, cb, cm, ci, int(n_vars),
                           _lib.ptr(desc), _lib.ptr(meta), _lib.ptr(stats), st)
    _lib.check(rc, "sr_tape_compile")
    if live:
        _lib.check(L.sr_tape_live_rows(_lib.ptr(desc), _lib.ptr(meta), B, M, _lib.ptr(stats), st), "sr_tape_live_rows")
    s = stats.tolist()
    if s[0]:
        raise RuntimeError(error_message(s[0], "input validation"))
    return CompiledTapes(desc=desc, meta=meta, B=B, M=M, max_len=s[1], max_root=s[2], max_consts=s[3],
                         max_operators=s[4], max_live=s[5] if live else 0)
