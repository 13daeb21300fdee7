"""``create_constants`` (reference symbolic_torch/utils.py:7-41).

The random values are drawn with torch's generator on the tensor's device in the
same call and order as the reference (``randn(n) * std + mean`` or
``rand(n) * (upper - lower) + lower`` in float32), so a seeded caller gets the same
constants; the count and the row-major scatter into the (B, M) table run in the
library's kernels.
"""
from __future__ import annotations

from typing import Any

import torch

from . import _lib


def create_constants(ops_tensor: torch.Tensor, method: str = "randn", **kwargs: Any) -> torch.Tensor:
    """Constants table shaped like ``ops_tensor``: random values at
    LEARNABLE_CONSTANT entries (row-major order), 0 elsewhere.

    method 'randn': mean (default 0.0), std (default 1.0).
    method 'range': lower (default 0.0), upper (default 1.0).
    """
    if method not in ("randn", "range"):
        raise ValueError(f"Unknown method for constant creation: {method}")
    dev = _lib.require_cuda(ops_tensor)
    if ops_tensor.dtype != torch.int64:
        ops_tensor = ops_tensor.to(torch.int64)
    shape = ops_tensor.shape
    ops2 = ops_tensor.reshape(-1, shape[-1]) if ops_tensor.dim() != 2 else ops_tensor
    if ops_tensor.dim() == 0:
        ops2 = ops_tensor.reshape(1, 1)
    R, Cc = ops2.shape
    s0, s1 = ops2.stride()
    L = _lib.lib()
    st = _lib.stream_ptr(dev)
    off = torch.empty(R + 1, dtype=torch.int64, device=dev)
    _lib.check(L.sr_const_offsets(_lib.ptr(ops2), R, Cc, s0, s1, _lib.ptr(off), st), "sr_const_offsets")
    num = int(off[R].item())
    dtype = torch.float32
    if method == "randn":
        mean = kwargs.get("mean", 0.0)
        std = kwargs.get("std", 1.0)
        flat = torch.randn(num, dtype=dtype, device=dev) * std + mean
    else:
        lower = kwargs.get("lower", 0.0)
        upper = kwargs.get("upper", 1.0)
        flat = torch.rand(num, dtype=dtype, device=dev) * (upper - lower) + lower
    flat = flat.to(dtype).contiguous()
    out = torch.empty((R, Cc), dtype=dtype, device=dev)
    _lib.check(L.sr_const_scatter(_lib.ptr(ops2), R, Cc, s0, s1, _lib.ptr(off), _lib.ptr(flat), _lib.ptr(out), st),
               "sr_const_scatter")
    return out.reshape(shape)
