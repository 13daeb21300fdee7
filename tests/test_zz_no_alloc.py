"""The fit entry point that allocates nothing (sr_fit_lbfgs_static_scratch).

It exists for callers that cannot give the library device memory -- a process whose
device memory belongs to its own pool allocator and forbids other cudaMalloc calls,
or a service that must not allocate while serving a request.  Its scratch is a
fixed array inside the library.  This file is collected last so that a run that
stops at the first failure has already run every other test; it passes alone in a
fresh process as well as after the other tests.
"""
import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _setup():
    from cudasymbolicregression_gb300 import _lib, workloads
    from cudasymbolicregression_gb300.tape import compile_tapes
    wl = workloads.ragged_fit(B=1500, N=200, M=48, seed=11)
    dev = torch.device("cuda")
    X, Y, O, Ch, C = (torch.tensor(a, device=dev) for a in (wl.X, wl.Y, wl.ops, wl.ch, wl.C))
    tp = compile_tapes(O, Ch, X.shape[1])
    return _lib, wl, dev, X, Y, tp, C


def _outputs(B, M, N, dev):
    return (torch.full((B, M), 7.0, device=dev), torch.full((B, N), 7.0, device=dev),
            torch.full((B,), -9, dtype=torch.int32, device=dev), torch.full((B,), 7.0, device=dev),
            torch.zeros(B, dtype=torch.int32, device=dev), torch.zeros(1, dtype=torch.int32, device=dev))


def _call(L, fn, X, Y, tp, C, outs, opts, ws=None):
    Cout, Yf, it, loss, ev, st = outs
    N, nx = X.shape
    args = [L.ptr(X), N, nx, L.ptr(Y), L.ptr(tp.desc), L.ptr(tp.meta), tp.B, tp.M, L.ptr(C), L.ptr(Cout),
            tp.M, 1, L.ptr(Yf), L.ptr(it), L.ptr(loss), L.ptr(ev), None, max(tp.max_root, 1), tp.max_consts,
            ctypes.byref(opts)]
    if ws is not None:
        args += [L.ptr(ws), ws.numel()]
    args += [L.ptr(st), L.stream_ptr(X.device)]
    rc = fn(*args)
    L.check(rc, fn.__name__)
    torch.cuda.synchronize()
    return [t.cpu().numpy() for t in outs]


def _same(a, b):
    return np.array_equal(np.nan_to_num(a, nan=12345.0), np.nan_to_num(b, nan=12345.0))


@pytest.mark.parametrize("history", [10, 200])  # 200: the grid is shrunk to fit the array
def test_static_scratch_matches_workspace_entry_point_twice(history):
    L, wl, dev, X, Y, tp, C = _setup()
    lib = L.lib()
    opts = L.FitOptions(max_iter=40, history_size=history, tolerance_grad=1e-7, line_search=0, line_search_max_iter=10,
                        eps=1e-10, objective=0, warps_per_block=0, points_per_lane=0, grid_blocks=0)
    wsb = lib.sr_fit_workspace_bytes(tp.B, X.shape[0], tp.M, max(tp.max_root, 1), tp.max_consts,
                                     ctypes.byref(opts))
    if history == 200:  # the full grid's rings would not fit the 16 MiB array: the shrinking path runs
        assert wsb > 16 << 20
    ws = torch.empty(int(wsb), dtype=torch.uint8, device=dev)
    ref = _call(L, lib.sr_fit_lbfgs, X, Y, tp, C, _outputs(tp.B, tp.M, X.shape[0], dev), opts, ws)
    outs = [_outputs(tp.B, tp.M, X.shape[0], dev) for _ in range(2)]
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info(dev)[0]
    for i in range(2):  # the array keeps the previous call's contents; results must not depend on them
        got = _call(L, lib.sr_fit_lbfgs_static_scratch, X, Y, tp, C, outs[i], opts)
        # the entry point allocated no device memory (a change would show in the device's free memory)
        assert torch.cuda.mem_get_info(dev)[0] == free0
        C_r, Y_r, it_r, loss_r, ev_r, st_r = ref
        C_g, Y_g, it_g, loss_g, ev_g, st_g = got
        assert st_g[0] == st_r[0]
        np.testing.assert_array_equal(it_g, it_r)
        # each problem's fit is independent of the grid that runs it, so the results agree
        # to the tolerance the fit tests use (final MSE within 1e-4 relative), here exactly
        m_r = ((Y_r.astype(np.float64) - wl.Y) ** 2).mean(1)
        m_g = ((Y_g.astype(np.float64) - wl.Y) ** 2).mean(1)
        with np.errstate(invalid="ignore", divide="ignore"):
            rel = np.abs(m_g - m_r) / np.maximum(np.abs(m_r), 1e-30)
        assert ((rel <= 1e-4) | (np.isnan(m_g) & np.isnan(m_r)) | (m_g == m_r)).all()
        assert _same(C_g, C_r) and _same(Y_g, Y_r) and _same(loss_g, loss_r)


def test_static_scratch_rejects_oversized_history():
    L, wl, dev, X, Y, tp, C = _setup()
    lib = L.lib()
    opts = L.FitOptions(max_iter=5, history_size=200000, tolerance_grad=1e-7, line_search=0, line_search_max_iter=10,
                        eps=1e-10, objective=0, warps_per_block=0, points_per_lane=0, grid_blocks=0)
    outs = _outputs(tp.B, tp.M, X.shape[0], dev)
    with pytest.raises(RuntimeError, match="static fit scratch is 16777216 bytes"):
        _call(L, lib.sr_fit_lbfgs_static_scratch, X, Y, tp, C, outs, opts)
