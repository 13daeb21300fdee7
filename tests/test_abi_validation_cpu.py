"""The C ABI's argument checks, on the host: each call below is rejected (or, for an
empty batch, accepted) by a check that runs before the library touches CUDA, so it
returns the status include/sr_gb300.h documents, with the reason in sr_last_error(),
on a machine without a GPU as on one with a GPU.  No kernel is launched."""
import ctypes

import pytest

SR_OK, SR_ERR_INVALID_ARGUMENT, SR_ERR_UNSUPPORTED = 0, -1, -3
MAX_NODES = 4095  # tapes longer than this are unsupported (12-bit child fields)


@pytest.fixture(scope="module")
def L():
    from cudasymbolicregression_gb300 import _lib
    return _lib.load()


def _rejected(L, rc, code, *words):
    assert rc == code, (rc, L.sr_last_error())
    msg = L.sr_last_error().decode()
    for w in words:
        assert w in msg, msg


def test_version_names_the_architecture(L):
    assert b"sm_103a" in L.sr_version()


NOTATION = ("sr_postfix_children", "sr_prefix_to_postfix", "sr_postfix_to_prefix", "sr_prefix_parent",
            "sr_infix_to_postfix", "sr_infix_to_prefix")


@pytest.mark.parametrize("fn", NOTATION)
def test_notation_sizes(L, fn):
    f = getattr(L, fn)
    _rejected(L, f(None, -1, 4, 1, None, None, None), SR_ERR_INVALID_ARGUMENT)
    _rejected(L, f(None, 2, -4, 1, None, None, None), SR_ERR_INVALID_ARGUMENT)
    # an empty batch is a valid call that launches nothing
    assert f(None, 0, 4, 1, None, None, None) == SR_OK


@pytest.mark.parametrize("fn", ("sr_postfix_to_infix", "sr_prefix_to_infix"))
def test_infix_rendering_sizes(L, fn):
    f = getattr(L, fn)
    _rejected(L, f(None, -1, 4, 1, None, 8, None, None), SR_ERR_INVALID_ARGUMENT)
    _rejected(L, f(None, 2, 4, 1, None, -1, None, None), SR_ERR_INVALID_ARGUMENT)
    assert f(None, 0, 4, 1, None, 8, None, None) == SR_OK


def test_infix_parsers_limits(L):
    for fn in ("sr_infix_to_postfix", "sr_infix_to_prefix"):
        f = getattr(L, fn)
        _rejected(L, f(None, 4, 129, 1, None, None, None), SR_ERR_UNSUPPORTED, "HARD_MAX_LENGTH")
        _rejected(L, f(None, 4, 16, -1, None, None, None), SR_ERR_UNSUPPORTED, "n_vars")
        _rejected(L, f(None, 4, 16, 1, None, None, None), SR_ERR_INVALID_ARGUMENT, "null")


def test_sampler_request_checks(L):
    f = L.sr_pcfg_sample_infix
    _rejected(L, f(None, None, None, None, 4, 0, -1, 32, 8, 1, None, None, None), SR_ERR_INVALID_ARGUMENT, "B=-1")
    _rejected(L, f(None, None, None, None, 4, 0, 8, 0, 8, 1, None, None, None), SR_ERR_INVALID_ARGUMENT,
              "max_length=0")
    _rejected(L, f(None, None, None, None, 4, 0, 8, 129, 8, 1, None, None, None), SR_ERR_INVALID_ARGUMENT,
              "max_length=129")
    _rejected(L, f(None, None, None, None, 0, 0, 8, 32, 8, 1, None, None, None), SR_ERR_UNSUPPORTED, "symbol ids")
    _rejected(L, f(None, None, None, None, 4, 40000, 8, 32, 8, 1, None, None, None), SR_ERR_UNSUPPORTED)
    _rejected(L, f(None, None, None, None, 4, 0, 8, 32, 8, 1, None, None, None), SR_ERR_INVALID_ARGUMENT, "null")
    assert f(None, None, None, None, 4, 0, 0, 32, 8, 1, None, None, None) == SR_OK


def test_tape_compile_checks(L):
    st = ctypes.c_int32()
    dummy = ctypes.byref(ctypes.c_int64())  # never dereferenced: every call below stops at a check
    _rejected(L, L.sr_tape_compile(None, None, -1, 4, 4, 1, 8, 2, 1, 1, None, None, ctypes.byref(st), None),
              SR_ERR_INVALID_ARGUMENT, "negative")
    _rejected(L, L.sr_tape_compile(None, None, 2, MAX_NODES + 1, 0, 1, 0, 2, 1, 1, None, None, ctypes.byref(st), None),
              SR_ERR_UNSUPPORTED, str(MAX_NODES))
    _rejected(L, L.sr_tape_compile(dummy, dummy, 2, 4, 4, 1, 8, 2, 1, 1, dummy, dummy, None, None),
              SR_ERR_INVALID_ARGUMENT, "null")
    _rejected(L, L.sr_tape_compile(dummy, dummy, 2, 4, 4, 1, 8, 2, 1, -1, dummy, dummy, dummy, None),
              SR_ERR_UNSUPPORTED, "n_vars")
    _rejected(L, L.sr_validate(None, None, -3, 4, 4, 1, 8, 2, 1, ctypes.byref(st), None), SR_ERR_INVALID_ARGUMENT)


@pytest.mark.parametrize("fn", ("sr_eval_forward_f32", "sr_eval_forward_f64"))
def test_forward_checks(L, fn):
    f = getattr(L, fn)
    _rejected(L, f(None, 8, 1, None, None, None, -1, 4, 4, None, 4, 1, None, None), SR_ERR_INVALID_ARGUMENT)
    _rejected(L, f(None, 8, 1, None, None, None, 2, MAX_NODES + 1, 4, None, 4, 1, None, None), SR_ERR_UNSUPPORTED)
    _rejected(L, f(None, -8, 1, None, None, None, 2, 4, 4, None, 4, 1, None, None), SR_ERR_INVALID_ARGUMENT)
    # empty batch, no tape positions, no points: nothing to do
    for B, M, N in ((0, 4, 8), (2, 0, 8), (2, 4, 0)):
        assert f(None, N, 1, None, None, None, B, M, 4, None, 4, 1, None, None) == SR_OK


def test_fit_option_checks(L):
    from cudasymbolicregression_gb300._lib import FitOptions
    for field, bad in (("max_iter", -1), ("history_size", 0), ("line_search", 2), ("objective", 3),
                       ("points_per_lane", 3), ("line_search_max_iter", -1)):
        o = FitOptions(max_iter=10, history_size=10, tolerance_grad=1e-7, line_search=0, line_search_max_iter=10,
                       eps=1e-10)
        setattr(o, field, bad)
        _rejected(L, L.sr_fit_workspace_bytes(8, 16, 32, 4, 4, ctypes.byref(o)), SR_ERR_INVALID_ARGUMENT)
        st = ctypes.c_int32()
        rc = L.sr_fit_lbfgs(None, 16, 1, None, None, None, 8, 32, None, None, 32, 1, None, None, None, None, None, 4, 4,
                            ctypes.byref(o), None, 0, ctypes.byref(st), None)
        _rejected(L, rc, SR_ERR_INVALID_ARGUMENT)
    st = ctypes.c_int32()
    _rejected(L, L.sr_fit_lbfgs(None, 16, 1, None, None, None, -8, 32, None, None, 32, 1, None, None, None, None, None,
                                4, 4, None, None, 0, ctypes.byref(st), None), SR_ERR_INVALID_ARGUMENT, "negative")
    _rejected(L, L.sr_fit_lbfgs(None, 16, 1, None, None, None, 8, MAX_NODES + 1, None, None, 32, 1, None, None, None,
                                None, None, 4, 4, None, None, 0, ctypes.byref(st), None), SR_ERR_UNSUPPORTED)
    _rejected(L, L.sr_fit_lbfgs(None, 16, 1, None, None, None, 8, 32, None, None, 32, 1, None, None, None, None, None,
                                4, 4, None, None, 0, None, None), SR_ERR_INVALID_ARGUMENT, "status")
    # screening: sizes and pointers are checked before any CUDA call; nothing to screen is fine
    _rejected(L, L.sr_fit_screen(None, 16, 1, None, None, None, 8, 32, None, 256, 32, 1, -1, None, 4, 4, None,
                                 ctypes.byref(st), None), SR_ERR_INVALID_ARGUMENT, "negative")
    _rejected(L, L.sr_fit_screen(None, 16, 1, None, None, None, 8, 32, None, 256, 32, 1, 2, None, -1, 4, None,
                                 ctypes.byref(st), None), SR_ERR_INVALID_ARGUMENT, "negative")
    _rejected(L, L.sr_fit_screen(None, 16, 1, None, None, None, 8, MAX_NODES + 1, None, 256, 32, 1, 2, None, 4, 4,
                                 None, ctypes.byref(st), None), SR_ERR_UNSUPPORTED)
    _rejected(L, L.sr_fit_screen(None, 16, 1, None, None, None, 8, 32, None, 256, 32, 1, 2, None, 4, 4, None, None,
                                 None), SR_ERR_INVALID_ARGUMENT, "status")
    _rejected(L, L.sr_fit_lbfgs(None, 16, 1, None, None, None, 8, 32, None, None, 32, 1, None, None, None, None, None,
                                -1, 4, None, None, 0, ctypes.byref(st), None), SR_ERR_INVALID_ARGUMENT, "negative")
    _rejected(L, L.sr_tape_live_rows(None, None, -1, 32, None, None), SR_ERR_INVALID_ARGUMENT, "negative")
    _rejected(L, L.sr_tape_live_rows(None, None, 4, MAX_NODES + 1, None, None), SR_ERR_UNSUPPORTED)
    _rejected(L, L.sr_tape_live_rows(None, None, 4, 32, None, None), SR_ERR_INVALID_ARGUMENT, "null pointer")
    assert L.sr_tape_live_rows(None, None, 0, 32, None, None) == 0
    shape = (ctypes.c_int32 * 3)()
    _rejected(L, L.sr_fit_launch_shape(8, 16, 1, 32, 4, 4, None, None), SR_ERR_INVALID_ARGUMENT, "shape")
    _rejected(L, L.sr_fit_launch_shape(-8, 16, 1, 32, 4, 4, None, ctypes.cast(shape, ctypes.c_void_p)),
              SR_ERR_INVALID_ARGUMENT, "negative")
    _rejected(L, L.sr_fit_launch_shape(8, 16, 1, MAX_NODES + 1, 4, 4, None, ctypes.cast(shape, ctypes.c_void_p)),
              SR_ERR_UNSUPPORTED)


def test_constant_table_checks(L):
    off = ctypes.byref(ctypes.c_int64())
    _rejected(L, L.sr_const_offsets(None, -1, 4, 4, 1, off, None), SR_ERR_INVALID_ARGUMENT)
    _rejected(L, L.sr_const_offsets(None, 2, 4, 4, 1, None, None), SR_ERR_INVALID_ARGUMENT)
    _rejected(L, L.sr_const_offsets(None, 2, 4, 4, 1, off, None), SR_ERR_INVALID_ARGUMENT)


def test_gemm_shape_checks(L):
    from cudasymbolicregression_gb300._lib import MlpEpilogue
    epi = MlpEpilogue()
    _rejected(L, L.sr_mlp_gemm(None, 128, 64, 64, None, 64, 64, None, None, None), SR_ERR_INVALID_ARGUMENT)
    _rejected(L, L.sr_mlp_gemm(None, -1, 64, 64, None, 64, 64, ctypes.byref(epi), None, None), SR_ERR_INVALID_ARGUMENT)
    assert L.sr_mlp_gemm(None, 0, 64, 64, None, 64, 64, ctypes.byref(epi), None, None) == SR_OK
    for k, n, lda in ((48, 64, 64), (64, 96, 64), (64, 64, 32), (128, 64, 132)):
        _rejected(L, L.sr_mlp_gemm(None, 128, k, lda, None, n, k, ctypes.byref(epi), None, None),
                  SR_ERR_INVALID_ARGUMENT, "multiple of 64")
    # split-K bookkeeping: the pieces the kernel actually uses for k and a requested split count
    assert [L.sr_mlp_gemm_splits_used(k, s) for k, s in ((256, 1), (256, 4), (256, 3), (256, 9), (0, 2))] == \
        [1, 4, 2, 4, 0]


def test_last_error_is_per_thread(L):
    """sr_last_error() holds the last failure of the calling host thread only."""
    import threading
    off = ctypes.byref(ctypes.c_int64())
    _rejected(L, L.sr_const_offsets(None, -1, 4, 4, 1, off, None), SR_ERR_INVALID_ARGUMENT, "invalid arguments")
    seen = {}

    def other():
        seen["fresh"] = L.sr_last_error()
        seen["rc"] = L.sr_pcfg_sample_infix(None, None, None, None, 4, 0, 8, 0, 8, 1, None, None, None)
        seen["own"] = L.sr_last_error()
    t = threading.Thread(target=other)
    t.start()
    t.join()
    assert seen["fresh"] == b"" and seen["rc"] == SR_ERR_INVALID_ARGUMENT and b"max_length=0" in seen["own"]
    assert b"invalid arguments" in L.sr_last_error()
