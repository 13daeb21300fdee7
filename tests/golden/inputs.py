"""Malformed inputs shared by the fixture generator (make_golden.py) and the tests
that replay the reference's exceptions for them."""
import torch

EVAL_INPUT_CASES = ("ops_1d", "ch_2d", "c_1d", "c_wrong_m", "ch_wrong_b", "ch_last_3", "x_1d", "x_0d", "x_3d", "x_int",
                    "c_int", "ops_float", "ch_int32", "c_f64", "x_f64", "ops_3d")
MULTI_INPUT_CASES = ("c_2d", "ops_1d", "x_1d", "x_3d", "c_f64", "c_wrong_b", "ch_int32")


def eval_input_case(name, multiple=False):
    """Malformed (X, Ops, Ch, C) for evaluate / evaluate_multiple, by name."""
    X = torch.ones(10, 2)
    ops = torch.tensor([[50, 1, 40]])
    ch = torch.tensor([[[-1, -1], [-1, -1], [0, 1]]])
    C = torch.zeros(1, 3, 2) if multiple else torch.zeros(1, 3)
    return {"ops_1d": (X, ops[0], ch, C), "ch_2d": (X, ops, ch[0], C), "c_1d": (X, ops, ch, torch.zeros(3)),
            "c_2d": (X, ops, ch, torch.zeros(1, 3)), "c_wrong_m": (X, ops, ch, torch.zeros(1, 4)),
            "ch_wrong_b": (X, ops, ch.repeat(2, 1, 1), C), "ch_last_3": (X, ops, torch.cat([ch, ch[..., :1]], -1), C),
            "x_1d": (X[:, 0], ops, ch, C), "x_0d": (torch.tensor(1.0), ops, ch, C), "x_3d": (X[:, :, None], ops, ch, C),
            "x_int": (X.int(), ops, ch, C), "c_int": (X, ops, ch, C.int()), "ops_float": (X, ops.float(), ch, C),
            "ch_int32": (X, ops, ch.int(), C), "c_f64": (X, ops, ch, C.double()), "x_f64": (X.double(), ops, ch, C),
            "ops_3d": (X, ops[None], ch, C), "c_wrong_b": (X, ops, ch, torch.zeros(2, 3, 2))}[name]
