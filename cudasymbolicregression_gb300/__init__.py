"""GB300-native batched expression fitting (drop-in for symbolic_torch's hot path).

Public API, mirroring the reference package ``symbolic_torch``:

* ``evaluation.evaluate(X, Ops, Ch, C)`` / ``evaluation.evaluate_backend`` --
  postfix-tape evaluation with autograd (forward + adjoint CUDA kernels);
* ``create_constants(ops, method='randn'|'range', **kw)``;
* ``optimize(X, Y, Ops, Ch, C_init, max_iter, history_size, tolerance_grad,
  line_search_fn)`` -- the fused batched L-BFGS kernel;
* ``ProbabilisticContextFreeGrammar`` -- grammar sampling and infix parsing on
  the device (``sample(B)`` gives postfix Ops and Ch for the fit);
* ``Operator``, ``get_arity``, ``is_valid_op``.

Every compute entry point runs hand-written sm_103a kernels from
``libsr_gb300.so`` on CUDA tensors; there is no CPU path.
"""
from . import evaluation, notation
from .operators import MAX_ARITY, NULL_CHILD, ErrorCode, Operator, get_arity, is_valid_op
from .optimization import FitPlan, FitResult, optimize, optimize_ex
from .pcfg import ProbabilisticContextFreeGrammar
from .utils import create_constants

__all__ = [
    "evaluation",
    "notation",
    "ProbabilisticContextFreeGrammar",
    "Operator",
    "ErrorCode",
    "create_constants",
    "optimize",
    "optimize_ex",
    "FitResult",
    "FitPlan",
    "get_arity",
    "is_valid_op",
    "MAX_ARITY",
    "NULL_CHILD",
]
