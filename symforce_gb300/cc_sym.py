"""The compiled binding of the GPU optimizer, shaped like the reference's `cc_sym` Optimizer
(symforce/pybind/cc_optimizer.cc:29-170).

    from symforce_gb300 import cc_sym
    opt = cc_sym.Optimizer(params, problem)          # params: dict or object with the
                                                      # optimizer_params_t field names
    stats = opt.optimize(values, num_iterations=-1, populate_best_linearization=False)
    lin = opt.linearize(values)

`problem` is the typed-factor form of the factors (any object with key_types, batches of (kind,
keys, consts) and optionally num_schur_keys, e.g. symforce_gb300._cabi.ProblemArrays); `values` is
the float64 storage of every key in key order, updated in place with the best values.  The stats
carry iterations (iteration, current_lambda, new_error, new_error_linear, relative_reduction,
update_angle_change, update_accepted), best_index, status, failure_reason and best_linearization.
The module is the CPython extension symforce_gb300/_cc_sym_gpu (built from csrc/py_cc_sym.cpp with
the library); importing it without the built extension raises ImportError, and constructing an
Optimizer without a CUDA device raises RuntimeError (there is no CPU fallback).
"""

from __future__ import annotations

from . import _build

_build.build()
from ._cc_sym_gpu import Optimizer, default_optimizer_params, optimize  # noqa: E402,F401

__all__ = ["Optimizer", "default_optimizer_params", "optimize"]
