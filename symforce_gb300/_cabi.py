"""ctypes mirror of the C ABI declared in include/sfgpu.h.

The structures here are byte-for-byte the POD structs of the header; `ProblemArrays.to_c()` keeps
the numpy buffers alive for as long as the returned structure is referenced.
"""

from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

# status codes / enums (include/sfgpu.h)
SFG_OK = 0
(SFG_ERR_INVALID_ARGUMENT, SFG_ERR_CUDA, SFG_ERR_NO_DEVICE, SFG_ERR_STRUCTURE, SFG_ERR_DEVICE_STATUS,
 SFG_ERR_OUT_OF_MEMORY, SFG_ERR_CAPACITY, SFG_ERR_NUMERICAL) = range(1, 9)
SFG_STATUS_INVALID, SFG_STATUS_SUCCESS, SFG_STATUS_HIT_ITERATION_LIMIT, SFG_STATUS_FAILED = 0, 1, 2, 3
SFG_FAILURE_INVALID, SFG_FAILURE_LAMBDA_OUT_OF_BOUNDS, SFG_FAILURE_INITIAL_ERROR_NOT_FINITE = 0, 1, 2
SFG_LAMBDA_UPDATE_STATIC, SFG_LAMBDA_UPDATE_DYNAMIC = 1, 2

SFG_KEY_VEC1, SFG_KEY_VEC2, SFG_KEY_VEC3, SFG_KEY_POSE2, SFG_KEY_POSE3 = 1, 2, 3, 4, 5
SFG_KEY_ROT3, SFG_KEY_VEC4, SFG_KEY_VEC5, SFG_KEY_VEC6 = 6, 7, 8, 9
KEY_DIMS = {  # storage, tangent
    SFG_KEY_VEC1: (1, 1),
    SFG_KEY_VEC2: (2, 2),
    SFG_KEY_VEC3: (3, 3),
    SFG_KEY_POSE2: (4, 3),
    SFG_KEY_POSE3: (7, 6),
    SFG_KEY_ROT3: (4, 3),
    SFG_KEY_VEC4: (4, 4),
    SFG_KEY_VEC5: (5, 5),
    SFG_KEY_VEC6: (6, 6),
}

SFG_FACTOR_BEARING_POSE2 = 1
SFG_FACTOR_ODOMETRY_POSE2 = 2
SFG_FACTOR_SNAVELY_REPROJECTION = 3
SFG_FACTOR_BETWEEN_POSE3 = 4
SFG_FACTOR_PRIOR_POSE3 = 5
SFG_FACTOR_RANGE_POSE3 = 6
# kinds generated from symbolic definitions (symforce_gb300/factor_defs.py)
SFG_FACTOR_PRIOR_ROT3 = 7
SFG_FACTOR_BETWEEN_ROT3 = 8
SFG_FACTOR_BARRON_VEC5 = 9
SFG_FACTOR_LINEAR_VEC5 = 10
SFG_FACTOR_LINEAR_SCALAR2 = 11
FACTOR_DIMS = {  # num_keys, num_consts, residual_dim, key types
    SFG_FACTOR_BEARING_POSE2: (1, 5, 1, (SFG_KEY_POSE2,)),
    SFG_FACTOR_ODOMETRY_POSE2: (2, 3, 1, (SFG_KEY_POSE2, SFG_KEY_POSE2)),
    SFG_FACTOR_SNAVELY_REPROJECTION: (3, 4, 2, (SFG_KEY_POSE3, SFG_KEY_VEC3, SFG_KEY_VEC3)),
    SFG_FACTOR_BETWEEN_POSE3: (2, 14, 6, (SFG_KEY_POSE3, SFG_KEY_POSE3)),
    SFG_FACTOR_PRIOR_POSE3: (1, 14, 6, (SFG_KEY_POSE3,)),
    SFG_FACTOR_RANGE_POSE3: (1, 6, 1, (SFG_KEY_POSE3,)),
    SFG_FACTOR_PRIOR_ROT3: (1, 8, 3, (SFG_KEY_ROT3,)),
    SFG_FACTOR_BETWEEN_ROT3: (2, 8, 3, (SFG_KEY_ROT3, SFG_KEY_ROT3)),
    SFG_FACTOR_BARRON_VEC5: (1, 7, 5, (SFG_KEY_VEC5,)),
    SFG_FACTOR_LINEAR_VEC5: (1, 54, 9, (SFG_KEY_VEC5,)),
    SFG_FACTOR_LINEAR_SCALAR2: (2, 6, 2, (SFG_KEY_VEC1, SFG_KEY_VEC1)),
}

SFG_PRECISION_FP64, SFG_PRECISION_MIXED = 0, 1
SFG_LINEAR_SOLVER_SPARSE_LDLT, SFG_LINEAR_SOLVER_SCHUR = 0, 1
SFG_LINEAR_SOLVER_PCG_BLOCK_JACOBI, SFG_LINEAR_SOLVER_PCG_LEARNED = 2, 3
SCHUR_SOLVERS = (SFG_LINEAR_SOLVER_SCHUR, SFG_LINEAR_SOLVER_PCG_BLOCK_JACOBI, SFG_LINEAR_SOLVER_PCG_LEARNED)

# learned preconditioner network (include/sfgpu.h)
PRECOND_BLOCK, PRECOND_FEATURES, PRECOND_HIDDEN, PRECOND_OUTPUTS = 9, 96, 256, 45
PRECOND_SAMPLE_FLOATS = PRECOND_FEATURES + 2 * PRECOND_BLOCK
PRECOND_NET_PARAMS = (PRECOND_FEATURES * PRECOND_HIDDEN + PRECOND_HIDDEN + PRECOND_HIDDEN * PRECOND_HIDDEN
                      + PRECOND_HIDDEN + PRECOND_HIDDEN * PRECOND_OUTPUTS + PRECOND_OUTPUTS)
SFG_ORDERING_NESTED_DISSECTION, SFG_ORDERING_NATURAL, SFG_ORDERING_MIN_DEGREE = 0, 1, 2

DEFAULT_EPSILON = 10.0 * np.finfo(np.float64).eps  # sym::kDefaultEpsilon<double>


class FactorBatch(C.Structure):
    _fields_ = [
        ("kind", C.c_int32),
        ("count", C.c_int32),
        ("keys", C.POINTER(C.c_int32)),
        ("consts", C.POINTER(C.c_double)),
    ]


class ProblemC(C.Structure):
    _fields_ = [
        ("num_keys", C.c_int32),
        ("key_types", C.POINTER(C.c_int32)),
        ("num_batches", C.c_int32),
        ("batches", C.POINTER(FactorBatch)),
        ("num_schur_keys", C.c_int32),
    ]


class OptimizerParams(C.Structure):
    """optimizer_params_t (lcmtypes/symforce.lcm:134-200)."""

    _fields_ = [
        ("verbose", C.c_int32),
        ("debug_stats", C.c_int32),
        ("check_derivatives", C.c_int32),
        ("include_jacobians", C.c_int32),
        ("debug_checks", C.c_int32),
        ("initial_lambda", C.c_double),
        ("lambda_lower_bound", C.c_double),
        ("lambda_upper_bound", C.c_double),
        ("lambda_update_type", C.c_int32),
        ("lambda_up_factor", C.c_double),
        ("lambda_down_factor", C.c_double),
        ("dynamic_lambda_update_beta", C.c_double),
        ("dynamic_lambda_update_gamma", C.c_double),
        ("dynamic_lambda_update_p", C.c_int32),
        ("use_diagonal_damping", C.c_int32),
        ("use_unit_damping", C.c_int32),
        ("keep_max_diagonal_damping", C.c_int32),
        ("diagonal_damping_min", C.c_double),
        ("iterations", C.c_int32),
        ("early_exit_min_reduction", C.c_double),
        ("early_exit_min_absolute_error", C.c_double),
        ("enable_bold_updates", C.c_int32),
    ]


def default_optimizer_params(**overrides) -> OptimizerParams:
    """sym::DefaultOptimizerParams (symforce/opt/optimizer.cc:8-56)."""
    p = OptimizerParams(
        verbose=0,
        debug_stats=0,
        check_derivatives=0,
        include_jacobians=0,
        debug_checks=0,
        initial_lambda=1.0,
        lambda_lower_bound=0.0,
        lambda_upper_bound=1000000.0,
        lambda_update_type=SFG_LAMBDA_UPDATE_STATIC,
        lambda_up_factor=4.0,
        lambda_down_factor=1 / 4.0,
        dynamic_lambda_update_beta=2.0,
        dynamic_lambda_update_gamma=3.0,
        dynamic_lambda_update_p=3,
        use_diagonal_damping=0,
        use_unit_damping=1,
        keep_max_diagonal_damping=0,
        diagonal_damping_min=1e-6,
        iterations=50,
        early_exit_min_reduction=1e-6,
        early_exit_min_absolute_error=0.0,
        enable_bold_updates=0,
    )
    for k, v in overrides.items():
        setattr(p, k, v)
    return p


class IterationC(C.Structure):
    """optimization_iteration_t (lcmtypes/symforce.lcm:229-262) + best_error + device time."""

    _fields_ = [
        ("iteration", C.c_int32),
        ("update_accepted", C.c_int32),
        ("current_lambda", C.c_double),
        ("new_error_linear", C.c_double),
        ("new_error", C.c_double),
        ("relative_reduction", C.c_double),
        ("update_angle_change", C.c_double),
        ("best_error", C.c_double),
        ("elapsed_ms", C.c_double),
    ]


class StatsC(C.Structure):
    _fields_ = [
        ("iterations", C.POINTER(IterationC)),
        ("capacity", C.c_int32),
        ("num_iterations", C.c_int32),
        ("best_index", C.c_int32),
        ("status", C.c_int32),
        ("failure_reason", C.c_int32),
        ("kernel_launches", C.c_int32),
        ("device_ms", C.c_double),
    ]


SFG_STAGE_LINEARIZE, SFG_STAGE_SCHUR, SFG_STAGE_FACTOR, SFG_STAGE_SOLVE = 0, 1, 2, 3


class FormParams(C.Structure):
    _fields_ = [
        ("precision", C.c_int32),
        ("linear_solver", C.c_int32),
        ("ordering", C.c_int32),
        ("device", C.c_int32),
        ("epsilon", C.c_double),
        ("refine_steps", C.c_int32),
        ("pcg_max_iters", C.c_int32),
        ("pcg_tol", C.c_double),
        ("pcg_coarse", C.c_int32),
        ("pcg_band", C.c_int32),
    ]


class PcgStatsC(C.Structure):
    _fields_ = [
        ("solves", C.c_int32),
        ("fallbacks", C.c_int32),
        ("iterations", C.c_int64),
        ("max_iterations", C.c_int32),
        ("last_iterations", C.c_int32),
        ("max_rel_residual", C.c_double),
        ("last_rel_residual", C.c_double),
    ]


class TrainParamsC(C.Structure):
    _fields_ = [
        ("steps", C.c_int32),
        ("batch", C.c_int32),
        ("lr", C.c_float),
        ("beta1", C.c_float),
        ("beta2", C.c_float),
        ("eps", C.c_float),
        ("seed", C.c_uint64),
        ("device", C.c_int32),
        ("kaporin", C.c_float),
    ]


def default_form_params(**overrides) -> FormParams:
    f = FormParams(
        precision=SFG_PRECISION_FP64,
        linear_solver=SFG_LINEAR_SOLVER_SPARSE_LDLT,
        ordering=SFG_ORDERING_NESTED_DISSECTION,
        device=0,
        epsilon=DEFAULT_EPSILON,
        refine_steps=1,
        pcg_max_iters=500,
        pcg_tol=1e-8,
        pcg_coarse=0,
        pcg_band=0,
    )
    for k, v in overrides.items():
        setattr(f, k, v)
    return f


def dptr(a: np.ndarray) -> C.POINTER(C.c_double):
    assert a.dtype == np.float64 and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(C.POINTER(C.c_double))


def iptr(a: np.ndarray) -> C.POINTER(C.c_int32):
    assert a.dtype == np.int32 and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(C.POINTER(C.c_int32))


def fptr(a: np.ndarray) -> C.POINTER(C.c_float):
    assert a.dtype == np.float32 and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(C.POINTER(C.c_float))


def lptr(a: np.ndarray) -> C.POINTER(C.c_int64):
    assert a.dtype == np.int64 and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(C.POINTER(C.c_int64))


@dataclass
class Batch:
    kind: int
    keys: np.ndarray  # int32 [count, num_keys]
    consts: np.ndarray  # float64 [count, num_consts]

    def __post_init__(self) -> None:
        nk, nc, _, _ = FACTOR_DIMS[self.kind]
        self.keys = np.ascontiguousarray(np.asarray(self.keys, dtype=np.int32).reshape(-1, nk))
        self.consts = np.ascontiguousarray(np.asarray(self.consts, dtype=np.float64).reshape(-1, nc))
        assert self.keys.shape[0] == self.consts.shape[0]

    @property
    def count(self) -> int:
        return int(self.keys.shape[0])


@dataclass
class ProblemArrays:
    """A problem in the layout of sfg_problem_t plus initial values (storage, key order)."""

    key_types: np.ndarray
    batches: list
    values: np.ndarray
    num_schur_keys: int = 0
    name: str = ""
    meta: dict = field(default_factory=dict)

    def __post_init__(self) -> None:
        self.key_types = np.ascontiguousarray(np.asarray(self.key_types, dtype=np.int32))
        self.values = np.ascontiguousarray(np.asarray(self.values, dtype=np.float64))
        assert self.values.size == self.storage_dim, (self.values.size, self.storage_dim)

    @property
    def storage_dim(self) -> int:
        return int(sum(KEY_DIMS[int(t)][0] for t in self.key_types))

    @property
    def tangent_dim(self) -> int:
        return int(sum(KEY_DIMS[int(t)][1] for t in self.key_types))

    @property
    def residual_dim(self) -> int:
        return int(sum(b.count * FACTOR_DIMS[b.kind][2] for b in self.batches))

    @property
    def num_factors(self) -> int:
        return int(sum(b.count for b in self.batches))

    def to_c(self) -> ProblemC:
        arr = (FactorBatch * max(1, len(self.batches)))()
        for i, b in enumerate(self.batches):
            arr[i] = FactorBatch(b.kind, b.count, iptr(b.keys), dptr(b.consts))
        pc = ProblemC(len(self.key_types), iptr(self.key_types), len(self.batches), arr,
                      self.num_schur_keys)
        pc._keepalive = (arr, self)  # type: ignore[attr-defined]
        return pc

    def key_storage_offsets(self) -> np.ndarray:
        dims = np.array([KEY_DIMS[int(t)][0] for t in self.key_types], dtype=np.int64)
        return np.concatenate([[0], np.cumsum(dims)])
