"""Batched form: many independent small problems (Pose3 chains) optimized by one persistent GPU
launch, one sym::Optimizer-equivalent LM loop per problem (include/sfgpu.h, "batched small
problems")."""

from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _cabi as A
from .optimizer import _check, lib


class BatchResultC(C.Structure):
    _fields_ = [
        ("num_iterations", C.c_int32),
        ("best_index", C.c_int32),
        ("status", C.c_int32),
        ("failure_reason", C.c_int32),
        ("initial_error", C.c_double),
        ("best_error", C.c_double),
    ]


def _bind(L: C.CDLL) -> None:
    if getattr(L, "_batch_bound", False):
        return
    L.sfg_batch_create.argtypes = [C.POINTER(A.ProblemC), C.c_int32, C.POINTER(A.FormParams),
                                   C.POINTER(C.c_void_p)]
    L.sfg_batch_destroy.argtypes = [C.c_void_p]
    L.sfg_batch_storage_dim.argtypes = [C.c_void_p, C.POINTER(C.c_int64)]
    L.sfg_batch_set_values.argtypes = [C.c_void_p, C.POINTER(C.c_double), C.c_int64]
    L.sfg_batch_get_values.argtypes = [C.c_void_p, C.POINTER(C.c_double), C.c_int64]
    L.sfg_batch_optimize.argtypes = [C.c_void_p, C.POINTER(A.OptimizerParams), C.c_int32,
                                     C.POINTER(BatchResultC), C.POINTER(C.c_double)]
    L.sfg_batch_records.argtypes = [C.c_void_p, C.c_int32, C.POINTER(A.IterationC), C.c_int32,
                                    C.POINTER(C.c_int32)]
    L.sfg_batch_autotune.argtypes = [C.c_void_p, C.POINTER(A.OptimizerParams), C.POINTER(C.c_int32),
                                     C.POINTER(C.c_int32)]
    L._batch_bound = True


@dataclass
class BatchResult:
    num_iterations: np.ndarray
    best_index: np.ndarray
    status: np.ndarray
    failure_reason: np.ndarray
    initial_error: np.ndarray
    best_error: np.ndarray
    device_ms: float


class BatchOptimizer:
    """One optimizer per problem, all problems in one launch (create once, optimize many)."""

    def __init__(self, problems: list, params: A.OptimizerParams | None = None,
                 form: A.FormParams | None = None):
        L = lib()
        _bind(L)
        self.problems = problems
        self.params = params or A.default_optimizer_params()
        self.form = form or A.default_form_params()
        pcs = [p.to_c() for p in problems]
        arr = (A.ProblemC * len(pcs))(*pcs)
        self._keep = (pcs, arr)
        self._h = C.c_void_p()
        _check(L.sfg_batch_create(arr, len(pcs), C.byref(self.form), C.byref(self._h)))
        n = C.c_int64()
        _check(L.sfg_batch_storage_dim(self._h, C.byref(n)))
        self.storage_dim = n.value
        self.offsets = np.concatenate([[0], np.cumsum([p.storage_dim for p in problems])])

    def close(self) -> None:
        if self._h:
            lib().sfg_batch_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self) -> None:
        try:
            self.close()
        except Exception:
            pass

    def initial_values(self) -> np.ndarray:
        return np.concatenate([p.values for p in self.problems])

    def set_values(self, values: np.ndarray) -> None:
        v = np.ascontiguousarray(values, dtype=np.float64)
        _check(lib().sfg_batch_set_values(self._h, A.dptr(v), v.size))

    def get_values(self, out: np.ndarray | None = None) -> np.ndarray:
        out = np.zeros(self.storage_dim) if out is None else out
        _check(lib().sfg_batch_get_values(self._h, A.dptr(out), out.size))
        return out

    def optimize(self, values: np.ndarray | None = None, params: A.OptimizerParams | None = None,
                 num_iterations: int = -1) -> BatchResult:
        if values is not None:
            self.set_values(values)
        p = params or self.params
        res = (BatchResultC * len(self.problems))()
        ms = C.c_double()
        _check(lib().sfg_batch_optimize(self._h, C.byref(p), num_iterations, res, C.byref(ms)))
        cols = {k: np.array([getattr(r, k) for r in res]) for k, _ in BatchResultC._fields_}
        return BatchResult(device_ms=ms.value, **cols)

    def records(self, problem: int) -> list:
        n = C.c_int32()
        _check(lib().sfg_batch_records(self._h, problem, None, 0, C.byref(n)))
        recs = (A.IterationC * max(n.value, 1))()
        _check(lib().sfg_batch_records(self._h, problem, recs, n.value, C.byref(n)))
        return [recs[i] for i in range(n.value)]

    def autotune(self, params: A.OptimizerParams | None = None) -> tuple[int, int]:
        w, c = C.c_int32(), C.c_int32()
        _check(lib().sfg_batch_autotune(self._h, C.byref(params or self.params), C.byref(w), C.byref(c)))
        return w.value, c.value
