"""Failure detection and run-to-run reproducibility on the GPU, without faulting it.

The reference reports solver failures in the stats, not as errors: INITIAL_ERROR_NOT_FINITE when
the first linearization is not finite (symforce/opt/levenberg_marquardt_solver.tcc:179-185) and
LAMBDA_OUT_OF_BOUNDS when lambda leaves its bounds (:288-290).  Both are provoked here from the
host (a NaN in the input values, a tiny lambda bound) and compared with the oracle.  There is no
race detector on this pool, so bit-identical repeated runs stand in for it: every device
reduction has a fixed order, so two runs on the same inputs must give the same bits."""

from __future__ import annotations

import numpy as np
import pytest

import oracle_lib as O
from symforce_gb300 import _cabi as A
from symforce_gb300 import learned, synth
from symforce_gb300.batch import BatchOptimizer
from symforce_gb300.optimizer import Optimizer

pytestmark = pytest.mark.gpu


def _ba():
    return synth.bundle_adjustment(num_cameras=10, num_points=300, num_observations=1300, seed=1)


@pytest.mark.parametrize("precision", [A.SFG_PRECISION_FP64, A.SFG_PRECISION_MIXED])
def test_nan_initial_values_report_initial_error_not_finite(precision):
    p = _ba()
    values = p.values.copy()
    values[7 * 10 + 3] = np.nan  # an intrinsics entry
    params = A.default_optimizer_params(lambda_update_type=A.SFG_LAMBDA_UPDATE_DYNAMIC, iterations=10)
    opt = Optimizer(p, params, A.default_form_params(precision=precision, linear_solver=A.SFG_LINEAR_SOLVER_SCHUR))
    _, stats = opt.optimize(values)
    ref = O.optimize(p, params, values=values)
    assert ref["status"] == A.SFG_STATUS_FAILED
    assert ref["failure_reason"] == A.SFG_FAILURE_INITIAL_ERROR_NOT_FINITE
    assert stats.status == ref["status"] and stats.failure_reason == ref["failure_reason"]
    assert len(stats.iterations) == len(ref["iterations"])
    # the handle stays usable: the next call on finite values succeeds like the oracle's
    _, stats2 = opt.optimize(p.values)
    ref2 = O.optimize(p, params)
    assert stats2.status == ref2["status"]
    assert stats2.best_error == pytest.approx(ref2["iterations"][ref2["best_index"]].new_error,
                                              rel=1e-9 if precision == A.SFG_PRECISION_FP64 else 1e-5)


def test_lambda_out_of_bounds_matches_oracle():
    p = _ba()
    # STATIC updates (x4 on rejection) with an upper bound the first rejections cross
    params = A.default_optimizer_params(iterations=20, lambda_upper_bound=3.0, initial_lambda=1.0)
    opt = Optimizer(p, params, A.default_form_params(linear_solver=A.SFG_LINEAR_SOLVER_SCHUR))
    _, stats = opt.optimize(p.values)
    ref = O.optimize(p, params)
    assert ref["status"] == A.SFG_STATUS_FAILED
    assert ref["failure_reason"] == A.SFG_FAILURE_LAMBDA_OUT_OF_BOUNDS
    assert (stats.status, stats.failure_reason) == (ref["status"], ref["failure_reason"])
    assert [r.update_accepted for r in stats.iterations] == [r.update_accepted for r in ref["iterations"]]
    for g, o in zip(stats.iterations, ref["iterations"]):
        assert g.new_error == pytest.approx(o.new_error, rel=1e-9)


@pytest.mark.parametrize("precision,solver", [
    (A.SFG_PRECISION_FP64, A.SFG_LINEAR_SOLVER_SCHUR),
    (A.SFG_PRECISION_FP64, A.SFG_LINEAR_SOLVER_SPARSE_LDLT),
    (A.SFG_PRECISION_MIXED, A.SFG_LINEAR_SOLVER_SCHUR),
    (A.SFG_PRECISION_MIXED, A.SFG_LINEAR_SOLVER_PCG_LEARNED),
])
def test_repeated_runs_are_bit_identical(precision, solver):
    p = synth.bundle_adjustment(num_cameras=20, num_points=1200, num_observations=5000, seed=2)
    params = A.default_optimizer_params(lambda_update_type=A.SFG_LAMBDA_UPDATE_DYNAMIC, iterations=25)
    runs = []
    for _ in range(2):  # two handles: nothing is carried over between them
        opt = Optimizer(p, params, A.default_form_params(precision=precision, linear_solver=solver),
                        weights=learned.load_weights() if solver == A.SFG_LINEAR_SOLVER_PCG_LEARNED else None)
        vals, stats = opt.optimize(p.values)
        _, stats_again = opt.optimize(p.values)  # and the same handle twice
        runs.append((vals, [(r.new_error, r.current_lambda, r.update_accepted) for r in stats.iterations],
                     [(r.new_error, r.current_lambda, r.update_accepted) for r in stats_again.iterations]))
        opt.close()
    (v0, r0, r0b), (v1, r1, r1b) = runs
    assert np.array_equal(v0, v1)
    assert r0 == r1 == r0b == r1b


def test_batched_runs_are_bit_identical():
    problems = synth.pose3_chains(64, seed=5, max_poses=50, max_landmarks=20)
    params = A.default_optimizer_params(iterations=30)
    out = []
    for _ in range(2):
        opt = BatchOptimizer(problems, params)
        res = opt.optimize(opt.initial_values())
        out.append((res.best_error.copy(), res.num_iterations.copy(), opt.get_values()))
        opt.close()
    assert all(np.array_equal(a, b) for a, b in zip(out[0], out[1]))


def test_device_wait_cap_ends_a_wait_that_nothing_satisfies():
    """Every dependency wait in the persistent kernels is capped; a wait on a flag that nothing
    sets ends at the cap with the error word set (no fault, no hang), and the device stays usable."""
    import ctypes as C
    from symforce_gb300.optimizer import lib
    L = lib()
    L.sfg_selftest_wait_cap.argtypes = [C.c_int32, C.POINTER(C.c_int32), C.POINTER(C.c_double)]
    status, ms = C.c_int32(-1), C.c_double()
    assert L.sfg_selftest_wait_cap(0, C.byref(status), C.byref(ms)) == 0
    assert status.value == 1  # the wait hit its cap
    assert 0.0 < ms.value < 10_000.0
    p = _ba()
    params = A.default_optimizer_params(lambda_update_type=A.SFG_LAMBDA_UPDATE_DYNAMIC, iterations=5)
    _, stats = Optimizer(p, params, A.default_form_params(linear_solver=A.SFG_LINEAR_SOLVER_SCHUR)).optimize(p.values)
    ref = O.optimize(p, params)
    assert stats.best_error == pytest.approx(ref["iterations"][ref["best_index"]].new_error, rel=1e-9)
