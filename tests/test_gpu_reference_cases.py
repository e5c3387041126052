"""The reference's own known-answer tests on the GPU, through the C ABI, with the factor kinds the
library generates from symbolic definitions (Rot3 prior / between, the GNC Barron factor, linear
factors) and the graduated non-convexity schedule over the device loop.  Each case is also checked
record by record against the CPU oracle."""

from __future__ import annotations

import numpy as np
import pytest

import oracle_lib as O
import reference_cases as R
from symforce_gb300 import _cabi as A
from symforce_gb300.optimizer import GncOptimizer, Optimizer

pytestmark = pytest.mark.gpu


def _match_records(gpu_iters, ref_iters, rel=1e-9):
    assert len(gpu_iters) == len(ref_iters)
    for g, o in zip(gpu_iters, ref_iters):
        assert g.iteration == o.iteration and g.update_accepted == o.update_accepted
        assert g.current_lambda == pytest.approx(o.current_lambda, rel=rel)
        assert g.new_error == pytest.approx(o.new_error, rel=rel, abs=1e-14)


def test_rot3_smoothing_known_answers():
    """test/symforce_optimizer_test.cc:183-261: last iteration 6, lambda ~2.4e-4, error ~2.174,
    SUCCESS; H == lower(J^T J) at the optimum (oracle Jacobians)."""
    p = R.rot3_smoothing(O.rot3_smoothing_initial_values())
    params = A.default_optimizer_params(**R.ROT3_SMOOTHING_PARAMS)
    opt = Optimizer(p, params)
    values, stats = opt.optimize(p.values)
    last = stats.iterations[-1]
    E = R.ROT3_SMOOTHING_EXPECTED
    assert last.iteration == E["last_iteration"]
    assert last.current_lambda == pytest.approx(E["lambda_approx"][0], rel=E["lambda_approx"][1])
    assert last.new_error == pytest.approx(E["error_approx"][0], rel=E["error_approx"][1])
    assert stats.status == A.SFG_STATUS_SUCCESS
    _match_records(stats.iterations, O.optimize(p, params)["iterations"])
    lin = opt.linearize(values)
    o = O.linearize(p, values)
    np.testing.assert_array_equal(lin["colptr"], o["colptr"])
    np.testing.assert_allclose(lin["hvals"], o["hvals"], rtol=1e-9, atol=1e-12 * np.abs(o["hvals"]).max())


@pytest.mark.parametrize("precision", [A.SFG_PRECISION_FP64, A.SFG_PRECISION_MIXED])
def test_linear_problem_converges_in_one_iteration(precision):
    """test/symforce_levenberg_marquardt_test.cc:17-88 (its double and float cases: the FP64 and the
    mixed-precision forms)."""
    J = O.mt19937_normal_vectors(12345, 1, 45)[0].reshape(5, 9).T
    p = R.linear_problem(J)
    form = A.default_form_params(precision=precision, epsilon=R.LINEAR_PROBLEM_EPSILON)
    opt = Optimizer(p, R.linear_problem_params(), form)
    values, stats = opt.optimize(p.values)
    assert stats.iterations[0].new_error > 1e4
    assert len(stats.iterations) == 2
    assert stats.iterations[-1].new_error < 1e-8
    assert np.linalg.norm(values) < 1e-4


def test_gnc_known_answers_and_oracle_records():
    """test/symforce_gnc_test.cc:22-76: 9 records over the GNC stages, |x| < 0.1, five times closer to
    zero than the plain optimization at mu = 0, SUCCESS; every record as the oracle's GNC run."""
    y = R.gnc_samples(O.mt19937_normal_vectors(42, 20, 5))
    params = A.default_optimizer_params()
    form = A.default_form_params(epsilon=R.GNC_OPTIMIZER_EPSILON)
    gnc = GncOptimizer(R.gnc_problem(y), params, R.gnc_params(), R.GNC_MU_SLOTS, form)
    x, stats = gnc.optimize(np.ones(5))
    assert len(stats.iterations) == R.GNC_EXPECTED["num_records"]
    assert stats.status == A.SFG_STATUS_SUCCESS
    assert np.linalg.norm(x) < 0.1
    plain_opt = Optimizer(R.gnc_problem(y), params)
    x_plain, _ = plain_opt.optimize(np.ones(5))
    assert np.linalg.norm(x) * 5 < np.linalg.norm(x_plain)
    ref = O.gnc_optimize(R.gnc_problem(y), params, R.gnc_params(), R.GNC_MU_SLOTS,
                         epsilon=R.GNC_OPTIMIZER_EPSILON)
    _match_records(stats.iterations, ref["iterations"])
    assert stats.best_index == ref["best_index"]
    np.testing.assert_allclose(x, ref["values"], rtol=1e-9, atol=1e-12)


@pytest.mark.parametrize("factor_order", ["dense_sparse", "sparse_dense"])
def test_linearizer_consistency(factor_order):
    """test/symforce_linearizer_test.cc:51-127 on the device: J^T J == H and J^T r == rhs exactly,
    the key order permutes the columns, and relinearizing gives identical bits."""
    J = np.vstack([np.diag([1.0, 2.0]), np.diag([3.0, 4.0])])
    if factor_order == "sparse_dense":
        J = np.vstack([J[2:], J[:2]])
    for key_order in ("xy", "yx"):
        p = R.linearizer_problem(factor_order, key_order)
        opt = Optimizer(p)
        lin = opt.linearize(p.values)
        Jk = J if key_order == "xy" else J[:, ::-1]
        H = np.zeros((2, 2))
        for c in range(2):
            for q in range(lin["colptr"][c], lin["colptr"][c + 1]):
                H[lin["rowidx"][q], c] = lin["hvals"][q]
        H = np.tril(H) + np.tril(H, -1).T
        np.testing.assert_array_equal(H, Jk.T @ Jk)
        np.testing.assert_array_equal(lin["rhs"], Jk.T @ lin["residual"])
        np.testing.assert_array_equal(lin["residual"], Jk @ p.values)
        again = opt.linearize(p.values)
        for k in ("residual", "rhs", "hvals"):
            np.testing.assert_array_equal(again[k], lin[k])
