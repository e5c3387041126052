"""GPU parity of the full Levenberg-Marquardt loop against the CPU oracle and the reference's own
known answers (all through the C ABI)."""

from __future__ import annotations

import numpy as np
import pytest

import oracle_lib as O
import reference_cases as R
from symforce_gb300 import _cabi as A
from symforce_gb300 import synth
from symforce_gb300.optimizer import Optimizer

pytestmark = pytest.mark.gpu


def _records(stats_iters):
    return [(r.iteration, r.current_lambda, r.new_error, r.update_accepted) for r in stats_iters]


def test_robot_2d_example_known_answers():
    p = R.robot_2d_localization()
    opt = Optimizer(p, form=A.default_form_params(ordering=A.SFG_ORDERING_NESTED_DISSECTION))
    values, stats = opt.optimize(p.values)
    E = R.ROBOT_2D_EXPECTED
    assert len(stats.iterations) == E["num_iterations"]
    assert E["first_error_range"][0] < stats.iterations[0].new_error < E["first_error_range"][1]
    assert stats.iterations[0].new_error == pytest.approx(E["first_error_python"], rel=1e-14)
    assert stats.best_error < E["best_error_below"]
    assert stats.status == A.SFG_STATUS_SUCCESS
    np.testing.assert_allclose(values.reshape(-1, 4), E["poses"], atol=1e-6)
    ref = O.optimize(p)
    for g, o in zip(stats.iterations, ref["iterations"]):
        assert g.iteration == o.iteration and g.update_accepted == o.update_accepted
        assert g.current_lambda == pytest.approx(o.current_lambda, rel=1e-12)
        assert g.new_error == pytest.approx(o.new_error, rel=1e-9, abs=1e-14)


def test_pose_smoothing_known_answers():
    v0 = O.pose_smoothing_initial_values()
    p = R.pose_smoothing(v0)
    params = A.default_optimizer_params(**R.POSE_SMOOTHING_PARAMS)
    opt = Optimizer(p, params)
    values, stats = opt.optimize(p.values)
    last = stats.iterations[-1]
    assert last.iteration == R.POSE_SMOOTHING_EXPECTED["last_iteration"]
    lam, tol = R.POSE_SMOOTHING_EXPECTED["lambda_approx"]
    assert last.current_lambda == pytest.approx(lam, rel=tol)
    err, tol = R.POSE_SMOOTHING_EXPECTED["error_approx"]
    assert last.new_error == pytest.approx(err, rel=tol)
    assert stats.status == A.SFG_STATUS_SUCCESS


def test_pose_smoothing_dynamic_lambda_known_answers():
    """test/symforce_optimizer_test.cc:461-506 on the GPU: SUCCESS / INVALID after 27 records, every
    record as the oracle's (accept flags exact, lambda and error at 1e-9), and the linearization at
    the best values has 66 residual rows and a 60 x 60 lower Hessian with 534 stored entries, all
    finite."""
    p = R.pose_smoothing(O.pose_smoothing_initial_values())
    params = A.default_optimizer_params(lambda_update_type=A.SFG_LAMBDA_UPDATE_DYNAMIC)
    opt = Optimizer(p, params)
    values, stats = opt.optimize(p.values)
    E = R.DYNAMIC_LAMBDA_EXPECTED
    assert stats.status == A.SFG_STATUS_SUCCESS
    assert stats.failure_reason == A.SFG_FAILURE_INVALID
    assert len(stats.iterations) == E["num_records"]
    ref = O.optimize(p, params)
    assert len(ref["iterations"]) == len(stats.iterations)
    for g, o in zip(stats.iterations, ref["iterations"]):
        assert g.iteration == o.iteration and g.update_accepted == o.update_accepted
        assert g.current_lambda == pytest.approx(o.current_lambda, rel=1e-9)
        assert g.new_error == pytest.approx(o.new_error, rel=1e-9)
    assert stats.best_index == ref["best_index"]
    lin = opt.linearize(values)
    assert lin["residual"].size == E["residual_rows"] and np.isfinite(lin["residual"]).all()
    assert lin["rhs"].size == E["rhs_rows"] and np.isfinite(lin["rhs"]).all()
    assert lin["colptr"].size == E["hessian_dim"] + 1
    assert lin["hvals"].size == E["hessian_nnz"] and np.isfinite(lin["hvals"]).all()
    o = O.linearize(p, values)
    np.testing.assert_array_equal(lin["colptr"], o["colptr"])
    np.testing.assert_array_equal(lin["rowidx"], o["rowidx"])
    np.testing.assert_allclose(lin["hvals"], o["hvals"], rtol=1e-9, atol=1e-12 * np.abs(o["hvals"]).max())


def test_debug_stats_and_best_linearization():
    """populate_best_linearization and debug_stats (symforce/opt/optimization_stats.h:34-58): the
    best linearization equals the oracle's at the best values; the ordering is a permutation and
    the factor's sparsity is a strict-lower CSC of the right size."""
    p = synth.bundle_adjustment(num_cameras=6, num_points=80, num_observations=320, seed=4)
    params = A.default_optimizer_params(lambda_update_type=A.SFG_LAMBDA_UPDATE_DYNAMIC, iterations=10,
                                        debug_stats=1)
    opt = Optimizer(p, params, A.default_form_params(linear_solver=A.SFG_LINEAR_SOLVER_SCHUR))
    values, stats = opt.optimize(p.values, populate_best_linearization=True)
    bl = stats.best_linearization
    o = O.linearize(p, values)
    np.testing.assert_allclose(bl["residual"], o["residual"], rtol=1e-12, atol=1e-12)
    np.testing.assert_allclose(bl["hessian_lower"]["values"], o["hvals"], rtol=1e-9,
                               atol=1e-12 * np.abs(o["hvals"]).max())
    assert bl["error"] == pytest.approx(stats.best_error, rel=1e-12)
    n = 6 * 9
    assert sorted(stats.linear_solver_ordering.tolist()) == list(range(n))
    sp = stats.cholesky_factor_sparsity
    assert sp["shape"] == (n, n) and sp["colptr"].size == n + 1
    for c in range(n):
        assert (sp["rowidx"][sp["colptr"][c]:sp["colptr"][c + 1]] > c).all()


def test_linearization_matches_oracle_ba_small():
    p = synth.bundle_adjustment(num_cameras=8, num_points=120, num_observations=500, seed=3)
    opt = Optimizer(p, form=A.default_form_params(linear_solver=A.SFG_LINEAR_SOLVER_SCHUR))
    g = opt.linearize(p.values)
    o = O.linearize(p)
    np.testing.assert_allclose(g["residual"], o["residual"], rtol=1e-12, atol=1e-12)
    np.testing.assert_array_equal(g["colptr"], o["colptr"])
    np.testing.assert_array_equal(g["rowidx"], o["rowidx"])
    scale = np.abs(o["hvals"]).max()
    np.testing.assert_allclose(g["hvals"], o["hvals"], rtol=1e-9, atol=1e-12 * scale)
    np.testing.assert_allclose(g["rhs"], o["rhs"], rtol=1e-9, atol=1e-12 * np.abs(o["rhs"]).max())


@pytest.mark.parametrize("solver", [A.SFG_LINEAR_SOLVER_SCHUR, A.SFG_LINEAR_SOLVER_SPARSE_LDLT])
def test_ba_small_matches_oracle(solver):
    p = synth.bundle_adjustment(num_cameras=10, num_points=300, num_observations=1300, seed=1)
    params = A.default_optimizer_params(lambda_update_type=A.SFG_LAMBDA_UPDATE_DYNAMIC, iterations=20)
    opt = Optimizer(p, params, A.default_form_params(linear_solver=solver))
    values, stats = opt.optimize(p.values)
    ref = O.optimize(p, params, linear_solver=A.SFG_LINEAR_SOLVER_SPARSE_LDLT)
    assert len(stats.iterations) == len(ref["iterations"])
    for g, o in zip(stats.iterations, ref["iterations"]):
        assert g.update_accepted == o.update_accepted
        assert g.new_error == pytest.approx(o.new_error, rel=1e-9)
    assert stats.best_error == pytest.approx(ref["iterations"][ref["best_index"]].new_error, rel=1e-9)
    assert stats.status == ref["status"]


def test_robot_2d_config_matches_oracle():
    p = synth.robot_2d(200, seed=2)
    params = A.default_optimizer_params(iterations=30)
    opt = Optimizer(p, params)
    values, stats = opt.optimize(p.values)
    ref = O.optimize(p, params)
    assert stats.best_error == pytest.approx(ref["iterations"][ref["best_index"]].new_error, rel=1e-9)


@pytest.mark.parametrize("name", ["robot2d_1000", "ba_50_7800", "ba_1000_200k"])
def test_benchmark_workloads_match_committed_oracle_records(name):
    """Full-size parity: the plain FP64 form on the benchmark workloads (2D localization with 1,000
    Pose2 and 50 iterations, sparse LDL^T; the 50- and 1,000-camera bundle adjustments, Schur) follows
    the CPU oracle's
    committed LM trajectory (tests/golden/oracle_costs.json, generated by
    tests/golden/make_oracle_costs.py): same number of records, same accept decisions, every
    error at 1e-9 relative, same status."""
    import json
    from pathlib import Path
    from symforce_gb300 import workloads
    ref = json.loads((Path(__file__).resolve().parent / "golden" / "oracle_costs.json").read_text())[name]
    w = workloads.get(name)
    p = w.problem()
    opt = Optimizer(p, w.params(), w.form(A.SFG_PRECISION_FP64))
    _, stats = opt.optimize(p.values)
    assert len(stats.iterations) == ref["num_records"]
    assert [int(r.update_accepted) for r in stats.iterations] == [int(a) for a in ref["accepted"]]
    for g, e in zip(stats.iterations, ref["errors"]):
        assert g.new_error == pytest.approx(e, rel=1e-9)
    assert stats.best_error == pytest.approx(ref["best_error"], rel=1e-9)
    assert stats.status == ref["status"]


def test_compute_covariances_matches_dense_inverse():
    """Optimizer::ComputeCovariances (Schur over the points, C damped by epsilon): per-key marginal
    covariances of the camera keys equal the diagonal blocks of the dense inverse of the damped
    Hessian (oracle linearization)."""
    p = synth.bundle_adjustment(num_cameras=6, num_points=150, num_observations=600, seed=9)
    # priors on two camera poses remove the similarity gauge, so the Hessian is invertible
    prior = [np.concatenate([p.values[7 * c:7 * c + 7], np.full(6, 10.0), [A.DEFAULT_EPSILON]]) for c in (0, 1)]
    p.batches.append(A.Batch(A.SFG_FACTOR_PRIOR_POSE3, np.array([[0], [1]]), np.array(prior)))
    opt = Optimizer(p, A.default_optimizer_params(lambda_update_type=A.SFG_LAMBDA_UPDATE_DYNAMIC, iterations=15),
                    A.default_form_params(linear_solver=A.SFG_LINEAR_SOLVER_SCHUR))
    best, _ = opt.optimize(p.values)
    nk = 2 * 6  # poses and intrinsics lead the key order
    cov = opt.compute_covariances(best, nk)
    o = O.linearize(p, best)
    N = o["rhs"].size
    H = np.zeros((N, N))
    for j in range(N):
        for q in range(o["colptr"][j], o["colptr"][j + 1]):
            H[o["rowidx"][q], j] = H[j, o["rowidx"][q]] = o["hvals"][q]
    bd = 6 * 6 + 6 * 3
    H[np.arange(bd, N), np.arange(bd, N)] += A.DEFAULT_EPSILON
    ref = np.linalg.inv(H)[:bd, :bd]
    offs = np.concatenate([[0], np.cumsum([6] * 6 + [3] * 6)])
    for k in range(nk):
        blk = ref[offs[k]:offs[k + 1], offs[k]:offs[k + 1]]
        np.testing.assert_allclose(cov[k], blk, rtol=1e-6, atol=1e-9 * np.abs(blk).max())
        np.testing.assert_allclose(cov[k], cov[k].T, rtol=0, atol=1e-12 * np.abs(blk).max())


@pytest.mark.parametrize("case", ["bundle_adjustment", "pose_smoothing"])
def test_dense_linearization_matches_oracle(case):
    """DenseLinearizer adapter (Optimizer.linearize_dense; symforce/opt/dense_linearizer.h): the
    device's residual, dense lower Hessian (upper triangle zero), rhs and error against the CPU
    oracle's linearization at the same values, at 1e-9."""
    if case == "bundle_adjustment":
        p = synth.bundle_adjustment(num_cameras=6, num_points=40, num_observations=150, seed=2)
    else:
        p = R.pose_smoothing(O.pose_smoothing_initial_values())
    opt = Optimizer(p)
    got = opt.linearize_dense(p.values)
    ref = O.linearize(p)
    n = len(ref["rhs"])
    Hd = np.zeros((n, n))
    for j in range(n):
        for q in range(int(ref["colptr"][j]), int(ref["colptr"][j + 1])):
            Hd[int(ref["rowidx"][q]), j] = ref["hvals"][q]
    Hd = np.tril(Hd + np.triu(Hd, 1).T)  # the oracle stores the lower triangle; keep it lower
    H = got["hessian_lower"]
    assert H.shape == (n, n)
    assert np.all(np.triu(H, 1) == 0.0)
    scale = max(1.0, np.abs(Hd).max())
    np.testing.assert_allclose(H, Hd, rtol=1e-9, atol=1e-9 * scale)
    np.testing.assert_allclose(got["rhs"], ref["rhs"], rtol=1e-9, atol=1e-9 * max(1.0, np.abs(ref["rhs"]).max()))
    np.testing.assert_allclose(got["residual"], ref["residual"], rtol=1e-9,
                               atol=1e-12 * max(1.0, np.abs(ref["residual"]).max()))
    assert got["error"] == pytest.approx(0.5 * float(ref["residual"] @ ref["residual"]), rel=1e-9)
    opt.close()
