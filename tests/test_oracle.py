"""The CPU oracle pinned against the reference's own known answers and symbolic definitions."""

from __future__ import annotations

import json
from pathlib import Path

import numpy as np
import pytest

import oracle_lib as O
import reference_cases as R
from symforce_gb300 import _cabi as A
from symforce_gb300 import synth

GOLDEN = Path(__file__).resolve().parent / "golden"


def test_robot_2d_example_known_answers():
    """symforce/examples/robot_2d_localization/run_localization.cc:85-96 and
    test/symforce_examples_robot_2d_localization_test.py:48-50."""
    r = O.optimize(R.robot_2d_localization())
    E = R.ROBOT_2D_EXPECTED
    assert len(r["iterations"]) == E["num_iterations"]
    first = r["iterations"][0].new_error
    assert E["first_error_range"][0] < first < E["first_error_range"][1]
    assert first == pytest.approx(E["first_error_python"], rel=1e-15)
    assert r["iterations"][r["best_index"]].new_error < E["best_error_below"]
    assert r["status"] == A.SFG_STATUS_SUCCESS
    np.testing.assert_allclose(r["values"].reshape(-1, 4), E["poses"], atol=1e-6)


def test_pose_smoothing_known_answers():
    """test/symforce_optimizer_test.cc:142-176."""
    p = R.pose_smoothing(O.pose_smoothing_initial_values())
    r = O.optimize(p, A.default_optimizer_params(**R.POSE_SMOOTHING_PARAMS))
    last = r["iterations"][-1]
    assert last.iteration == R.POSE_SMOOTHING_EXPECTED["last_iteration"]
    lam, tol = R.POSE_SMOOTHING_EXPECTED["lambda_approx"]
    assert last.current_lambda == pytest.approx(lam, rel=tol)
    err, tol = R.POSE_SMOOTHING_EXPECTED["error_approx"]
    assert last.new_error == pytest.approx(err, rel=tol)
    assert r["status"] == A.SFG_STATUS_SUCCESS


def test_pose_smoothing_dynamic_lambda_known_answers():
    """test/symforce_optimizer_test.cc:461-506: DYNAMIC lambda on the pose-smoothing problem with
    otherwise default parameters gives SUCCESS / INVALID after 27 records, and the best
    linearization has 66 residual rows and a 60 x 60 lower Hessian with 534 stored entries."""
    p = R.pose_smoothing(O.pose_smoothing_initial_values())
    params = A.default_optimizer_params(lambda_update_type=A.SFG_LAMBDA_UPDATE_DYNAMIC)
    r = O.optimize(p, params)
    E = R.DYNAMIC_LAMBDA_EXPECTED
    assert r["status"] == A.SFG_STATUS_SUCCESS
    assert r["failure_reason"] == A.SFG_FAILURE_INVALID
    assert len(r["iterations"]) == E["num_records"]
    lin = O.linearize(p, r["values"])
    assert lin["residual"].size == E["residual_rows"] and np.isfinite(lin["residual"]).all()
    assert lin["rhs"].size == E["rhs_rows"] and np.isfinite(lin["rhs"]).all()
    assert lin["colptr"].size == E["hessian_dim"] + 1
    assert lin["hvals"].size == E["hessian_nnz"] and np.isfinite(lin["hvals"]).all()


def test_pose_smoothing_hessian_is_jtj():
    """H == lower(J^T J) (test/symforce_optimizer_test.cc:170-175), built from per-factor jets."""
    p = R.pose_smoothing(O.pose_smoothing_initial_values())
    lin = O.linearize(p)
    N = p.tangent_dim
    J = np.zeros((p.residual_dim, N))
    row = 0
    offs = np.cumsum([0] + [A.KEY_DIMS[int(t)][1] for t in p.key_types])
    soffs = p.key_storage_offsets()
    for b in p.batches:
        for f in range(b.count):
            keys = b.keys[f]
            st = np.concatenate([p.values[soffs[k]:soffs[k + 1]] for k in keys])
            res, Jf = O.factor_linearize(b.kind, [p.key_types[k] for k in keys], st, b.consts[f])
            c = 0
            for k in keys:
                d = A.KEY_DIMS[int(p.key_types[k])][1]
                J[row:row + len(res), offs[k]:offs[k] + d] = Jf[:, c:c + d]
                c += d
            row += len(res)
    H = np.zeros((N, N))
    for col in range(N):
        for q in range(lin["colptr"][col], lin["colptr"][col + 1]):
            H[lin["rowidx"][q], col] = lin["hvals"][q]
    np.testing.assert_allclose(np.tril(H), np.tril(J.T @ J), rtol=1e-12, atol=1e-10)
    np.testing.assert_allclose(lin["rhs"], J.T @ lin["residual"], rtol=1e-12, atol=1e-10)


def _golden_vectors():
    return json.loads((GOLDEN / "factor_vectors.json").read_text())["vectors"]


@pytest.mark.parametrize("vec", _golden_vectors(), ids=lambda v: f"kind{v['kind']}")
def test_factor_matches_symforce_symbolic(vec):
    """Residual and tangent Jacobian against the reference's symbolic factor definitions
    (fixtures made by tests/golden/make_symforce_factor_vectors.py)."""
    res, J = O.factor_linearize(vec["kind"], vec["key_types"], vec["storage"], vec["consts"])
    np.testing.assert_allclose(res, vec["residual"], rtol=1e-10, atol=1e-12)
    Jg = np.array(vec["jacobian"])
    np.testing.assert_allclose(J, Jg, rtol=1e-8, atol=1e-9 * max(1.0, np.abs(Jg).max()))


def _random_spd_csc(n, density, seed):
    rng = np.random.default_rng(seed)
    M = rng.normal(size=(n, n)) * (rng.uniform(size=(n, n)) < density)
    A_ = M @ M.T + n * np.eye(n)
    L = np.tril(A_)
    colptr, rowidx, vals = [0], [], []
    for c in range(n):
        rows = np.nonzero(L[:, c])[0]
        rows = rows[rows >= c]
        rowidx += list(rows)
        vals += list(L[rows, c])
        colptr.append(len(rowidx))
    return A_, np.array(colptr, np.int64), np.array(rowidx, np.int32), np.array(vals)


@pytest.mark.parametrize("ordering", [A.SFG_ORDERING_NATURAL, A.SFG_ORDERING_MIN_DEGREE])
def test_ldlt_matches_dense(ordering):
    """Random SPD systems (test/sparse_cholesky_solver_test.cc:59-131)."""
    for seed in range(3):
        A_, cp, ri, v = _random_spd_csc(40, 0.1, seed)
        b = np.random.default_rng(seed + 10).normal(size=40)
        x, D, perm = O.ldlt_solve(40, cp, ri, v, b, ordering=ordering)
        np.testing.assert_allclose(x, np.linalg.solve(A_, b), rtol=1e-10, atol=1e-12)
        assert sorted(perm) == list(range(40))


def test_schur_matches_ldlt():
    """Schur vs full LDL^T on a BA Hessian (test/sparse_schur_solver_test.cc:105-250)."""
    p = synth.bundle_adjustment(num_cameras=5, num_points=40, num_observations=160, seed=2)
    lin = O.linearize(p)
    N = p.tangent_dim
    vals = lin["hvals"].copy()
    for c in range(N):  # damp to make it SPD
        q = lin["colptr"][c] + np.searchsorted(lin["rowidx"][lin["colptr"][c]:lin["colptr"][c + 1]], c)
        vals[q] += 1.0
    b = lin["rhs"]
    x1, _, _ = O.ldlt_solve(N, lin["colptr"], lin["rowidx"], vals, b)
    x2 = O.schur_solve(N, lin["colptr"], lin["rowidx"], vals, 3 * p.num_schur_keys, b)
    np.testing.assert_allclose(x2, x1, rtol=1e-8, atol=1e-10 * np.abs(x1).max())


def test_retract_pose3_matches_reference_formula():
    q = np.array([0.1, -0.2, 0.3, 0.9])
    q /= np.linalg.norm(q)
    st = np.concatenate([q, [1.0, 2.0, 3.0]])
    d = np.array([0.01, -0.02, 0.03, 0.1, 0.2, 0.3])
    out = O.retract(A.SFG_KEY_POSE3, st, d)
    th = np.linalg.norm(d[:3])
    dq = np.concatenate([np.sin(th / 2) / th * d[:3], [np.cos(th / 2)]])
    expect = synth.quat_mul(q, dq)
    np.testing.assert_allclose(out[:4], expect, atol=1e-14)
    np.testing.assert_allclose(out[4:], st[4:] + d[3:], atol=1e-15)


def test_ba_oracle_fixture_is_reproducible():
    """The committed oracle cost of the benchmark workload is what the oracle computes now."""
    from symforce_gb300 import workloads
    fx = json.loads((GOLDEN / "oracle_costs.json").read_text())
    w = workloads.get("robot2d_1000")
    r = O.optimize(w.problem(), w.params())
    assert r["iterations"][r["best_index"]].new_error == pytest.approx(fx["robot2d_1000"]["best_error"], rel=1e-12)


def test_rot3_smoothing_known_answers():
    """test/symforce_optimizer_test.cc:183-261 (generated Rot3 prior / between kinds): last
    iteration 6, lambda ~2.4e-4, error ~2.174, SUCCESS, and H == lower(J^T J)."""
    p = R.rot3_smoothing(O.rot3_smoothing_initial_values())
    r = O.optimize(p, A.default_optimizer_params(**R.ROT3_SMOOTHING_PARAMS))
    last = r["iterations"][-1]
    E = R.ROT3_SMOOTHING_EXPECTED
    assert last.iteration == E["last_iteration"]
    assert last.current_lambda == pytest.approx(E["lambda_approx"][0], rel=E["lambda_approx"][1])
    assert last.new_error == pytest.approx(E["error_approx"][0], rel=E["error_approx"][1])
    assert r["status"] == A.SFG_STATUS_SUCCESS


def _linear_J():
    # sym::Random<Eigen::Matrix<double, 9, 5>>(std::mt19937(12345)): column-major coefficient order
    return O.mt19937_normal_vectors(12345, 1, 45)[0].reshape(5, 9).T


def test_linear_problem_converges_in_one_iteration():
    """test/symforce_levenberg_marquardt_test.cc:17-88: initial error > 1e4, after one undamped
    Gauss-Newton iteration the error is below 1e-8 and |x| < 1e-4."""
    p = R.linear_problem(_linear_J())
    r = O.optimize(p, R.linear_problem_params(), epsilon=R.LINEAR_PROBLEM_EPSILON)
    assert r["iterations"][0].new_error > 1e4
    assert len(r["iterations"]) == 2
    assert r["iterations"][-1].new_error < 1e-8
    assert np.linalg.norm(r["values"]) < 1e-4


def test_gnc_known_answers():
    """test/symforce_gnc_test.cc:22-76: 9 records in all, |x| < 0.1, five times closer to zero than
    the plain optimization at mu = 0, SUCCESS."""
    y = R.gnc_samples(O.mt19937_normal_vectors(42, 20, 5))
    p = R.gnc_problem(y)
    params = A.default_optimizer_params()
    r = O.gnc_optimize(p, params, R.gnc_params(), R.GNC_MU_SLOTS, epsilon=R.GNC_OPTIMIZER_EPSILON)
    assert len(r["iterations"]) == R.GNC_EXPECTED["num_records"]
    assert r["status"] == A.SFG_STATUS_SUCCESS
    x = r["values"]
    assert np.linalg.norm(x) < 0.1
    plain = O.optimize(R.gnc_problem(y), params)
    assert np.linalg.norm(x) * 5 < np.linalg.norm(plain["values"])


@pytest.mark.parametrize("factor_order", ["dense_sparse", "sparse_dense"])
def test_linearizer_consistency(factor_order):
    """test/symforce_linearizer_test.cc:51-127: J^T J == H and J^T r == rhs exactly in either factor
    order, and the key order permutes the Jacobian's columns."""
    J = np.vstack([np.diag([1.0, 2.0]), np.diag([3.0, 4.0])])
    if factor_order == "sparse_dense":
        J = np.vstack([J[2:], J[:2]])
    for key_order in ("xy", "yx"):
        p = R.linearizer_problem(factor_order, key_order)
        lin = O.linearize(p)
        Jk = J if key_order == "xy" else J[:, ::-1]
        H = np.zeros((2, 2))
        for c in range(2):
            for q in range(lin["colptr"][c], lin["colptr"][c + 1]):
                H[lin["rowidx"][q], c] = lin["hvals"][q]
        H = np.tril(H) + np.tril(H, -1).T
        np.testing.assert_array_equal(H, Jk.T @ Jk)
        np.testing.assert_array_equal(lin["rhs"], Jk.T @ lin["residual"])
        np.testing.assert_array_equal(lin["residual"], Jk @ p.values)
