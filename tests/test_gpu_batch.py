"""The batched form: every problem of a batch reaches the CPU oracle's result (same LM records,
best cost within 1e-9 relative, same status), in one launch — Pose3 chains on the block-tridiagonal
path, any other problems on the dense path."""

from __future__ import annotations

import numpy as np
import pytest

import oracle_lib as O
import reference_cases as R
from symforce_gb300 import _cabi as A
from symforce_gb300 import synth
from symforce_gb300.batch import BatchOptimizer
from symforce_gb300.optimizer import SfgError

pytestmark = pytest.mark.gpu


def _check_against_oracle(problems, params, res, opt, records_for=()):
    for i, p in enumerate(problems):
        r = O.optimize(p, params)
        best = r["iterations"][r["best_index"]].new_error
        assert res.status[i] == r["status"], (i, res.status[i], r["status"])
        assert res.num_iterations[i] == len(r["iterations"]), (i, res.num_iterations[i], len(r["iterations"]))
        assert abs(res.best_error[i] - best) <= 1e-9 * best, (i, res.best_error[i], best)
        if i in records_for:
            got = opt.records(i)
            for a, b in zip(got, r["iterations"]):
                assert a.update_accepted == b.update_accepted
                assert abs(a.new_error - b.new_error) <= 1e-9 * abs(b.new_error)
                # lambda follows the gain ratio, which amplifies rounding of the linearized error
                assert abs(a.current_lambda - b.current_lambda) <= 1e-8 * abs(b.current_lambda)


def test_batch_matches_oracle_per_problem():
    problems = synth.pose3_chains(48, seed=7, max_poses=60, max_landmarks=20)
    params = A.default_optimizer_params(iterations=50)
    opt = BatchOptimizer(problems, params)
    res = opt.optimize(opt.initial_values())
    _check_against_oracle(problems, params, res, opt, records_for=(0, 1, 2))
    # best values come back in problem order
    vals = opt.get_values()
    for i in (0, 5, 47):
        p = problems[i]
        r = O.optimize(p, params)
        np.testing.assert_allclose(vals[opt.offsets[i]:opt.offsets[i + 1]], r["values"], rtol=0, atol=1e-7)


def test_batch_dynamic_lambda_and_large_problems():
    problems = [synth.pose3_chain(200, 50, 11), synth.pose3_chain(5, 10, 12), synth.pose3_chain(150, 33, 13)]
    params = A.default_optimizer_params(iterations=50, lambda_update_type=A.SFG_LAMBDA_UPDATE_DYNAMIC)
    opt = BatchOptimizer(problems, params)
    res = opt.optimize(opt.initial_values())
    _check_against_oracle(problems, params, res, opt, records_for=(0,))


def test_batch_autotune_keeps_results():
    problems = synth.pose3_chains(64, seed=3, max_poses=40, max_landmarks=15)
    params = A.default_optimizer_params(iterations=30)
    opt = BatchOptimizer(problems, params)
    a = opt.optimize(opt.initial_values())
    w, c = opt.autotune()
    assert w in (1, 2, 4, 8) and c > 0
    b = opt.optimize(opt.initial_values())
    # launch shapes are different kernel instantiations: the same algorithm, rounding may differ
    assert np.array_equal(a.num_iterations, b.num_iterations) and np.array_equal(a.status, b.status)
    np.testing.assert_allclose(b.best_error, a.best_error, rtol=1e-12)


def _mixed_problems():
    """Problems of uneven size and structure that are not Pose3 chains: 2D localization (Pose2,
    odometry and bearings), small bundle adjustments (Pose3, intrinsics, points; Snavely factors),
    Pose3 and Rot3 smoothing (a generated factor kind), and a Pose3 chain closed into a loop."""
    probs = [synth.robot_2d(num_poses=n, num_landmarks=6, seed=20 + n) for n in (8, 21, 40)]
    probs += [synth.bundle_adjustment(num_cameras=c, num_points=pts, num_observations=3 * pts, seed=c + pts,
                                      max_views=3)
              for c, pts in ((3, 12), (4, 25), (3, 8))]
    probs.append(R.pose_smoothing(O.pose_smoothing_initial_values()))
    probs.append(R.rot3_smoothing(O.rot3_smoothing_initial_values()))
    probs.append(synth.loop_closed_pose3_chain(12, 10, 5))
    return probs


def test_batch_dense_path_matches_oracle_per_problem():
    problems = _mixed_problems()
    for params in (A.default_optimizer_params(iterations=40),
                   A.default_optimizer_params(iterations=40, lambda_update_type=A.SFG_LAMBDA_UPDATE_DYNAMIC)):
        opt = BatchOptimizer(problems, params)
        res = opt.optimize(opt.initial_values())
        _check_against_oracle(problems, params, res, opt, records_for=(0, 3, 7))
        vals = opt.get_values()
        for i in (2, 6, 8):  # problems with priors; bundle adjustment leaves a gauge free
            r = O.optimize(problems[i], params)
            np.testing.assert_allclose(vals[opt.offsets[i]:opt.offsets[i + 1]], r["values"], rtol=0, atol=1e-7)
        opt.close()


def test_batch_dense_path_autotune_and_repeat():
    problems = _mixed_problems() * 20
    params = A.default_optimizer_params(iterations=30)
    opt = BatchOptimizer(problems, params)
    a = opt.optimize(opt.initial_values())
    b = opt.optimize(opt.initial_values())
    np.testing.assert_array_equal(a.best_error, b.best_error)  # fixed orders: the same bits
    w, c = opt.autotune()
    assert w in (1, 2, 4, 8) and c > 0
    d = opt.optimize(opt.initial_values())
    assert np.array_equal(a.num_iterations, d.num_iterations) and np.array_equal(a.status, d.status)
    np.testing.assert_allclose(d.best_error, a.best_error, rtol=1e-12)


def test_batch_rejects_unsupported_structure():
    # a tangent dimension above the dense path's 128
    p = synth.pose3_chain(30, 10, 1)
    loop = A.Batch(A.SFG_FACTOR_BETWEEN_POSE3, np.array([[0, 29]]), p.batches[1].consts[:1])
    big = A.ProblemArrays(key_types=p.key_types, batches=list(p.batches) + [loop], values=p.values)
    with pytest.raises(SfgError) as e:
        BatchOptimizer([big])
    assert e.value.code == 4  # SFG_ERR_STRUCTURE
    # a factor whose two keys are the same key
    q = synth.pose3_chain(6, 10, 1)
    same = A.Batch(A.SFG_FACTOR_BETWEEN_POSE3, np.array([[2, 2]]), q.batches[1].consts[:1])
    bad = A.ProblemArrays(key_types=q.key_types, batches=list(q.batches) + [same], values=q.values)
    with pytest.raises(SfgError) as e:
        BatchOptimizer([bad])
    assert e.value.code == 4
