"""The batched form: every problem of a batch of Pose3 chains reaches the CPU oracle's result
(same LM records, best cost within 1e-9 relative, same status), in one launch."""

from __future__ import annotations

import numpy as np
import pytest

import oracle_lib as O
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


def test_batch_rejects_unsupported_structure():
    p = synth.pose3_chain(6, 10, 1)
    bad = A.ProblemArrays(key_types=p.key_types,
                          batches=[A.Batch(A.SFG_FACTOR_BETWEEN_POSE3, np.array([[0, 2]]), p.batches[1].consts[:1])],
                          values=p.values)
    with pytest.raises(SfgError) as e:
        BatchOptimizer([bad])
    assert e.value.code == 4  # SFG_ERR_STRUCTURE
