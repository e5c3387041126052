"""The PCG forms and the learned preconditioner on the GPU: network gradient / inference against
the oracle, device-recorded training samples against the oracle's reduced system, PCG forms reaching
the FP64 oracle's cost, the exact-factorization fallback and judge, and the trained network's gain
over block Jacobi."""

from __future__ import annotations

import json
from pathlib import Path

import numpy as np
import pytest

import oracle_lib as O
import precond_cases as PC
from oracle import precond_net as PN
from symforce_gb300 import _cabi as A
from symforce_gb300 import learned, synth, workloads
from symforce_gb300.optimizer import Optimizer

pytestmark = pytest.mark.gpu

ROOT = Path(__file__).resolve().parents[1]


def test_network_gradient_matches_oracle():
    samples = PC.oracle_samples((3, 5)).astype(np.float32)
    w = PC.random_weights(4, out_scale=0.1)
    loss, grad = learned.loss_grad(samples, w)
    ref_loss, ref_grad = PN.loss_grad(w.astype(np.float64), samples.astype(np.float64))
    assert abs(loss - ref_loss) <= 1e-4 * ref_loss, (loss, ref_loss)
    offs = np.cumsum([0, 96 * 256, 256, 256 * 256, 256, 256 * 45, 45])
    for a, b in zip(offs[:-1], offs[1:]):  # per layer, relative to the layer's largest entry
        scale = np.abs(ref_grad[a:b]).max()
        np.testing.assert_allclose(grad[a:b], ref_grad[a:b], rtol=0, atol=2e-4 * scale)


def test_network_inference_matches_oracle():
    samples = PC.oracle_samples((3,)).astype(np.float32)
    w = PC.random_weights(5, out_scale=0.1)
    z = learned.infer(samples[:, :96], w)
    ref = PN.forward(w.astype(np.float64), samples[:, :96].astype(np.float64))
    np.testing.assert_allclose(z, ref, rtol=0, atol=1e-4 * np.abs(ref).max())


def test_training_reduces_loss():
    samples = PC.oracle_samples((3, 5, 6, 7)).astype(np.float32)
    w0 = learned.init_weights(0)
    l0, _ = learned.loss_grad(samples, w0)
    w, curve = learned.train(samples, steps=300, batch=16, lr=1e-3, seed=1, weights=w0)
    l1, _ = learned.loss_grad(samples, w)
    assert np.all(np.isfinite(curve))
    assert l1 < 0.9 * l0, (l0, l1)
    # deterministic: same inputs, same bits
    w2, curve2 = learned.train(samples, steps=300, batch=16, lr=1e-3, seed=1, weights=w0)
    assert np.array_equal(w, w2) and np.array_equal(curve, curve2)


def test_recorded_samples_match_oracle_system():
    """Samples the plain FP64 Schur path records on the device at the first LM iteration equal the
    oracle's restatement on the reduced system S y = v (lambda = 1, unit damping)."""
    p = PC.small_ba(3)
    params = A.default_optimizer_params(lambda_update_type=A.SFG_LAMBDA_UPDATE_DYNAMIC, iterations=1)
    opt = Optimizer(p, params, A.default_form_params(linear_solver=A.SFG_LINEAR_SOLVER_SCHUR))
    opt.collect_samples(4)
    opt.optimize(p.values, num_iterations=1)
    got = opt.samples()
    S, v = PC.reduced_system(p, lam=1.0)
    gidx, degree = PC.camera_blocks(p)
    ref = PN.samples_of_system(S, v, gidx, degree)
    assert got.shape == ref.shape
    np.testing.assert_allclose(got[:, :96], ref[:, :96], rtol=0, atol=2e-5)
    for part in (slice(96, 105), slice(105, 114)):
        scale = np.abs(ref[:, part]).max(axis=1, keepdims=True)
        dev = np.abs(got[:, part] - ref[:, part]) / scale
        assert dev.max() <= 1e-4, dev.max()


def _oracle_best(p, params):
    r = O.optimize(p, params)
    return r["iterations"][r["best_index"]].new_error


@pytest.mark.parametrize("precision", [A.SFG_PRECISION_FP64, A.SFG_PRECISION_MIXED])
@pytest.mark.parametrize("solver", [A.SFG_LINEAR_SOLVER_PCG_BLOCK_JACOBI, A.SFG_LINEAR_SOLVER_PCG_LEARNED])
def test_pcg_forms_reach_oracle_cost(solver, precision):
    p = synth.bundle_adjustment(num_cameras=12, num_points=400, num_observations=1700, seed=4)
    params = A.default_optimizer_params(lambda_update_type=A.SFG_LAMBDA_UPDATE_DYNAMIC, iterations=30)
    ref = _oracle_best(p, params)
    # the learned form with small random weights (every layer active); the trained weights are
    # exercised on the benchmark workload below
    w = PC.random_weights(7, out_scale=0.02) if solver == A.SFG_LINEAR_SOLVER_PCG_LEARNED else None
    opt = Optimizer(p, params, A.default_form_params(precision=precision, linear_solver=solver), weights=w)
    _, stats = opt.optimize(p.values)
    best = min(r.best_error for r in stats.iterations)
    assert best <= ref * (1 + 1e-6), (best, ref)
    ps = opt.pcg_stats()
    assert ps["solves"] == len(stats.iterations) - 1 and ps["fallbacks"] == 0, ps
    assert ps["max_rel_residual"] <= 1e-8, ps


def test_learned_form_reaches_oracle_cost_on_benchmark_workload():
    wl = workloads.get("ba_50_7800")
    p = wl.problem()
    ref = json.loads((ROOT / "tests" / "golden" / "oracle_costs.json").read_text())["ba_50_7800"]["best_error"]
    opt = Optimizer(p, wl.params(), A.default_form_params(precision=A.SFG_PRECISION_MIXED,
                                                        linear_solver=A.SFG_LINEAR_SOLVER_PCG_LEARNED))
    _, stats = opt.optimize(p.values)
    best = min(r.best_error for r in stats.iterations)
    assert abs(best - ref) <= 1e-6 * ref, (best, ref)
    ps = opt.pcg_stats()
    assert ps["fallbacks"] == 0, ps
    judge = opt.pcg_step_error()
    assert judge["rel_residual"] <= 1e-8, judge
    assert judge["rel_step_error"] <= 1e-4, judge


def test_fallback_runs_exact_factorization():
    """An iteration cap of 2 makes every PCG solve miss 1e-8: the exact LDL^T takes over and the
    optimizer still reaches the oracle's cost."""
    p = synth.bundle_adjustment(num_cameras=12, num_points=400, num_observations=1700, seed=4)
    params = A.default_optimizer_params(lambda_update_type=A.SFG_LAMBDA_UPDATE_DYNAMIC, iterations=30)
    ref = _oracle_best(p, params)
    for precision in (A.SFG_PRECISION_FP64, A.SFG_PRECISION_MIXED):
        opt = Optimizer(p, params, A.default_form_params(precision=precision, pcg_max_iters=2,
                                                         linear_solver=A.SFG_LINEAR_SOLVER_PCG_BLOCK_JACOBI))
        _, stats = opt.optimize(p.values)
        ps = opt.pcg_stats()
        assert ps["solves"] > 0 and ps["fallbacks"] == ps["solves"], ps
        best = min(r.best_error for r in stats.iterations)
        assert best <= ref * (1 + 1e-6), (precision, best, ref)


def test_trained_network_beats_block_jacobi():
    """Held-out problems (seeds outside the training set): the trained preconditioner needs fewer
    PCG iterations than block Jacobi for the same LM solve."""
    w = learned.load_weights()
    params = A.default_optimizer_params(lambda_update_type=A.SFG_LAMBDA_UPDATE_DYNAMIC, iterations=100)
    tot = {"block_jacobi": 0, "learned": 0}
    for seed in (0, 1):
        r = learned.compare(synth.bundle_adjustment(50, 7800, 32000, seed=seed), w, params)
        for k in tot:
            assert r[k]["fallbacks"] == 0, r
            tot[k] += r[k]["pcg_iterations"] / r[k]["solves"]
    assert tot["learned"] < tot["block_jacobi"], tot
