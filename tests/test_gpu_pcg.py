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


@pytest.mark.parametrize("kaporin", [0.0, 0.5])
def test_network_gradient_matches_oracle(kaporin):
    samples = PC.oracle_samples((3, 5)).astype(np.float32)
    w = PC.random_weights(4, out_scale=0.1)
    loss, grad = learned.loss_grad(samples, w, kaporin=kaporin)
    ref_loss, ref_grad = PN.loss_grad(w.astype(np.float64), samples.astype(np.float64), kaporin)
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
    """The learned-preconditioner forms on the 50-camera workload: both reach the oracle's cost.  In
    FP64 every PCG solve meets 1e-8 and the exact LDL^T, as judge of one step, agrees with it.  In
    the mixed form the FP32 inner iterations miss 1e-8 within the cap on part of the (ill-conditioned,
    lambda -> 1e-5) late systems; those solves fall back to the exact factorization, which is the
    designed safety net, and the fallback count is what the benchmark reports."""
    wl = workloads.get("ba_50_7800")
    p = wl.problem()
    ref = json.loads((ROOT / "tests" / "golden" / "oracle_costs.json").read_text())["ba_50_7800"]["best_error"]
    for precision in (A.SFG_PRECISION_FP64, A.SFG_PRECISION_MIXED):
        # the oracle stops on the reference's early-exit rule (relative reduction < 1e-6); the mixed
        # form's LM path differs, and by the same rule it can stop up to ~1e-6 above the oracle's
        # cost, so it runs on (relative reduction < 1e-9, as the benchmark does for every form but
        # the plain one)
        params = wl.params()
        if precision == A.SFG_PRECISION_MIXED:
            params.early_exit_min_reduction = 1e-9
        opt = Optimizer(p, params, A.default_form_params(precision=precision,
                                                        linear_solver=A.SFG_LINEAR_SOLVER_PCG_LEARNED))
        _, stats = opt.optimize(p.values)
        best = min(r.best_error for r in stats.iterations)
        # "reaches the oracle's cost": at or below it within 1e-6 (below is possible: the oracle
        # stopped on its early-exit rule); a different minimum would be far off
        assert best <= ref * (1 + 1e-6), (precision, best, ref)
        assert best >= ref * (1 - 1e-5), (precision, best, ref)
        ps = opt.pcg_stats()
        assert ps["solves"] == len(stats.iterations) - 1, ps
        if precision == A.SFG_PRECISION_FP64:
            assert ps["fallbacks"] == 0, ps
            # the judge: at the last accepted state the exact LDL^T's step and the PCG step agree to
            # what the residual allows (|e| / |y| <= cond(S) |r| / |v|; cond(S) ~ 1e9-1e11 at the
            # converged lambda, so 1e-8 in the residual leaves ~1e-2 in the step)
            judge = opt.pcg_step_error()
            assert judge["rel_residual"] <= 1e-8, judge
            assert judge["rel_step_error"] <= 5e-2, judge
        else:
            assert ps["fallbacks"] < ps["solves"], ps


@pytest.mark.parametrize("precision", [A.SFG_PRECISION_FP64, A.SFG_PRECISION_MIXED])
def test_multi_cta_pcg_reaches_plain_cost(precision):
    """300 camera blocks (100 warps): the PCG solve runs as a cooperative multi-CTA launch with grid
    barriers and grid reductions.  It reaches the plain FP64 form's cost (itself pinned to the
    oracle by the optimizer tests)."""
    p = synth.bundle_adjustment(num_cameras=300, num_points=6000, num_observations=30000, seed=11)
    params = A.default_optimizer_params(lambda_update_type=A.SFG_LAMBDA_UPDATE_DYNAMIC, iterations=30,
                                        early_exit_min_reduction=1e-9)
    plain = Optimizer(p, params, A.default_form_params(linear_solver=A.SFG_LINEAR_SOLVER_SCHUR))
    _, plain_stats = plain.optimize(p.values)
    ref = min(r.best_error for r in plain_stats.iterations)
    opt = Optimizer(p, params, A.default_form_params(precision=precision,
                                                    linear_solver=A.SFG_LINEAR_SOLVER_PCG_BLOCK_JACOBI))
    _, stats = opt.optimize(p.values)
    best = min(r.best_error for r in stats.iterations)
    assert abs(best - ref) <= 1e-6 * ref, (best, ref)
    ps = opt.pcg_stats()
    assert ps["solves"] == len(stats.iterations) - 1, ps
    if precision == A.SFG_PRECISION_FP64:
        assert ps["fallbacks"] == 0 and ps["max_rel_residual"] <= 1e-8, ps
    else:
        assert ps["fallbacks"] < ps["solves"], ps


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


def test_trained_network_against_block_jacobi():
    """What the trained network gains over the method without it (block Jacobi, which is the
    network with zero outputs), on held-out problems (seeds outside the training set), FP64 PCG so
    that only the preconditioner differs: fewer PCG iterations in total and no more fallbacks.

    The gain is small by construction: block Jacobi minimizes Kaporin's condition number
    (tr(K)/n) / det(K)^(1/n) of K = P^1/2 S P^1/2 over all block-diagonal preconditioners, a bound
    on the CG iteration count, and the network is trained with that condition number as a penalty
    (include/sfgpu.h, learned preconditioner).  Trained on the regression term alone, the same
    network needs 15-35 % more iterations than block Jacobi on these problems."""
    w = learned.load_weights()
    params = A.default_optimizer_params(lambda_update_type=A.SFG_LAMBDA_UPDATE_DYNAMIC, iterations=100)
    tot = {"block_jacobi": [0, 0], "learned": [0, 0]}
    for seed in (0, 1):
        r = learned.compare(synth.bundle_adjustment(50, 7800, 32000, seed=seed), w, params,
                            precision=A.SFG_PRECISION_FP64)
        for k in tot:
            assert r[k]["solves"] == r[k]["lm_iterations"], r
            tot[k][0] += r[k]["pcg_iterations"]
            tot[k][1] += r[k]["fallbacks"]
    assert tot["learned"][0] < tot["block_jacobi"][0], tot
    assert tot["learned"][1] <= tot["block_jacobi"][1], tot


@pytest.mark.parametrize("precision", [A.SFG_PRECISION_FP64, A.SFG_PRECISION_MIXED])
def test_gauge_coarse_correction_cuts_iterations(precision):
    """The coarse correction on the camera poses' similarity gauge (pcg_coarse) against the camera
    blocks alone, block Jacobi, multi-CTA launch: the same cost, and fewer PCG iterations in total
    (the 7 gauge directions are the near-null space of a bundle-adjustment reduced system; damping
    lifts them only as far as lambda does)."""
    p = synth.bundle_adjustment(num_cameras=300, num_points=6000, num_observations=30000, seed=11)
    params = A.default_optimizer_params(lambda_update_type=A.SFG_LAMBDA_UPDATE_DYNAMIC, iterations=30,
                                        early_exit_min_reduction=1e-9)
    out = {}
    for coarse in (0, 1):
        opt = Optimizer(p, params, A.default_form_params(precision=precision, pcg_coarse=coarse,
                                                        linear_solver=A.SFG_LINEAR_SOLVER_PCG_BLOCK_JACOBI))
        _, stats = opt.optimize(p.values)
        out[coarse] = (min(r.best_error for r in stats.iterations), opt.pcg_stats())
        opt.close()
    (best0, ps0), (best1, ps1) = out[0], out[1]
    assert abs(best1 - best0) <= 1e-6 * best0, (best0, best1)
    assert ps1["fallbacks"] <= ps0["fallbacks"], (ps0, ps1)
    assert ps1["iterations"] < ps0["iterations"], (ps0, ps1)


@pytest.mark.parametrize("band", [2, 5])
@pytest.mark.parametrize("solver", [A.SFG_LINEAR_SOLVER_PCG_BLOCK_JACOBI, A.SFG_LINEAR_SOLVER_PCG_LEARNED])
def test_band_preconditioner_iterations_match_oracle(band, solver):
    """One FP64 PCG solve with the band preconditioner (one CTA, 16 cameras): the same iteration
    count, within 2, as the oracle's float64 PCG with its M = G^T Lambda G on the same reduced
    system (the first LM iteration: initial values, lambda = 1), for Lambda = I and for the
    network's blocks (small random weights, every layer active)."""
    p = synth.bundle_adjustment(num_cameras=16, num_points=800, num_observations=4800, seed=4)
    params = A.default_optimizer_params(lambda_update_type=A.SFG_LAMBDA_UPDATE_DYNAMIC, iterations=1)
    w = PC.random_weights(7, out_scale=0.05) if solver == A.SFG_LINEAR_SOLVER_PCG_LEARNED else None
    opt = Optimizer(p, params, A.default_form_params(linear_solver=solver, pcg_band=band), weights=w)
    opt.optimize(p.values, num_iterations=1)
    ps = opt.pcg_stats()
    S, v = PC.reduced_system(p)
    gidx, degree = PC.camera_blocks(p)
    z = None
    if w is not None:
        z = PN.forward(w.astype(np.float64), PN.block_features(S, gidx, degree)[0])
    _, it, _ = PN.pcg_dense(S, v, PN.band_preconditioner(S, gidx, band, z), tol=0.5e-8)
    _, it0, _ = PN.pcg_dense(S, v, PN.band_preconditioner(S, gidx, 0, z), tol=0.5e-8)
    assert ps["solves"] == 1 and ps["fallbacks"] == 0, ps
    assert abs(ps["iterations"] - it) <= 2, (ps, it, it0)
    assert it < it0, (it, it0)


@pytest.mark.parametrize("precision", [A.SFG_PRECISION_FP64, A.SFG_PRECISION_MIXED])
def test_band_preconditioner_multi_cta_reaches_plain_cost(precision):
    """300 cameras (a cooperative multi-CTA launch whose rows of M read the other CTAs' residuals):
    block Jacobi and the band preconditioner over 4 neighbouring camera blocks reach the plain FP64
    form's cost, and the band needs fewer PCG iterations in total."""
    p = synth.bundle_adjustment(num_cameras=300, num_points=6000, num_observations=30000, seed=11)
    params = A.default_optimizer_params(lambda_update_type=A.SFG_LAMBDA_UPDATE_DYNAMIC, iterations=30,
                                        early_exit_min_reduction=1e-9)
    plain = Optimizer(p, params, A.default_form_params(linear_solver=A.SFG_LINEAR_SOLVER_SCHUR))
    _, plain_stats = plain.optimize(p.values)
    ref = min(r.best_error for r in plain_stats.iterations)
    its = {}
    for band in (0, 4):
        opt = Optimizer(p, params, A.default_form_params(precision=precision, pcg_band=band,
                                                        linear_solver=A.SFG_LINEAR_SOLVER_PCG_BLOCK_JACOBI))
        _, stats = opt.optimize(p.values)
        best = min(r.best_error for r in stats.iterations)
        assert abs(best - ref) <= 1e-6 * ref, (band, best, ref)
        ps = opt.pcg_stats()
        assert ps["solves"] == len(stats.iterations) - 1, ps
        if precision == A.SFG_PRECISION_FP64:
            assert ps["fallbacks"] == 0 and ps["max_rel_residual"] <= 1e-8, ps
        its[band] = ps["iterations"] / ps["solves"]
    assert its[4] < 0.85 * its[0], its


def test_band_option_rejects_bad_values():
    p = PC.small_ba(3)
    params = A.default_optimizer_params()
    for bad in (dict(pcg_band=-1), dict(pcg_band=7), dict(pcg_band=2, pcg_coarse=1)):
        with pytest.raises(RuntimeError):
            Optimizer(p, params, A.default_form_params(linear_solver=A.SFG_LINEAR_SOLVER_PCG_BLOCK_JACOBI, **bad))
