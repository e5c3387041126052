"""Graduated non-convexity: the schedule of sym::GncOptimizer (symforce/opt/gnc_optimizer.h:22-110).

The cost's convexity is controlled by a parameter mu (0: convex, towards 1: robust).  The optimizer
first iterates to convergence at mu_initial with the looser early-exit threshold
gnc_update_min_reduction, then repeatedly steps mu by mu_step (capped at mu_max), relaxes the
damping to its initial value and continues the same Levenberg-Marquardt run (ResetState: lambda, nu
and the iteration counter carry over; the records accumulate) until the iteration budget is spent,
a stage does not end in SUCCESS, or mu has reached mu_max and that last stage converged with the
user's own early-exit threshold.

`run_gnc` is the schedule over two callbacks, so that the GPU optimizer and the CPU oracle run the
same schedule; `GncOptimizer` (symforce_gb300.optimizer) binds it to the device loop.
"""

from __future__ import annotations

from dataclasses import dataclass
from typing import Callable, List, Tuple

from . import _cabi as A


@dataclass
class GncParams:
    """optimizer_gnc_params_t (lcmtypes/symforce.lcm:203-226)."""

    gnc_update_min_reduction: float = 1e-3
    mu_initial: float = 0.0
    mu_step: float = 0.33
    mu_max: float = 0.99


# optimize(params, num_iterations, continue_state, relax_damping) -> (records, best_index, status,
# failure_reason); best_index is -1 in a continued run whose records did not improve on its start.
OptimizeFn = Callable[[A.OptimizerParams, int, bool, bool], Tuple[list, int, int, int]]


def _copy_params(p: A.OptimizerParams) -> A.OptimizerParams:
    q = A.default_optimizer_params()
    for f, _ in A.OptimizerParams._fields_:
        setattr(q, f, getattr(p, f))
    return q


def run_gnc(params: A.OptimizerParams, gnc: GncParams, set_mu: Callable[[float], None],
            optimize: OptimizeFn, num_iterations: int = -1) -> dict:
    """GncOptimizer::Optimize (symforce/opt/gnc_optimizer.h:45-110).  Returns the accumulated
    records, best_index, status, failure_reason and the final mu."""
    if num_iterations < 0:
        num_iterations = params.iterations
    updating = gnc.mu_initial < gnc.mu_max and gnc.mu_step > 0.0
    mu = gnc.mu_initial
    set_mu(mu)
    p = _copy_params(params)
    early_exit = params.early_exit_min_reduction
    if updating:
        p.early_exit_min_reduction = gnc.gnc_update_min_reduction
    records: List = []
    recs, best, status, reason = optimize(p, num_iterations, False, False)
    records += recs
    best_index = best
    while len(records) < num_iterations:
        if status != A.SFG_STATUS_SUCCESS or not updating:
            break
        mu += gnc.mu_step
        relax = True
        if mu >= gnc.mu_max:
            mu = gnc.mu_max
            p.early_exit_min_reduction = early_exit
            updating = False
        set_mu(mu)
        recs, best, status, reason = optimize(p, num_iterations - len(records), True, relax)
        if best >= 0:
            best_index = len(records) + best
        records += recs
    return dict(iterations=records, best_index=best_index, status=status, failure_reason=reason, mu=mu)
