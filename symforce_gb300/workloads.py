"""Named benchmark workloads: the synthetic problem, optimizer parameters and solver form."""

from __future__ import annotations

from dataclasses import dataclass

from . import _cabi as A
from . import synth


@dataclass(frozen=True)
class Workload:
    name: str
    seed: int
    description: str

    def problem(self) -> A.ProblemArrays:
        return synth.config_problem(self.name, seed=self.seed)

    def params(self) -> A.OptimizerParams:
        if self.name.startswith("ba_"):
            # the reference's bundle-adjustment example uses DYNAMIC lambda updates
            # (symforce/examples/bundle_adjustment_in_the_large/bundle_adjustment_in_the_large.cc:131-133)
            # cap of 100 iterations: the optimizer stops at convergence (relative reduction < 1e-6),
            # which the FP64 oracle reaches after 58 on the 50-camera workload
            return A.default_optimizer_params(lambda_update_type=A.SFG_LAMBDA_UPDATE_DYNAMIC,
                                              iterations=100)
        return A.default_optimizer_params()

    def form(self, precision: int = A.SFG_PRECISION_FP64) -> A.FormParams:
        solver = A.SFG_LINEAR_SOLVER_SCHUR if self.name.startswith("ba_") else A.SFG_LINEAR_SOLVER_SPARSE_LDLT
        return A.default_form_params(precision=precision, linear_solver=solver)


_WORKLOADS = {
    "ba_50_7800": Workload("ba_50_7800", 0, "bundle adjustment, 50 cameras, 7,800 points, ~32k "
                           "observations, Cauchy loss, Schur over points, FP64"),
    "robot2d_1000": Workload("robot2d_1000", 0, "2D localization, 1,000 Pose2, odometry + bearing, "
                             "sparse LDL^T, FP64"),
    "ba_1000_200k": Workload("ba_1000_200k", 0, "bundle adjustment, 1,000 cameras, 200k points, "
                             "~1.2M observations"),
    "ba_10k_1m": Workload("ba_10k_1m", 0, "bundle adjustment, 10,000 cameras, 1M points, ~5M "
                          "observations (reduced camera system of 90k unknowns)"),
}


def get(name: str) -> Workload:
    return _WORKLOADS[name]
