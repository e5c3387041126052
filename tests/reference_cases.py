"""Problems taken from the reference's own tests and examples, with their known answers.

- robot_2d_localization: symforce/examples/robot_2d_localization/run_localization.cc:27-97
  (asserted by test/symforce_examples_robot_2d_localization_test.cc and
  test/symforce_examples_robot_2d_localization_test.py:48-50)
- pose smoothing: test/symforce_optimizer_test.cc:80-176
"""

from __future__ import annotations

import math

import numpy as np

from symforce_gb300 import _cabi as A


def robot_2d_localization() -> A.ProblemArrays:
    num_poses, num_landmarks = 3, 3
    landmarks = [(-2.0, 2.0), (1.0, -3.0), (5.0, 2.0)]
    distances = [1.7, 1.4]
    angles = [[55, 245, -35], [95, 220, -20], [125, 220, -20]]
    eps = A.DEFAULT_EPSILON
    bearing_keys, bearing_consts = [], []
    for i in range(num_poses):
        for j in range(num_landmarks):
            bearing_keys.append([i])
            bearing_consts.append([landmarks[j][0], landmarks[j][1], angles[i][j] * math.pi / 180, eps, 1.0])
    odo_keys = [[i, i + 1] for i in range(num_poses - 1)]
    odo_consts = [[distances[i], eps, 1.0] for i in range(num_poses - 1)]
    values = np.tile([1.0, 0.0, 0.0, 0.0], num_poses)
    return A.ProblemArrays(
        key_types=[A.SFG_KEY_POSE2] * num_poses,
        batches=[A.Batch(A.SFG_FACTOR_BEARING_POSE2, bearing_keys, bearing_consts),
                 A.Batch(A.SFG_FACTOR_ODOMETRY_POSE2, odo_keys, odo_consts)],
        values=values,
        name="robot_2d_localization",
    )


ROBOT_2D_EXPECTED = dict(
    num_iterations=9,
    first_error_range=(6.39635, 6.39637),
    first_error_python=6.396357319110695,
    best_error_below=0.00022003,
    poses=np.array([[0.477063, 0.878869, -0.583038, -0.824491],
                    [0.65425, 0.756279, 1.01671, -0.238356],
                    [0.779849, 0.625967, 1.79785, 0.920551]]),
)


def ypr_quaternion(yaw: float, pitch: float, roll: float) -> np.ndarray:
    """Rot3::FromYawPitchRoll as a [x, y, z, w] quaternion (z-y-x intrinsic order)."""
    cy, sy = math.cos(yaw / 2), math.sin(yaw / 2)
    cp, sp = math.cos(pitch / 2), math.sin(pitch / 2)
    cr, sr = math.cos(roll / 2), math.sin(roll / 2)
    return np.array([
        sr * cp * cy - cr * sp * sy,
        cr * sp * cy + sr * cp * sy,
        cr * cp * sy - sr * sp * cy,
        cr * cp * cy + sr * sp * sy,
    ])


def pose_smoothing(initial_values: np.ndarray, num_keys: int = 10) -> A.ProblemArrays:
    eps = 1e-10
    prior_start = np.array([0, 0, 0, 1, 0, 0, 0], dtype=float)
    prior_last = np.concatenate([ypr_quaternion(math.pi, 0, 0), [5.0, 0.0, 0.0]])
    prior_sqrt_info = [1 / 0.1] * 6
    between_sqrt_info = [1 / 0.5] * 6
    prior_keys = [[0], [num_keys - 1]]
    prior_consts = [list(prior_start) + prior_sqrt_info + [eps], list(prior_last) + prior_sqrt_info + [eps]]
    identity = [0, 0, 0, 1, 0, 0, 0]
    between_keys = [[i, i + 1] for i in range(num_keys - 1)]
    between_consts = [identity + between_sqrt_info + [eps] for _ in range(num_keys - 1)]
    return A.ProblemArrays(
        key_types=[A.SFG_KEY_POSE3] * num_keys,
        batches=[A.Batch(A.SFG_FACTOR_PRIOR_POSE3, prior_keys, prior_consts),
                 A.Batch(A.SFG_FACTOR_BETWEEN_POSE3, between_keys, between_consts)],
        values=initial_values,
        name="pose_smoothing",
    )


POSE_SMOOTHING_PARAMS = dict(iterations=50, early_exit_min_reduction=0.0001)
POSE_SMOOTHING_EXPECTED = dict(last_iteration=12, lambda_approx=(0.0039, 1e-1), error_approx=(7.801, 1e-3))

# "Test dynamic lambda update" and "The best linearization can be filled out without debug_stats"
# (test/symforce_optimizer_test.cc:461-506): DefaultOptimizerParams with DYNAMIC lambda updates on the
# pose-smoothing problem; SUCCESS with failure reason INVALID after 27 records, and the best
# linearization has 66 residual rows, a 60 x 60 lower Hessian with 534 stored entries and 60 rhs rows.
DYNAMIC_LAMBDA_EXPECTED = dict(num_records=27, residual_rows=66, hessian_dim=60, hessian_nnz=534,
                               rhs_rows=60)
