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


def rot3_smoothing(initial_values: np.ndarray, num_keys: int = 10) -> A.ProblemArrays:
    """"Test Rotation smoothing" (test/symforce_optimizer_test.cc:183-261): Rot3 priors at the first
    (identity, sigma 0.1 rad) and last key (yaw pi, sigma 0.1 rad), identity between factors
    (sigma 0.5 rad) in a chain, factor epsilon 1e-15; generated PRIOR_ROT3 / BETWEEN_ROT3 kinds."""
    eps = 1e-15
    prior_start = [0.0, 0.0, 0.0, 1.0]
    prior_last = list(ypr_quaternion(math.pi, 0, 0))
    prior_consts = [prior_start + [1 / 0.1] * 3 + [eps], prior_last + [1 / 0.1] * 3 + [eps]]
    between_consts = [[0.0, 0.0, 0.0, 1.0] + [1 / 0.5] * 3 + [eps] for _ in range(num_keys - 1)]
    return A.ProblemArrays(
        key_types=[A.SFG_KEY_ROT3] * num_keys,
        batches=[A.Batch(A.SFG_FACTOR_PRIOR_ROT3, [[0], [num_keys - 1]], prior_consts),
                 A.Batch(A.SFG_FACTOR_BETWEEN_ROT3, [[i, i + 1] for i in range(num_keys - 1)], between_consts)],
        values=initial_values,
        name="rot3_smoothing",
    )


ROT3_SMOOTHING_PARAMS = dict(iterations=50, early_exit_min_reduction=0.0001)
ROT3_SMOOTHING_EXPECTED = dict(last_iteration=6, lambda_approx=(2.4e-4, 1e-1), error_approx=(2.174, 1e-3))


def linear_problem(J: np.ndarray) -> A.ProblemArrays:
    """"Converges for a linear problem in one iteration" (test/symforce_levenberg_marquardt_test.cc:
    17-88): r = J x for a random 9 x 5 J, x initialised to 100 * ones."""
    return A.ProblemArrays(
        key_types=[A.SFG_KEY_VEC5],
        batches=[A.Batch(A.SFG_FACTOR_LINEAR_VEC5, [[0]], [np.concatenate([J.ravel(), np.zeros(9)])])],
        values=np.full(5, 100.0),
        name="linear_problem",
    )


def linear_problem_params() -> A.OptimizerParams:
    """The test's optimizer_params_t{} (value-initialised) with the fields it sets: one iteration of
    undamped Gauss-Newton (no diagonal or unit damping), STATIC lambda."""
    p = A.default_optimizer_params()
    for f, _ in A.OptimizerParams._fields_:
        setattr(p, f, 0)
    p.debug_stats = 1
    p.initial_lambda = 1.0
    p.lambda_update_type = A.SFG_LAMBDA_UPDATE_STATIC
    p.lambda_up_factor = 3.0
    p.lambda_down_factor = 1.0 / 3.0
    p.lambda_lower_bound = 0.0
    p.lambda_upper_bound = 0.0
    p.iterations = 1
    p.use_diagonal_damping = 0
    p.use_unit_damping = 0
    return p


LINEAR_PROBLEM_EPSILON = 1e-10


def gnc_problem(y: np.ndarray) -> A.ProblemArrays:
    """"Test GNC" (test/symforce_gnc_test.cc:22-76): x in R^5 (initialised to ones) pulled towards 20
    samples y_i by Barron-whitened factors whose convexity parameter mu is a constant of the
    generated BARRON_VEC5 kind (constant 5); factor epsilon kDefaultEpsilon."""
    n = y.shape[0]
    eps = A.DEFAULT_EPSILON
    consts = np.concatenate([y, np.zeros((n, 1)), np.full((n, 1), eps)], axis=1)
    return A.ProblemArrays(
        key_types=[A.SFG_KEY_VEC5],
        batches=[A.Batch(A.SFG_FACTOR_BARRON_VEC5, [[0]] * n, consts)],
        values=np.ones(5),
        name="gnc",
    )


def gnc_samples(draws: np.ndarray, n_outliers: int = 3) -> np.ndarray:
    """y_i = 10 + 0.1 r_i for the first n_outliers samples, 0.1 r_i after (symforce_gnc_test.cc:34-42)."""
    y = 0.1 * draws
    y[:n_outliers] += 10.0
    return y


GNC_OPTIMIZER_EPSILON = 1e-12
GNC_MU_SLOTS = [(0, 5)]
GNC_EXPECTED = dict(num_records=9)


def gnc_params():
    from symforce_gb300.gnc import GncParams
    return GncParams(gnc_update_min_reduction=1e-3, mu_initial=0.0, mu_step=0.33, mu_max=0.99)


def linearizer_problem(factor_order: str, key_order: str) -> A.ProblemArrays:
    """test/symforce_linearizer_test.cc:16-127: two linear factors J1 = diag(1, 2) and J2 = diag(3, 4)
    on scalar keys x = 10, y = -20, in either factor order and either key order (the reference's
    dense and sparse factors have the same math; both are the LINEAR_SCALAR2 kind here)."""
    J1 = [1.0, 0.0, 0.0, 2.0]
    J2 = [3.0, 0.0, 0.0, 4.0]
    xy = {"x": 10.0, "y": -20.0}
    order = list(key_order)  # e.g. "xy" or "yx"
    idx = {k: i for i, k in enumerate(order)}
    factors = [J1, J2] if factor_order == "dense_sparse" else [J2, J1]
    keys = [[idx["x"], idx["y"]]] * 2
    consts = [J + [0.0, 0.0] for J in factors]
    return A.ProblemArrays(
        key_types=[A.SFG_KEY_VEC1, A.SFG_KEY_VEC1],
        batches=[A.Batch(A.SFG_FACTOR_LINEAR_SCALAR2, keys, consts)],
        values=np.array([xy[k] for k in order]),
        name="linearizer",
    )
