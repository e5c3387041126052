"""Seeded synthetic problems with the shapes, sizes and value distributions of the benchmark
configurations (no datasets are available; every number here comes from numpy's PCG64 stream,
which is platform- and compiler-independent).

- robot_2d(num_poses=1000): 2D localization, Pose2 random walk, odometry distance + bearing factors.
- bundle_adjustment(num_cameras, num_points, num_observations): Snavely reprojection with Cauchy
  norm whitening, cameras on a ring looking inward, points in a 10 m cube, each point seen by
  2..8 angularly adjacent cameras (so the reduced camera system is banded).
- pose3_chains(num_problems): independent 3D localization problems (between + range factors).
"""

from __future__ import annotations

import math

import numpy as np

from . import _cabi as A


def _quat_from_rotmat(R: np.ndarray) -> np.ndarray:
    """[x, y, z, w] quaternion of a rotation matrix (w >= 0)."""
    tr = np.trace(R)
    if tr > 0:
        s = math.sqrt(tr + 1.0) * 2
        w = 0.25 * s
        x = (R[2, 1] - R[1, 2]) / s
        y = (R[0, 2] - R[2, 0]) / s
        z = (R[1, 0] - R[0, 1]) / s
    elif R[0, 0] > R[1, 1] and R[0, 0] > R[2, 2]:
        s = math.sqrt(1.0 + R[0, 0] - R[1, 1] - R[2, 2]) * 2
        w = (R[2, 1] - R[1, 2]) / s
        x = 0.25 * s
        y = (R[0, 1] + R[1, 0]) / s
        z = (R[0, 2] + R[2, 0]) / s
    elif R[1, 1] > R[2, 2]:
        s = math.sqrt(1.0 + R[1, 1] - R[0, 0] - R[2, 2]) * 2
        w = (R[0, 2] - R[2, 0]) / s
        x = (R[0, 1] + R[1, 0]) / s
        y = 0.25 * s
        z = (R[1, 2] + R[2, 1]) / s
    else:
        s = math.sqrt(1.0 + R[2, 2] - R[0, 0] - R[1, 1]) * 2
        w = (R[1, 0] - R[0, 1]) / s
        x = (R[0, 2] + R[2, 0]) / s
        y = (R[1, 2] + R[2, 1]) / s
        z = 0.25 * s
    q = np.array([x, y, z, w])
    if q[3] < 0:
        q = -q
    return q / np.linalg.norm(q)


def quat_rotate(q: np.ndarray, v: np.ndarray) -> np.ndarray:
    """Rotate vectors v [..., 3] by unit quaternions q [..., 4] ([x, y, z, w])."""
    x, y, z, w = q[..., 0], q[..., 1], q[..., 2], q[..., 3]
    R = np.stack([
        np.stack([1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y)], -1),
        np.stack([2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x)], -1),
        np.stack([2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y)], -1),
    ], -2)
    return np.einsum("...ij,...j->...i", R, v)


def quat_mul(p: np.ndarray, q: np.ndarray) -> np.ndarray:
    px, py, pz, pw = p[..., 0], p[..., 1], p[..., 2], p[..., 3]
    qx, qy, qz, qw = q[..., 0], q[..., 1], q[..., 2], q[..., 3]
    return np.stack([
        pw * qx + px * qw + py * qz - pz * qy,
        pw * qy - px * qz + py * qw + pz * qx,
        pw * qz + px * qy - py * qx + pz * qw,
        pw * qw - px * qx - py * qy - pz * qz,
    ], -1)


def quat_exp(w: np.ndarray) -> np.ndarray:
    th = np.linalg.norm(w, axis=-1, keepdims=True)
    s = np.where(th > 1e-12, np.sin(th / 2) / np.maximum(th, 1e-300), 0.5)
    return np.concatenate([w * s, np.cos(th / 2)], -1)


# ---------------------------------------------------------------------------------------------
# Config 0: 2D robot localization
# ---------------------------------------------------------------------------------------------
def robot_2d(num_poses: int = 1000, num_landmarks: int = 20, bearings_per_pose: int = 3,
             seed: int = 0) -> A.ProblemArrays:
    """1,000 Pose2 states, odometry distance factors (sigma 0.1 m) between consecutive poses,
    3 bearing factors per pose (sigma 0.05 rad) to landmarks ~U[-10, 10]^2; ground truth is a
    random walk with 1 m steps and N(0, 0.3) heading changes; poses start at identity."""
    rng = np.random.Generator(np.random.PCG64(seed))
    eps = A.DEFAULT_EPSILON
    landmarks = rng.uniform(-10, 10, size=(num_landmarks, 2))
    heading = np.cumsum(np.concatenate([[0.0], rng.normal(0, 0.3, size=num_poses - 1)]))
    steps = np.stack([np.cos(heading), np.sin(heading)], -1)
    pos = np.concatenate([[[0.0, 0.0]], np.cumsum(steps[1:], axis=0)], 0)
    # odometry: distance between consecutive poses + noise
    d = np.linalg.norm(pos[1:] - pos[:-1], axis=1) + rng.normal(0, 0.1, size=num_poses - 1)
    odo_keys = np.stack([np.arange(num_poses - 1), np.arange(1, num_poses)], -1)
    odo_consts = np.stack([d, np.full_like(d, eps), np.full_like(d, 1 / 0.1)], -1)
    # bearings
    lm_idx = rng.integers(0, num_landmarks, size=(num_poses, bearings_per_pose))
    rel = landmarks[lm_idx] - pos[:, None, :]
    c, s = np.cos(heading)[:, None], np.sin(heading)[:, None]
    bx = c * rel[..., 0] + s * rel[..., 1]
    by = -s * rel[..., 0] + c * rel[..., 1]
    ang = np.arctan2(by, bx) + rng.normal(0, 0.05, size=bx.shape)
    bkeys = np.repeat(np.arange(num_poses), bearings_per_pose)
    L = landmarks[lm_idx].reshape(-1, 2)
    bconsts = np.stack([L[:, 0], L[:, 1], ang.reshape(-1), np.full(L.shape[0], eps),
                        np.full(L.shape[0], 1 / 0.05)], -1)
    values = np.tile([1.0, 0.0, 0.0, 0.0], num_poses)
    return A.ProblemArrays(
        key_types=[A.SFG_KEY_POSE2] * num_poses,
        batches=[A.Batch(A.SFG_FACTOR_BEARING_POSE2, bkeys[:, None], bconsts),
                 A.Batch(A.SFG_FACTOR_ODOMETRY_POSE2, odo_keys, odo_consts)],
        values=values,
        name=f"robot_2d_{num_poses}",
        meta=dict(seed=seed, truth_xy=pos, truth_heading=heading),
    )


# ---------------------------------------------------------------------------------------------
# Config 3: batches of independent 3D localization problems
# ---------------------------------------------------------------------------------------------
def _pose3_draws(n: int, L: int, seed: int) -> dict:
    rng = np.random.Generator(np.random.PCG64(seed))
    d = dict(q0=rng.normal(size=4), t0=rng.uniform(-20, 20, size=3))
    d["rot_inc"] = rng.normal(0, 0.1, size=(n - 1, 3))
    d["jitter"] = rng.normal(0, 0.1, size=(n - 1, 3))
    d["landmarks"] = rng.uniform(-20, 20, size=(L, 3))
    d["n_rot"] = rng.normal(0, 0.05, size=(n - 1, 3))
    d["n_t"] = rng.normal(0, 0.1, size=(n - 1, 3))
    d["n_range"] = rng.normal(0, 0.1, size=(n, L))
    return d


def _pose3_build(sizes, lms, seeds) -> list:
    """The problems of pose3_chain for every (n, L, seed), with the sequential trajectory and dead
    reckoning recursions evaluated for all problems at once."""
    eps = A.DEFAULT_EPSILON
    P = len(sizes)
    nmax = int(max(sizes))
    draws = [_pose3_draws(int(sizes[i]), int(lms[i]), int(seeds[i])) for i in range(P)]
    pad = lambda key: np.stack([np.concatenate([d[key], np.zeros((nmax - 1 - d[key].shape[0], 3))], 0)
                                for d in draws], 0)
    rot_inc, jitter, n_rot, n_t = pad("rot_inc"), pad("jitter"), pad("n_rot"), pad("n_t")
    q = np.zeros((P, nmax, 4))
    t = np.zeros((P, nmax, 3))
    q0 = np.stack([d["q0"] for d in draws])
    q[:, 0] = q0 / np.linalg.norm(q0, axis=1, keepdims=True)
    t[:, 0] = np.stack([d["t0"] for d in draws])
    fwd = np.array([1.0, 0.0, 0.0])
    for k in range(1, nmax):
        q[:, k] = quat_mul(q[:, k - 1], quat_exp(rot_inc[:, k - 1]))
        t[:, k] = t[:, k - 1] + quat_rotate(q[:, k - 1], fwd) + jitter[:, k - 1]
    qa_inv = q[:, :-1] * np.array([-1, -1, -1, 1.0])
    q_meas = quat_mul(quat_mul(qa_inv, q[:, 1:]), quat_exp(n_rot))
    t_meas = quat_rotate(qa_inv, t[:, 1:] - t[:, :-1]) + n_t
    qi = np.zeros_like(q)
    ti = np.zeros_like(t)
    qi[:, 0], ti[:, 0] = q[:, 0], t[:, 0]
    for k in range(1, nmax):
        qi[:, k] = quat_mul(qi[:, k - 1], q_meas[:, k - 1])
        ti[:, k] = ti[:, k - 1] + quat_rotate(qi[:, k - 1], t_meas[:, k - 1])
    s_between = np.array([1 / 0.05] * 3 + [1 / 0.1] * 3)
    s_prior = np.array([1 / 0.1] * 3 + [1 / 1.0] * 3)
    out = []
    for i, d in enumerate(draws):
        n, L = int(sizes[i]), int(lms[i])
        bw_consts = np.concatenate([q_meas[i, :n - 1], t_meas[i, :n - 1], np.tile(s_between, (n - 1, 1)),
                                    np.full((n - 1, 1), eps)], 1)
        bw_keys = np.stack([np.arange(n - 1), np.arange(1, n)], -1)
        lm = d["landmarks"]
        rng_d = np.linalg.norm(t[i, :n, None, :] - lm[None, :, :], axis=-1) + d["n_range"]
        r_keys = np.repeat(np.arange(n), L)
        r_consts = np.concatenate([np.tile(lm, (n, 1)), rng_d.reshape(-1, 1), np.full((n * L, 1), 1 / 0.1),
                                   np.full((n * L, 1), eps)], 1)
        p_consts = np.concatenate([q[i, 0], t[i, 0], s_prior, [eps]])[None, :]
        values = np.concatenate([qi[i, :n], ti[i, :n]], 1).reshape(-1)
        out.append(A.ProblemArrays(
            key_types=[A.SFG_KEY_POSE3] * n,
            batches=[A.Batch(A.SFG_FACTOR_PRIOR_POSE3, np.zeros((1, 1)), p_consts),
                     A.Batch(A.SFG_FACTOR_BETWEEN_POSE3, bw_keys, bw_consts),
                     A.Batch(A.SFG_FACTOR_RANGE_POSE3, r_keys[:, None], r_consts)],
            values=values,
            name=f"pose3_chain_{n}_{L}",
            meta=dict(seed=int(seeds[i]), num_poses=n, num_landmarks=L),
        ))
    return out


def pose3_chain(num_poses: int, num_landmarks: int, seed: int) -> A.ProblemArrays:
    """One 3D localization problem: a Pose3 random walk (1 m forward steps in the body frame with
    N(0, 0.1) m jitter, N(0, 0.1) rad rotation increments) starting uniformly in a 40 m cube,
    between factors on consecutive poses (noise and sqrt_info diag(1/0.05 x3, 1/0.1 x3)), a range
    factor from every pose to every landmark (landmarks ~U in the 40 m cube, sigma 0.1 m), and a
    weak prior on the first pose (sigma 0.1 rad / 1 m) that fixes the global rotation, which ranges
    and relative poses leave unobservable.  Initial values are dead reckoning: the prior pose
    composed with the measured relative poses."""
    return _pose3_build([num_poses], [num_landmarks], [seed])[0]


def pose3_chains(num_problems: int = 4096, seed: int = 0, min_poses: int = 5, max_poses: int = 200,
                 min_landmarks: int = 10, max_landmarks: int = 50) -> list:
    """Independent 3D localization problems of uneven size: problem i has U{5..200} poses and
    U{10..50} landmarks drawn from the batch seed, and its own seed (seed * 1_000_003 + i);
    problem i equals pose3_chain(n_i, L_i, seed * 1_000_003 + i)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    sizes = rng.integers(min_poses, max_poses + 1, size=num_problems)
    lms = rng.integers(min_landmarks, max_landmarks + 1, size=num_problems)
    return _pose3_build(sizes, lms, [seed * 1_000_003 + i for i in range(num_problems)])


def loop_closed_pose3_chain(num_poses: int, num_landmarks: int, seed: int) -> A.ProblemArrays:
    """pose3_chain with one more between factor, from the last pose back to the first (a loop
    closure): no longer block tridiagonal."""
    p = pose3_chain(num_poses, num_landmarks, seed)
    bw = next(b for b in p.batches if b.kind == A.SFG_FACTOR_BETWEEN_POSE3)
    # the closure measures the dead-reckoned relative pose last -> first (zero residual at the
    # initial values), with the chain's noise model
    v = p.values.reshape(num_poses, 7)
    qa_inv = v[-1, :4] * np.array([-1, -1, -1, 1.0])
    c = bw.consts[:1].copy()
    c[0, :4] = quat_mul(qa_inv, v[0, :4])
    c[0, 4:7] = quat_rotate(qa_inv, v[0, 4:7] - v[-1, 4:7])
    loop = A.Batch(A.SFG_FACTOR_BETWEEN_POSE3, np.array([[num_poses - 1, 0]], dtype=np.int32), c)
    return A.ProblemArrays(key_types=p.key_types, batches=list(p.batches) + [loop], values=p.values,
                           name=f"loop_pose3_chain_{num_poses}_{num_landmarks}", meta=dict(p.meta))


def rot3_chain(num_keys: int, seed: int) -> A.ProblemArrays:
    """Rotation smoothing: a Rot3 random walk (N(0, 0.2) rad increments), a PRIOR_ROT3 on every key
    measured with N(0, 0.1) rad noise (sqrt_info 1/0.1) and a BETWEEN_ROT3 on consecutive keys
    measured with N(0, 0.05) rad noise (sqrt_info 1/0.05) (the generated factor kinds); every key
    starts at identity."""
    rng = np.random.Generator(np.random.PCG64(seed))
    eps = A.DEFAULT_EPSILON
    q = np.zeros((num_keys, 4))
    q[0] = quat_exp(rng.normal(0, 1.0, size=3))
    for k in range(1, num_keys):
        q[k] = quat_mul(q[k - 1], quat_exp(rng.normal(0, 0.2, size=3)))
    meas = quat_mul(q, quat_exp(rng.normal(0, 0.1, size=(num_keys, 3))))
    rel = quat_mul(quat_mul(q[:-1] * np.array([-1, -1, -1, 1.0]), q[1:]),
                   quat_exp(rng.normal(0, 0.05, size=(num_keys - 1, 3))))
    prior = np.concatenate([meas, np.full((num_keys, 3), 1 / 0.1), np.full((num_keys, 1), eps)], 1)
    between = np.concatenate([rel, np.full((num_keys - 1, 3), 1 / 0.05), np.full((num_keys - 1, 1), eps)], 1)
    values = np.tile([0.0, 0.0, 0.0, 1.0], num_keys)
    return A.ProblemArrays(
        key_types=[A.SFG_KEY_ROT3] * num_keys,
        batches=[A.Batch(A.SFG_FACTOR_PRIOR_ROT3, np.arange(num_keys)[:, None], prior),
                 A.Batch(A.SFG_FACTOR_BETWEEN_ROT3, np.stack([np.arange(num_keys - 1), np.arange(1, num_keys)], -1),
                         between)],
        values=values, name=f"rot3_chain_{num_keys}", meta=dict(seed=seed))


def mixed_small_problems(num_problems: int = 4096, seed: int = 0) -> list:
    """Independent small problems of uneven size and structure for the batched form's dense path
    (tangent dimension at most 120): in turn a 2D localization (U{5..40} Pose2 states, robot_2d), a
    loop-closed Pose3 chain of U{5..20} poses with U{4..12} range landmarks, and a Rot3 smoothing
    chain of U{5..40} keys; problem i has its own seed (seed * 1_000_003 + i)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    out = []
    for i in range(num_problems):
        s = seed * 1_000_003 + i
        k = i % 3
        if k == 0:
            out.append(robot_2d(num_poses=int(rng.integers(5, 41)), num_landmarks=6, seed=s))
        elif k == 1:
            out.append(loop_closed_pose3_chain(int(rng.integers(5, 21)), int(rng.integers(4, 13)), s))
        else:
            out.append(rot3_chain(int(rng.integers(5, 41)), s))
    return out


# ---------------------------------------------------------------------------------------------
# Configs 1/2/4: bundle adjustment
# ---------------------------------------------------------------------------------------------
def bundle_adjustment(num_cameras: int = 50, num_points: int = 7800,
                      num_observations: int = 32000, seed: int = 0, outlier_fraction: float = 0.02,
                      cauchy_delta: float = 1.0, pixel_sigma: float = 1.0,
                      ring_radius: float = 20.0, cube: float = 10.0,
                      max_views: int = 8) -> A.ProblemArrays:
    """Synthetic BA: cameras (Pose3 cam_T_world + intrinsics (f ~ U(400, 600), k1, k2 ~ N(0, 1e-3)))
    on a ring looking at a 10 m cube of points; each point is seen by n_j in 2..max_views angularly
    adjacent cameras, n_j = 2 + Binomial(max_views - 2, p) with p chosen so that the expected number
    of observations is num_observations.  Pixel noise N(0, 1); a fraction of observations are
    outliers with uniform pixel error in [-50, 50]; residuals are Cauchy-whitened (delta = 1 px).
    Initial values: rotations perturbed by N(0, 0.01) rad, translations by N(0, 0.1) m, points by
    N(0, 0.2) m; intrinsics start at their true values.  Key order: poses 'c', intrinsics 'i',
    points 'p' (lexical), so the points are the trailing Schur block."""
    rng = np.random.Generator(np.random.PCG64(seed))
    eps = A.DEFAULT_EPSILON
    nc, npt = num_cameras, num_points
    # cameras on a horizontal ring, -z axis toward the origin
    theta = 2 * np.pi * np.arange(nc) / nc
    centers = np.stack([ring_radius * np.cos(theta), ring_radius * np.sin(theta),
                        rng.uniform(-1.0, 1.0, size=nc)], -1)
    q_true = np.zeros((nc, 4))
    t_true = np.zeros((nc, 3))
    up = np.array([0.0, 0.0, 1.0])
    for k in range(nc):
        zc = centers[k] / np.linalg.norm(centers[k])
        xc = np.cross(up, zc)
        xc /= np.linalg.norm(xc)
        yc = np.cross(zc, xc)
        R_wc = np.stack([xc, yc, zc], -1)
        R_cw = R_wc.T
        q_true[k] = _quat_from_rotmat(R_cw)
        t_true[k] = -R_cw @ centers[k]
    intr = np.stack([rng.uniform(400, 600, size=nc), rng.normal(0, 1e-3, size=nc),
                     rng.normal(0, 1e-3, size=nc)], -1)
    points = rng.uniform(-cube / 2, cube / 2, size=(npt, 3))
    # views per point
    extra = max_views - 2
    p = np.clip((num_observations / npt - 2) / extra, 0.0, 1.0)
    nviews = 2 + rng.binomial(extra, p, size=npt)
    start = rng.integers(0, nc, size=npt)
    obs_pt = np.repeat(np.arange(npt), nviews)
    offs = np.concatenate([np.arange(n) for n in nviews]) if npt else np.zeros(0, int)
    obs_cam = (np.repeat(start, nviews) + offs) % nc
    # sort observations by camera, then point (a deterministic factor order)
    order = np.lexsort((obs_pt, obs_cam))
    obs_cam, obs_pt = obs_cam[order], obs_pt[order]
    nobs = obs_cam.size
    pc = quat_rotate(q_true[obs_cam], points[obs_pt]) + t_true[obs_cam]
    uv = pc[:, :2] / (-pc[:, 2:3])
    r2 = np.sum(uv * uv, axis=1, keepdims=True)
    f, k1, k2 = intr[obs_cam, 0:1], intr[obs_cam, 1:2], intr[obs_cam, 2:3]
    pix = f * (1 + k1 * r2 + k2 * r2 * r2) * uv
    pix = pix + rng.normal(0, pixel_sigma, size=pix.shape)
    outl = rng.uniform(size=nobs) < outlier_fraction
    pix[outl] += rng.uniform(-50, 50, size=(int(outl.sum()), 2))
    # initial values
    q0 = quat_mul(q_true, quat_exp(rng.normal(0, 0.01, size=(nc, 3))))
    t0 = t_true + rng.normal(0, 0.1, size=(nc, 3))
    p0 = points + rng.normal(0, 0.2, size=(npt, 3))
    key_types = [A.SFG_KEY_POSE3] * nc + [A.SFG_KEY_VEC3] * nc + [A.SFG_KEY_VEC3] * npt
    values = np.concatenate([np.concatenate([q0, t0], 1).reshape(-1), intr.reshape(-1),
                             p0.reshape(-1)])
    keys = np.stack([obs_cam, nc + obs_cam, 2 * nc + obs_pt], -1)
    consts = np.stack([pix[:, 0], pix[:, 1], np.full(nobs, eps), np.full(nobs, cauchy_delta)], -1)
    return A.ProblemArrays(
        key_types=key_types,
        batches=[A.Batch(A.SFG_FACTOR_SNAVELY_REPROJECTION, keys, consts)],
        values=values,
        num_schur_keys=npt,
        name=f"ba_{nc}_{npt}_{nobs}",
        meta=dict(seed=seed, num_cameras=nc, num_points=npt, num_observations=nobs,
                  outliers=int(outl.sum())),
    )


def config_problem(name: str, seed: int = 0) -> A.ProblemArrays:
    """The benchmark configurations by name."""
    if name == "robot2d_1000":
        return robot_2d(1000, seed=seed)
    if name == "ba_50_7800":
        return bundle_adjustment(50, 7800, 32000, seed=seed)
    if name == "ba_1000_200k":
        return bundle_adjustment(1000, 200000, 1200000, seed=seed)
    if name == "ba_10k_1m":
        return bundle_adjustment(10000, 1000000, 5000000, seed=seed)
    raise KeyError(name)
