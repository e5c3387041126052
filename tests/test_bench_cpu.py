"""Host-side helpers of bench.py (no GPU): the gauge-aligned per-state comparison of two bundle-
adjustment solutions vanishes for solutions that differ by a similarity transform of the world,
and sees a real change."""

from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

sys.path.insert(0, str(Path(__file__).resolve().parents[1]))

import bench  # noqa: E402
from symforce_gb300 import synth  # noqa: E402


def _quat_mul(p, q):
    return synth.quat_mul(p, q)


def _similarity(problem, x, rotvec, scale, t):
    """World transform x_w -> scale R x_w + t applied to a solution: points move, camera poses
    (cam_T_world) absorb the inverse, so every projection (and the cost) is unchanged."""
    nc = int(problem.meta["num_cameras"])
    q = synth.quat_exp(np.asarray(rotvec, dtype=float)[None, :])[0]
    R = bench._quat_to_rot(q[None, :])[0]
    y = x.copy()
    pts = x[10 * nc:].reshape(-1, 3)
    y[10 * nc:] = (scale * pts @ R.T + t).reshape(-1)
    cam = x[:7 * nc].reshape(nc, 7)
    q_inv = q * np.array([-1.0, -1.0, -1.0, 1.0])
    for k in range(nc):
        qk = _quat_mul(cam[k:k + 1, :4], q_inv[None, :])[0]          # R_c R^T
        Rk = bench._quat_to_rot(qk[None, :])[0]
        y[7 * k:7 * k + 4] = qk
        y[7 * k + 4:7 * k + 7] = scale * cam[k, 4:] - Rk @ t
    return y


def test_state_errors_are_gauge_invariant():
    p = synth.bundle_adjustment(num_cameras=12, num_points=400, num_observations=1600, seed=2)
    x = p.values
    y = _similarity(p, x, [0.2, -0.1, 0.3], 1.7, np.array([0.5, -2.0, 3.0]))
    e = bench._state_errors(p, y, x)
    assert e["rotation_rad"] < 1e-12 and e["camera_centre_m"] < 1e-9 and e["point_m"] < 1e-9, e
    assert abs(e["gauge_scale"] * 1.7 - 1.0) < 1e-12
    # a real change is seen
    z = x.copy()
    z[-3:] += np.array([0.1, 0.0, 0.0])
    assert abs(bench._state_errors(p, z, x)["point_m"] - 0.1) < 1e-3
