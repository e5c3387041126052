"""Synthetic workload generators: determinism and the configured shapes."""

from __future__ import annotations

import numpy as np

from symforce_gb300 import _cabi as A
from symforce_gb300 import synth


def test_ba_generator_shapes_and_determinism():
    p1 = synth.bundle_adjustment(50, 7800, 32000, seed=0)
    p2 = synth.bundle_adjustment(50, 7800, 32000, seed=0)
    np.testing.assert_array_equal(p1.values, p2.values)
    np.testing.assert_array_equal(p1.batches[0].consts, p2.batches[0].consts)
    m = p1.meta
    assert m["num_cameras"] == 50 and m["num_points"] == 7800
    assert 30000 < m["num_observations"] < 34000
    keys = p1.batches[0].keys
    nviews = np.bincount(keys[:, 2] - 100, minlength=7800)
    assert nviews.min() >= 2 and nviews.max() <= 8
    assert p1.num_schur_keys == 7800
    assert p1.tangent_dim == 50 * 6 + 50 * 3 + 7800 * 3


def test_robot2d_generator():
    p = synth.robot_2d(1000, seed=0)
    assert p.tangent_dim == 3000
    assert p.residual_dim == 3000 + 999
    assert np.all(p.values.reshape(-1, 4) == [1, 0, 0, 0])
