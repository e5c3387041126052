"""The compiled cc_sym-shaped binding (symforce_gb300.cc_sym, CPython C API over the C ABI) on the
GPU: the reference's robot_2d known answers, in-place values, record parity with the oracle on a
small bundle adjustment, and linearize against the oracle's linearization."""

from __future__ import annotations

import numpy as np
import pytest

import oracle_lib as O
import reference_cases as R
from symforce_gb300 import _cabi as A
from symforce_gb300 import synth

pytestmark = pytest.mark.gpu


def test_cc_sym_robot_2d_known_answers():
    from symforce_gb300 import cc_sym
    p = R.robot_2d_localization()
    opt = cc_sym.Optimizer(cc_sym.default_optimizer_params(), p)
    values = p.values.copy()
    stats = opt.optimize(values, populate_best_linearization=True)
    E = R.ROBOT_2D_EXPECTED
    assert len(stats.iterations) == E["num_iterations"]
    assert stats.iterations[0].new_error == pytest.approx(E["first_error_python"], rel=1e-14)
    assert stats.iterations[stats.best_index].new_error < E["best_error_below"]
    assert stats.status == A.SFG_STATUS_SUCCESS
    np.testing.assert_allclose(values.reshape(-1, 4), E["poses"], atol=1e-6)  # updated in place
    bl = stats.best_linearization
    assert bl.error == pytest.approx(stats.iterations[stats.best_index].new_error, rel=1e-12)
    assert opt.keys() == [0, 1, 2]


def test_cc_sym_matches_oracle_records_ba_small():
    from symforce_gb300 import cc_sym
    p = synth.bundle_adjustment(num_cameras=8, num_points=150, num_observations=600, seed=2)
    params = dict(cc_sym.default_optimizer_params(), lambda_update_type=A.SFG_LAMBDA_UPDATE_DYNAMIC,
                  iterations=20)
    opt = cc_sym.Optimizer(params, p)
    values = p.values.copy()
    stats = opt.optimize(values)
    ref = O.optimize(p, A.default_optimizer_params(lambda_update_type=A.SFG_LAMBDA_UPDATE_DYNAMIC, iterations=20))
    assert len(stats.iterations) == len(ref["iterations"])
    for g, o in zip(stats.iterations, ref["iterations"]):
        assert bool(g.update_accepted) == bool(o.update_accepted)
        assert g.new_error == pytest.approx(o.new_error, rel=1e-9)
    lin = opt.linearize(values)
    o = O.linearize(p, values)
    np.testing.assert_allclose(np.asarray(lin.residual), o["residual"], rtol=1e-12, atol=1e-12)
    np.testing.assert_array_equal(np.asarray(lin.hessian_col_ptr), o["colptr"])
    np.testing.assert_allclose(np.asarray(lin.hessian_values), o["hvals"], rtol=1e-9,
                               atol=1e-12 * np.abs(o["hvals"]).max())
    # the module-level one-call wrapper
    v2 = p.values.copy()
    s2 = cc_sym.optimize(params, p, v2)
    assert s2.iterations[s2.best_index].new_error == pytest.approx(stats.iterations[stats.best_index].new_error,
                                                                   rel=1e-12)
