"""GPU factor linearization against the reference's symbolic definitions (golden vectors) and
against the oracle, through the C ABI."""

from __future__ import annotations

import json
from pathlib import Path

import numpy as np
import pytest

from symforce_gb300 import _cabi as A
from symforce_gb300.optimizer import Optimizer

pytestmark = pytest.mark.gpu

GOLDEN = Path(__file__).resolve().parent / "golden"


def _vectors():
    return json.loads((GOLDEN / "factor_vectors.json").read_text())["vectors"]


@pytest.mark.parametrize("vec", _vectors(), ids=lambda v: f"kind{v['kind']}")
def test_gpu_factor_matches_symforce_symbolic(vec):
    kt = vec["key_types"]
    p = A.ProblemArrays(key_types=kt, batches=[A.Batch(vec["kind"], [list(range(len(kt)))], [vec["consts"]])],
                        values=np.array(vec["storage"]))
    lin = Optimizer(p).linearize(p.values)
    r = np.array(vec["residual"])
    J = np.array(vec["jacobian"])
    np.testing.assert_allclose(lin["residual"], r, rtol=1e-10, atol=1e-12)
    H = np.zeros((J.shape[1], J.shape[1]))
    for c in range(J.shape[1]):
        for q in range(lin["colptr"][c], lin["colptr"][c + 1]):
            H[lin["rowidx"][q], c] = lin["hvals"][q]
    JtJ = J.T @ J
    scale = max(1.0, np.abs(JtJ).max())
    np.testing.assert_allclose(np.tril(H), np.tril(JtJ), rtol=1e-7, atol=1e-9 * scale)
    np.testing.assert_allclose(lin["rhs"], J.T @ r, rtol=1e-7, atol=1e-9 * max(1.0, np.abs(J.T @ r).max()))
