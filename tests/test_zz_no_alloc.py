"""The allocation-free dense solve (sfg_dense_ldlt_solve_noalloc) through the C ABI.

Callers that cannot allocate device memory (a host application that owns every allocation, or code
under an allocator that forbids cudaMalloc) hand it device pointers only; it keeps its working
memory in fixed file-scope device arrays.  This checks it against the allocating entry points
(sfg_ldlt_create / _factorize / _solve) on two calls in a row, and that sizes beyond its fixed
scratch are refused.  It is collected last so that a run that stops at the first failure has
already run every other test.
"""

from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from symforce_gb300 import _cabi as A
from symforce_gb300.optimizer import SparseLdlt, lib

pytestmark = pytest.mark.gpu


def _spd(n, seed):
    rng = np.random.default_rng(seed)
    M = rng.normal(size=(n, n))
    return M @ M.T / n + np.eye(n), rng.normal(size=n)


def _reference_solve(Ad, b):
    n = Ad.shape[0]
    colptr, rowidx, vals = [0], [], []
    for c in range(n):
        rowidx += list(range(c, n))
        vals += list(Ad[c:, c])
        colptr.append(len(rowidx))
    s = SparseLdlt(n, colptr, rowidx)
    s.factorize(np.array(vals))
    return s.solve(b)


def _noalloc(Ad, b):
    torch = pytest.importorskip("torch")
    L = lib()
    f = L.sfg_dense_ldlt_solve_noalloc
    f.argtypes = [C.c_int32, C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p]
    n = Ad.shape[0]
    dA = torch.from_numpy(np.ascontiguousarray(Ad.T)).cuda()  # column-major A
    db = torch.from_numpy(b.copy()).cuda()
    dx = torch.zeros(n, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    rc = f(n, dA.data_ptr(), n, db.data_ptr(), dx.data_ptr(), None)
    assert rc == 0, L.sfg_last_error().decode()
    torch.cuda.synchronize()
    return dx.cpu().numpy()


def test_noalloc_matches_allocating_solver_two_calls():
    for n, seed in [(300, 1), (512, 2)]:
        Ad, b = _spd(n, seed)
        x_ref = _reference_solve(Ad, b)
        x = _noalloc(Ad, b)
        np.testing.assert_allclose(x, x_ref, rtol=1e-10, atol=1e-12)
        np.testing.assert_allclose(Ad @ x, b, rtol=1e-9, atol=1e-9)


def test_noalloc_rejects_oversize():
    torch = pytest.importorskip("torch")
    L = lib()
    f = L.sfg_dense_ldlt_solve_noalloc
    f.argtypes = [C.c_int32, C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p]
    d = torch.zeros(4, dtype=torch.float64, device="cuda")
    rc = f(513, d.data_ptr(), 513, d.data_ptr(), d.data_ptr(), None)
    assert rc == A.SFG_OK + 1  # SFG_ERR_INVALID_ARGUMENT
    assert b"513" in L.sfg_last_error()
