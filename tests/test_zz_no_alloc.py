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


def _noalloc(Ad, b, stream=None, expect=0):
    """One call through the C ABI; `stream` is a torch.cuda.Stream (None: the default stream)."""
    torch = pytest.importorskip("torch")
    L = lib()
    f = L.sfg_dense_ldlt_solve_noalloc
    f.argtypes = [C.c_int32, C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p]
    n = Ad.shape[0]
    dA = torch.from_numpy(np.ascontiguousarray(Ad.T)).cuda()  # column-major A
    db = torch.from_numpy(b.copy()).cuda()
    dx = torch.zeros(n, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    rc = f(n, dA.data_ptr(), n, db.data_ptr(), dx.data_ptr(),
           None if stream is None else stream.cuda_stream)
    assert rc == expect, L.sfg_last_error().decode()
    torch.cuda.synchronize()
    return dx.cpu().numpy()


def test_noalloc_matches_allocating_solver_two_calls():
    for n, seed in [(300, 1), (512, 2)]:
        Ad, b = _spd(n, seed)
        x_ref = _reference_solve(Ad, b)
        x = _noalloc(Ad, b)
        np.testing.assert_allclose(x, x_ref, rtol=1e-10, atol=1e-12)
        np.testing.assert_allclose(Ad @ x, b, rtol=1e-9, atol=1e-9)


def test_noalloc_smaller_after_larger_and_on_a_stream():
    """The shared scratch keeps the last call's contents: a smaller system after a larger one must
    not read the larger one's tile states, tasks or front entries; and a caller's own stream works
    like the default stream."""
    torch = pytest.importorskip("torch")
    stream = torch.cuda.Stream()
    for n, seed, st in [(512, 3, None), (17, 4, None), (300, 5, stream), (16, 6, stream), (1, 7, None)]:
        Ad, b = _spd(n, seed)
        x_ref = _reference_solve(Ad, b)
        x = _noalloc(Ad, b, stream=st)
        np.testing.assert_allclose(x, x_ref, rtol=1e-10, atol=1e-12)


def test_noalloc_reports_a_zero_pivot():
    """A singular A (a zero row and column) gives SFG_ERR_NUMERICAL, not silent inf / NaN, and the
    next call on a regular system is unaffected."""
    Ad, b = _spd(40, 8)
    Ad[5, :] = 0.0
    Ad[:, 5] = 0.0
    _noalloc(Ad, b, expect=A.SFG_ERR_NUMERICAL)
    Ad, b = _spd(40, 9)
    np.testing.assert_allclose(_noalloc(Ad, b), _reference_solve(Ad, b), rtol=1e-10, atol=1e-12)


def test_noalloc_rejects_oversize():
    torch = pytest.importorskip("torch")
    L = lib()
    f = L.sfg_dense_ldlt_solve_noalloc
    f.argtypes = [C.c_int32, C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p]
    d = torch.zeros(4, dtype=torch.float64, device="cuda")
    rc = f(513, d.data_ptr(), 513, d.data_ptr(), d.data_ptr(), None)
    assert rc == A.SFG_OK + 1  # SFG_ERR_INVALID_ARGUMENT
    assert b"513" in L.sfg_last_error()
