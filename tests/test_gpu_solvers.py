"""The standalone LinearSolver boundaries on the GPU, against dense solves.

- `sfg_ldlt_*` (SparseCholeskySolver: AnalyzeSparsityPattern / Factorize / Solve / D() /
  Permutation(), symforce/opt/sparse_cholesky/sparse_cholesky_solver.h:28-163) on the random
  sparse symmetric systems of test/sparse_cholesky_solver_test.cc:26-184: the pattern of M^T M for an
  M with a random diagonal and 5 n random entries, then the diagonal overwritten with N(0, 1) draws
  (so the systems are indefinite: LDL^T without pivoting, like the reference), a vector and an
  11-column right-hand side, every block ordering the library offers.  D() is checked against the
  dense LDL^T of the permuted matrix, Permutation() for being a permutation.
- `sfg_schur_*` (SparseSchurSolver, symforce/opt/sparse_schur_solver.h:62-135) on bundle-adjustment
  shaped systems with 3 x 3 block-diagonal C, against a dense solve
  (test/sparse_schur_solver_test.cc:105-250).
"""

from __future__ import annotations

import numpy as np
import pytest

from symforce_gb300 import _cabi as A
from symforce_gb300.optimizer import SparseLdlt, SparseSchur

pytestmark = pytest.mark.gpu

ORDERINGS = [A.SFG_ORDERING_NATURAL, A.SFG_ORDERING_MIN_DEGREE, A.SFG_ORDERING_NESTED_DISSECTION]


def _csc_lower(Ad: np.ndarray):
    n = Ad.shape[0]
    L = np.tril(Ad)
    colptr, rowidx, vals = [0], [], []
    for c in range(n):
        rows = np.nonzero(L[:, c])[0]
        rows = rows[rows >= c]
        if c not in rows:
            rows = np.sort(np.append(rows, c))
        rowidx += list(rows)
        vals += list(L[rows, c])
        colptr.append(len(rowidx))
    return np.array(colptr, np.int32), np.array(rowidx, np.int32), np.array(vals)


def _random_symmetric(n: int, rng: np.random.Generator) -> np.ndarray:
    """MakeRandomSymmetricSparseMatrix (test/sparse_cholesky_solver_test.cc:26-48) with numpy
    draws, then the diagonal set to N(0, 1) as the test's A_modified (:92-96)."""
    M = np.zeros((n, n))
    M[np.arange(n), np.arange(n)] = rng.normal(size=n)
    rows = rng.integers(0, n, size=5 * n)
    cols = rng.integers(0, n, size=5 * n)
    M[rows, cols] = rng.normal(size=5 * n)
    Ad = M.T @ M
    Ad[np.arange(n), np.arange(n)] = rng.normal(size=n)
    return Ad


def _is_approx(x, y, tol):
    """Eigen's isApprox: |x - y| <= tol * min(|x|, |y|)."""
    return np.linalg.norm(x - y) <= tol * min(np.linalg.norm(x), np.linalg.norm(y))


def _dense_ldlt_d(Ap: np.ndarray) -> np.ndarray:
    """Diagonal D of the unpivoted LDL^T of a symmetric matrix (right-looking, FP64)."""
    a = Ap.copy()
    n = a.shape[0]
    d = np.zeros(n)
    for k in range(n):
        d[k] = a[k, k]
        l = a[k + 1:, k] / d[k]
        a[k + 1:, k + 1:] -= np.outer(l, a[k + 1:, k])
    return d


@pytest.mark.parametrize("ordering", ORDERINGS)
def test_ldlt_random_indefinite_systems_against_dense(ordering):
    """test/sparse_cholesky_solver_test.cc:59-131 (dim 300, tolerance 1e-5 as there; our FP64 LDL^T
    meets far tighter bounds on these systems, checked at 1e-8 through the residual)."""
    n = 300
    rng = np.random.default_rng(42 + ordering)
    for _ in range(3):
        Ad = _random_symmetric(n, rng)
        cp, ri, v = _csc_lower(Ad)
        s = SparseLdlt(n, cp, ri, ordering=ordering)
        for _ in range(3):
            # the reference's loop: same pattern, a new diagonal per factorization
            Ad[np.arange(n), np.arange(n)] = rng.normal(size=n)
            _, _, v = _csc_lower(Ad)
            b = rng.normal(size=n)
            s.factorize(v)
            x = s.solve(b)
            x_ref = np.linalg.solve(Ad, b)
            assert _is_approx(x, x_ref, 1e-5)
            cond = np.linalg.cond(Ad)
            assert np.linalg.norm(Ad @ x - b) <= 1e-12 * cond * np.linalg.norm(b) + 1e-8 * np.linalg.norm(b)
        perm = s.permutation()
        assert sorted(perm.tolist()) == list(range(n))
        P = np.zeros((n, n))
        P[perm, np.arange(n)] = 1.0  # row perm[i] of P A P^T is row i of A
        Ap = P @ Ad @ P.T
        np.testing.assert_allclose(s.diagonal(), _dense_ldlt_d(Ap), rtol=1e-8,
                                   atol=1e-10 * np.abs(np.diag(Ap)).max())


@pytest.mark.parametrize("ordering", ORDERINGS)
def test_ldlt_matrix_rhs_and_spd_at_1e10(ordering):
    """test/sparse_cholesky_solver_test.cc:134-184: an 11-column right-hand side; on a well
    conditioned SPD system the FP64 result agrees with a dense solve at 1e-10."""
    n = 300
    rng = np.random.default_rng(7)
    Ad = _random_symmetric(n, rng)
    Ad = Ad @ Ad.T / n + np.eye(n)  # SPD with a fill pattern of its own
    Ad[np.abs(Ad) < 0.05] = 0.0
    Ad = 0.5 * (Ad + Ad.T) + n * np.eye(n) * 0.05
    cp, ri, v = _csc_lower(Ad)
    s = SparseLdlt(n, cp, ri, ordering=ordering)
    s.factorize(v)
    B = rng.normal(size=(n, 11))
    X = s.solve(B)
    X_ref = np.linalg.solve(Ad, B)
    np.testing.assert_allclose(X, X_ref, rtol=1e-10, atol=1e-12 * np.abs(X_ref).max())
    assert _is_approx(X, X_ref, 1e-10)


def _ba_shaped(nb_cams: int, n_pts: int, rng: np.random.Generator):
    """A symmetric positive definite [[B, E^T], [E, C]] with 9-wide camera blocks (pose 6 +
    intrinsics 3), 3 x 3 point blocks, each point seen by 2-4 cameras."""
    nb = 9 * nb_cams
    n = nb + 3 * n_pts
    J_rows = []
    for p in range(n_pts):
        cams = rng.choice(nb_cams, size=rng.integers(2, 5), replace=False)
        for c in cams:
            row = np.zeros((2, n))
            row[:, 9 * c:9 * c + 9] = rng.normal(size=(2, 9))
            row[:, nb + 3 * p:nb + 3 * p + 3] = rng.normal(size=(2, 3))
            J_rows.append(row)
    J = np.vstack(J_rows)
    H = J.T @ J + 1e-1 * np.eye(n)
    return H, nb


def test_schur_against_dense():
    rng = np.random.default_rng(3)
    H, nb = _ba_shaped(6, 60, rng)
    n = H.shape[0]
    cp, ri, v = _csc_lower(H)
    s = SparseSchur(n, cp, ri, n - nb)
    s.factorize(v)
    b = rng.normal(size=n)
    x = s.solve(b)
    np.testing.assert_allclose(x, np.linalg.solve(H, b), rtol=1e-10, atol=1e-12 * np.abs(x).max())
    B = rng.normal(size=(n, 5))
    X = s.solve(B)
    np.testing.assert_allclose(X, np.linalg.solve(H, B), rtol=1e-10, atol=1e-12 * np.abs(X).max())
    # refactorize with other values on the same structure
    H2 = H.copy()
    H2[np.arange(n), np.arange(n)] += rng.uniform(0.5, 2.0, size=n)
    _, _, v2 = _csc_lower(H2)
    s.factorize(v2)
    x2 = s.solve(b)
    np.testing.assert_allclose(x2, np.linalg.solve(H2, b), rtol=1e-10, atol=1e-12 * np.abs(x2).max())


@pytest.mark.parametrize("ordering", ORDERINGS)
def test_ldlt_lower_reconstructs_permuted_matrix(ordering):
    """L() with D() and Permutation(): P A P^T == (I + L) D (I + L)^T, the contract the reference's
    debug stats read (symforce/opt/levenberg_marquardt_solver.tcc:209-211)."""
    n = 120
    rng = np.random.default_rng(11 + ordering)
    Ad = _random_symmetric(n, rng)
    Ad = Ad @ Ad.T / n + np.eye(n)
    Ad[np.abs(Ad) < 0.3] = 0.0
    Ad = 0.5 * (Ad + Ad.T) + 2.0 * np.eye(n)
    cp, ri, v = _csc_lower(Ad)
    s = SparseLdlt(n, cp, ri, ordering=ordering)
    s.factorize(v)
    low = s.lower()
    assert low["colptr"][0] == 0 and low["colptr"][-1] == low["rowidx"].size
    Ld = np.eye(n)
    for c in range(n):
        rows = low["rowidx"][low["colptr"][c]:low["colptr"][c + 1]]
        assert (rows > c).all() and (np.diff(rows) > 0).all()
        Ld[rows, c] = low["values"][low["colptr"][c]:low["colptr"][c + 1]]
    perm = s.permutation()
    P = np.zeros((n, n))
    P[perm, np.arange(n)] = 1.0
    np.testing.assert_allclose(Ld @ np.diag(s.diagonal()) @ Ld.T, P @ Ad @ P.T, rtol=1e-10,
                               atol=1e-11 * np.abs(Ad).max())
