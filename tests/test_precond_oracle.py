"""The learned-preconditioner oracle pinned on the CPU: finite-difference gradient of the loss,
zero weights = block Jacobi, the block assembly identity P_g S_gg = I, and the PCG restatement."""

from __future__ import annotations

import numpy as np
import pytest

import precond_cases as PC
from oracle import precond_net as PN
from symforce_gb300 import synth


@pytest.mark.parametrize("kaporin", [0.0, 0.7])
def test_loss_gradient_matches_finite_differences(kaporin):
    rng = np.random.Generator(np.random.PCG64(1))
    samples = PC.oracle_samples((3,))[:12].astype(np.float64)
    w = PC.random_weights(2, out_scale=0.2).astype(np.float64)
    f = lambda x: PN.loss_grad(x, samples, kaporin)[0]  # noqa: E731
    loss, grad = PN.loss_grad(w, samples, kaporin)
    assert np.isfinite(loss) and loss > 0
    # directional derivatives along random directions and along single coordinates of each layer
    for _ in range(4):
        d = rng.normal(size=w.size)
        h = 1e-6
        fd = (f(w + h * d) - f(w - h * d)) / (2 * h)
        assert abs(fd - grad @ d) <= 1e-5 * max(1.0, abs(fd)), (fd, grad @ d)
    offs = np.cumsum([0, 96 * 256, 256, 256 * 256, 256, 256 * 45, 45])
    for a, b in zip(offs[:-1], offs[1:]):
        i = int(a + np.argmax(np.abs(grad[a:b])))
        e = np.zeros(w.size)
        e[i] = 1.0
        h = 1e-6
        fd = (f(w + h * e) - f(w - h * e)) / (2 * h)
        assert abs(fd - grad[i]) <= 1e-5 * max(1e-3, abs(fd)), (i, fd, grad[i])


def test_kaporin_term_is_zero_only_at_block_jacobi():
    """The Kaporin term is tr(M) - log det(M) - 9 over 9 for M = L L^T: zero outputs (L = I, block
    Jacobi) give exactly zero and zero gradient; any other output raises it."""
    samples = PC.oracle_samples((3,))[:8].astype(np.float64)
    w = PC.random_weights(4, out_scale=0.2).astype(np.float64)
    w_bj = w.copy()
    w_bj[-(256 * 45 + 45):] = 0.0
    l0, g0 = PN.loss_grad(w_bj, samples, 0.0)
    l1, g1 = PN.loss_grad(w_bj, samples, 3.0)
    assert l1 == pytest.approx(l0, rel=1e-12)
    np.testing.assert_allclose(g1, g0, rtol=0, atol=1e-12 * max(1.0, np.abs(g0).max()))
    assert PN.loss_grad(w, samples, 3.0)[0] > PN.loss_grad(w, samples, 0.0)[0]


def test_zero_output_layer_is_block_jacobi():
    p = PC.small_ba(3)
    S, v = PC.reduced_system(p)
    gidx, degree = PC.camera_blocks(p)
    feats, (C, dis) = PN.block_features(S, gidx, degree)
    w = PC.random_weights(0)
    w[-(256 * 45 + 45):] = 0.0
    z = PN.forward(w.astype(np.float64), feats)
    assert np.abs(z).max() == 0.0
    P = PN.assemble(C, dis, z)
    for g in range(gidx.shape[0]):
        Sgg = S[np.ix_(gidx[g], gidx[g])]
        np.testing.assert_allclose(P[g] @ Sgg, np.eye(9), atol=1e-9)
    # features: unit diagonal of the scaled block, symmetric
    A = feats[:, :81].reshape(-1, 9, 9)
    np.testing.assert_allclose(np.diagonal(A, axis1=1, axis2=2), 1.0, atol=1e-12)
    np.testing.assert_allclose(A, np.transpose(A, (0, 2, 1)), atol=1e-12)


def test_samples_whitening_identities():
    p = PC.small_ba(5)
    S, v = PC.reduced_system(p)
    gidx, degree = PC.camera_blocks(p)
    s = PN.samples_of_system(S, v, gidx, degree)
    _, (C, dis) = PN.block_features(S, gidx, degree)
    y = np.linalg.solve(S, v)
    for g in range(gidx.shape[0]):
        # L = I: P_g v_g - y_g in the S_gg norm equals |g_hat - x_hat|
        Sgg = S[np.ix_(gidx[g], gidx[g])]
        e = np.linalg.solve(Sgg, v[gidx[g]]) - y[gidx[g]]
        gh, xh = s[g, 96:105], s[g, 105:]
        assert np.isclose(e @ Sgg @ e, np.sum((gh - xh) ** 2), rtol=1e-8)


def test_oracle_pcg_solves_reduced_system():
    p = PC.small_ba(3)
    S, v = PC.reduced_system(p)
    gidx, degree = PC.camera_blocks(p)
    _, (C, dis) = PN.block_features(S, gidx, degree)
    P = PN.assemble(C, dis, None)
    x, it, rel = PN.pcg(S, v, P, gidx, tol=1e-10)
    assert rel <= 1e-10 and it < S.shape[0]
    np.testing.assert_allclose(x, np.linalg.solve(S, v), rtol=1e-7, atol=1e-9 * np.abs(x).max())


def _block_matrix(P, gidx, n):
    M = np.zeros((n, n))
    for g in range(gidx.shape[0]):
        idx = gidx[g]
        M[np.ix_(idx, idx)] = P[g]
    return M


@pytest.mark.parametrize("with_net", [False, True])
def test_band_zero_is_the_block_diagonal_preconditioner(with_net):
    """pcg_band = 0 of the band preconditioner is P_g = D^-1/2 C^-T L L^T C^-1 D^-1/2: block
    Jacobi with L = I, the learned blocks with the network's L (the same normalization of G)."""
    p = PC.small_ba(3)
    S, v = PC.reduced_system(p)
    gidx, degree = PC.camera_blocks(p)
    feats, (C, dis) = PN.block_features(S, gidx, degree)
    z = PN.forward(PC.random_weights(3, out_scale=0.2).astype(np.float64), feats) if with_net else None
    M = PN.band_preconditioner(S, gidx, 0, z)
    ref = _block_matrix(PN.assemble(C, dis, z), gidx, S.shape[0])
    np.testing.assert_allclose(M, ref, rtol=0, atol=1e-12 * np.abs(ref).max())


def test_band_factor_normalizes_diagonal_blocks():
    """G S G^T has identity diagonal blocks (M = G^T G with Lambda = I), M is symmetric positive
    definite, and wider bands cut the CG iterations of a 30-camera reduced system."""
    p = synth.bundle_adjustment(num_cameras=30, num_points=3000, num_observations=18000, seed=2)
    S, v = PC.reduced_system(p)
    gidx, _ = PC.camera_blocks(p)
    M, G = PN.band_preconditioner(S, gidx, 3, return_factor=True)
    np.testing.assert_allclose(M, G.T @ G, rtol=0, atol=1e-9 * np.abs(M).max())
    K = G @ S @ G.T
    for g in range(gidx.shape[0]):
        np.testing.assert_allclose(K[np.ix_(gidx[g], gidx[g])], np.eye(9), rtol=0, atol=1e-8)
    # G is block lower triangular over at most 3 + 1 groups of a row
    for g in range(gidx.shape[0]):
        for h in range(gidx.shape[0]):
            if h > g or h < g - 3:
                assert not np.any(G[np.ix_(gidx[g], gidx[h])])
    np.testing.assert_allclose(M, M.T, rtol=0, atol=1e-9 * np.abs(M).max())
    assert np.linalg.eigvalsh(M).min() > 0
    its = [PN.pcg_dense(S, v, PN.band_preconditioner(S, gidx, k), tol=1e-8)[1] for k in (0, 2, 4)]
    assert its[1] < its[0] and its[2] < its[1], its
