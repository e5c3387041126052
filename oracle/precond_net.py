"""Oracle (test infrastructure only) for the learned camera-block preconditioner.

CPU restatement, in float64 numpy, of the preconditioner path of the PCG forms: the camera-block
features of a reduced camera system S, the network's forward pass, its loss and gradient, the
assembly of the preconditioner blocks P_g, and a preconditioned conjugate-gradient solve.  The
reference has no learned preconditioner (its GPU back end, Caspar, uses block-Jacobi PCG:
symforce/caspar/code_generation/factor.py:218-251), so this restates the project's own
definitions from include/sfgpu.h ("learned preconditioner") and is pinned by finite differences
(loss gradient), by exact identities (zero weights give block Jacobi, P_g S_gg = I) and by the
CPU tests; the GPU kernels are compared against it.

Only tests/ may import this module.
"""

from __future__ import annotations

import numpy as np

BLOCK, FEATURES, HIDDEN, OUTPUTS = 9, 96, 256, 45
SAMPLE = FEATURES + 2 * BLOCK
DIAG_SHIFT = np.log(np.e - 1.0)  # softplus(DIAG_SHIFT) = 1
TRI = [(i, j) for i in range(BLOCK) for j in range(i + 1)]  # row-major lower triangle


def split(w: np.ndarray):
    w = np.asarray(w, dtype=np.float64)
    o = 0
    out = []
    for shape in [(FEATURES, HIDDEN), (HIDDEN,), (HIDDEN, HIDDEN), (HIDDEN,), (HIDDEN, OUTPUTS), (OUTPUTS,)]:
        n = int(np.prod(shape))
        out.append(w[o:o + n].reshape(shape))
        o += n
    assert o == w.size, (o, w.size)
    return out


def num_params() -> int:
    return FEATURES * HIDDEN + HIDDEN + HIDDEN * HIDDEN + HIDDEN + HIDDEN * OUTPUTS + OUTPUTS


def forward(w: np.ndarray, X: np.ndarray) -> np.ndarray:
    W1, b1, W2, b2, W3, b3 = split(w)
    H1 = np.maximum(X @ W1 + b1, 0.0)
    H2 = np.maximum(H1 @ W2 + b2, 0.0)
    return H2 @ W3 + b3


def softplus(x):
    return np.where(x > 20, x, np.log1p(np.exp(np.minimum(x, 20))))


def factor_from_outputs(z: np.ndarray) -> np.ndarray:
    """L (n, 9, 9) from the 45 outputs: off-diagonal z, diagonal softplus(z + ln(e - 1))."""
    n = z.shape[0]
    L = np.zeros((n, BLOCK, BLOCK))
    for t, (i, j) in enumerate(TRI):
        L[:, i, j] = softplus(z[:, t] + DIAG_SHIFT) if i == j else z[:, t]
    return L


def loss_grad(w: np.ndarray, samples: np.ndarray, kaporin: float = 0.0):
    """Mean of |L L^T g_hat - x_hat|^2 / (|x_hat|^2 + 1e-30) + kaporin (tr(L L^T) - log det(L L^T) - 9) / 9
    and its gradient w.r.t. the weights."""
    S = np.asarray(samples, dtype=np.float64)
    n = S.shape[0]
    X, gh, xh = S[:, :FEATURES], S[:, FEATURES:FEATURES + BLOCK], S[:, FEATURES + BLOCK:]
    W1, b1, W2, b2, W3, b3 = split(w)
    A1 = X @ W1 + b1
    H1 = np.maximum(A1, 0.0)
    A2 = H1 @ W2 + b2
    H2 = np.maximum(A2, 0.0)
    Z = H2 @ W3 + b3
    L = factor_from_outputs(Z)
    M = L @ np.transpose(L, (0, 2, 1))
    u = np.einsum("nij,nj->ni", M, gh) - xh
    s = np.sum(xh * xh, axis=1) + 1e-30
    diag = np.diagonal(L, axis1=1, axis2=2)
    kap = (np.sum(L * L, axis=(1, 2)) - 2.0 * np.sum(np.log(diag), axis=1) - BLOCK) / BLOCK
    per = np.sum(u * u, axis=1) / s + kaporin * kap
    loss = per.mean()
    # d/dL = (G + G^T) L, G = 2 u g^T / (s n); Kaporin term: kaporin (2 L - 2 diag(1/L_ii)) / (9 n)
    G = 2.0 * u[:, :, None] * gh[:, None, :] / (s * n)[:, None, None]
    dL = np.tril((G + np.transpose(G, (0, 2, 1))) @ L)
    dL += kaporin * 2.0 / (BLOCK * n) * (L - np.einsum("ni,ij->nij", 1.0 / diag, np.eye(BLOCK)))
    dZ = np.zeros_like(Z)
    for t, (i, j) in enumerate(TRI):
        if i == j:
            x = Z[:, t] + DIAG_SHIFT
            dZ[:, t] = dL[:, i, i] / (1.0 + np.exp(-x))
        else:
            dZ[:, t] = dL[:, i, j]
    gW3 = H2.T @ dZ
    gb3 = dZ.sum(0)
    dH2 = (dZ @ W3.T) * (A2 > 0)
    gW2 = H1.T @ dH2
    gb2 = dH2.sum(0)
    dH1 = (dH2 @ W2.T) * (A1 > 0)
    gW1 = X.T @ dH1
    gb1 = dH1.sum(0)
    grad = np.concatenate([gW1.ravel(), gb1, gW2.ravel(), gb2, gW3.ravel(), gb3])
    return loss, grad


def block_features(S: np.ndarray, gidx: np.ndarray, degree: np.ndarray):
    """Inputs of the network and the scaled Cholesky factor of every camera block.

    S: dense symmetric reduced system (n x n).  gidx: [ng, 9] scalar indices (-1 padding).
    Returns feats [ng, 96] and (C [ng, 9, 9] lower, dis [ng, 9] = diag^-1/2).
    """
    n = S.shape[0]
    ng = gidx.shape[0]
    group = np.full(n, -1)
    for g in range(ng):
        for a in range(BLOCK):
            if gidx[g, a] >= 0:
                group[gidx[g, a]] = g
    d = np.diag(S).copy()
    rho = np.zeros(n)
    for r in range(n):
        mask = group != group[r]
        rho[r] = np.sum(S[r, mask] ** 2 / np.maximum(d[r] * d[mask], 1e-30))
    feats = np.zeros((ng, FEATURES))
    C = np.zeros((ng, BLOCK, BLOCK))
    dis = np.ones((ng, BLOCK))
    for g in range(ng):
        idx = gidx[g]
        valid = idx >= 0
        A = np.eye(BLOCK)
        for a in range(BLOCK):
            if valid[a]:
                dis[g, a] = 1.0 / np.sqrt(S[idx[a], idx[a]]) if S[idx[a], idx[a]] > 0 else 1.0
        for a in range(BLOCK):
            for b in range(BLOCK):
                if valid[a] and valid[b]:
                    A[a, b] = S[idx[a], idx[b]] * dis[g, a] * dis[g, b]
        feats[g, :81] = A.ravel()
        feats[g, 81:90] = np.where(valid, np.log1p(rho[np.maximum(idx, 0)]), 0.0)
        feats[g, 90] = degree[g] / 16.0
        C[g] = np.linalg.cholesky(A)
    return feats, (C, dis)


def assemble(C: np.ndarray, dis: np.ndarray, z: np.ndarray | None) -> np.ndarray:
    """P_g = D^-1/2 C^-T L L^T C^-1 D^-1/2 for every block (L = I when z is None)."""
    ng = C.shape[0]
    L = np.broadcast_to(np.eye(BLOCK), (ng, BLOCK, BLOCK)) if z is None else factor_from_outputs(z)
    P = np.zeros((ng, BLOCK, BLOCK))
    for g in range(ng):
        Q = dis[g][:, None] * np.linalg.solve(C[g].T, L[g])
        P[g] = Q @ Q.T
    return P


def samples_of_system(S: np.ndarray, v: np.ndarray, gidx: np.ndarray, degree: np.ndarray) -> np.ndarray:
    """Training samples (114 floats per camera block) of one reduced system S y = v."""
    y = np.linalg.solve(S, v)
    feats, (C, dis) = block_features(S, gidx, degree)
    out = np.zeros((gidx.shape[0], SAMPLE))
    for g in range(gidx.shape[0]):
        idx = gidx[g]
        valid = idx >= 0
        vg = np.where(valid, v[np.maximum(idx, 0)], 0.0)
        yg = np.where(valid, y[np.maximum(idx, 0)], 0.0)
        out[g, :FEATURES] = feats[g]
        out[g, FEATURES:FEATURES + BLOCK] = np.linalg.solve(C[g], dis[g] * vg)
        out[g, FEATURES + BLOCK:] = C[g].T @ (yg / dis[g])
    return out


def band_preconditioner(S: np.ndarray, gidx: np.ndarray, band: int, z: np.ndarray | None = None,
                        tiny: float = 1e-12, return_factor: bool = False):
    """The band preconditioner M = G^T Lambda G (dense, n x n) of the PCG forms' pcg_band option.

    Group pattern: groups l, h are coupled when S has a nonzero entry between their scalars.  Per
    group row l: J_l = {h : l - band <= h < l, coupled to l} + {l} (ascending); A = D^-1/2 S_JJ
    D^-1/2 (identity on padding and non-positive-diagonal rows), R R^T = A, block row l of G = the
    last 9 rows of R^-1 times D^-1/2.  A Cholesky that meets a pivot <= tiny retries with J_l = {l};
    if that fails too the row is D^-1/2 (Jacobi).  Lambda_l = L L^T from the network outputs z
    (factor_from_outputs), or I.  band = 0 gives assemble()'s block-diagonal P_g.  With
    return_factor, (M, G) with G dense in the same scalar indices."""
    n = S.shape[0]
    ng = gidx.shape[0]
    valid = gidx >= 0
    sidx = np.where(valid, gidx, 0)

    def block(a, b):
        return np.where(valid[a][:, None] & valid[b][None, :], S[np.ix_(sidx[a], sidx[b])], 0.0)

    def coupled(a, b):
        return bool(np.any(block(a, b) != 0.0))

    d = np.where(valid, np.diag(S)[sidx], 0.0)
    dis = np.where(valid & (d > 0), 1.0 / np.sqrt(np.where(d > 0, d, 1.0)), -1.0)  # -1: identity row
    Lam = (np.broadcast_to(np.eye(BLOCK), (ng, BLOCK, BLOCK)) if z is None
           else np.einsum("nij,nkj->nik", factor_from_outputs(z), factor_from_outputs(z)))

    def chol(A):
        m = A.shape[0]
        R = np.zeros_like(A)
        for j in range(m):
            s = A[j:, j] - R[j:, :j] @ R[j, :j]
            if not s[0] > tiny:
                return None
            R[j, j] = np.sqrt(s[0])
            R[j + 1:, j] = s[1:] / R[j, j]
        return R

    G = {}  # (l, h) -> 9 x 9 block of G
    for l in range(ng):
        J = [h for h in range(max(0, l - band), l) if coupled(l, h)] + [l]
        done = False
        for Jt in (J, [l]):
            m = len(Jt)
            A = np.zeros((9 * m, 9 * m))
            for i1, a in enumerate(Jt):
                for i2, b in enumerate(Jt):
                    A[9 * i1:9 * i1 + 9, 9 * i2:9 * i2 + 9] = block(a, b)
            ds = np.concatenate([dis[h] for h in Jt])
            ident = ds < 0
            A = A * np.where(ident, 1.0, ds)[:, None] * np.where(ident, 1.0, ds)[None, :]
            A[ident, :] = 0.0
            A[:, ident] = 0.0
            A[ident, ident] = 1.0
            R = chol(A)
            if R is None:
                continue
            X = np.linalg.inv(R)[-9:, :] * np.where(ident, 1.0, ds)[None, :]
            for i, h in enumerate(Jt):
                G[(l, h)] = X[:, 9 * i:9 * i + 9]
            done = True
            break
        if not done:
            G[(l, l)] = np.diag(np.where(d[l] > 0, 1.0 / np.sqrt(np.where(d[l] > 0, d[l], 1.0)), 1.0))
    Mg = np.zeros((ng, BLOCK, ng, BLOCK))
    for (l, a), Ga in G.items():
        for (l2, b), Gb in G.items():
            if l2 == l:
                Mg[a, :, b, :] += Ga.T @ Lam[l] @ Gb
    M = np.zeros((n, n))
    for a in range(ng):
        for b in range(ng):
            blk = Mg[a, :, b, :][np.ix_(valid[a], valid[b])]
            M[np.ix_(gidx[a][valid[a]], gidx[b][valid[b]])] = blk
    if not return_factor:
        return M
    Gd = np.zeros((n, n))
    for (l, h), blk in G.items():
        Gd[np.ix_(gidx[l][valid[l]], gidx[h][valid[h]])] = blk[np.ix_(valid[l], valid[h])]
    return M, Gd


def pcg_dense(S: np.ndarray, v: np.ndarray, M: np.ndarray, tol: float = 1e-8, max_iters: int = 1000):
    """CG preconditioned by the dense M in float64 (x0 = 0); returns (x, iterations, relative residual)."""
    x = np.zeros_like(v)
    r = v.copy()
    zr = M @ r
    p = zr.copy()
    rz = r @ zr
    vn = np.linalg.norm(v)
    it = 0
    while np.linalg.norm(r) > tol * vn and it < max_iters:
        q = S @ p
        alpha = rz / (p @ q)
        x += alpha * p
        r -= alpha * q
        zr = M @ r
        rz_new = r @ zr
        p = zr + (rz_new / rz) * p
        rz = rz_new
        it += 1
    return x, it, np.linalg.norm(v - S @ x) / vn


def pcg(S: np.ndarray, v: np.ndarray, P: np.ndarray, gidx: np.ndarray, tol: float = 1e-8,
        max_iters: int = 1000):
    """Block-preconditioned CG in float64 (x0 = 0); returns (x, iterations, relative residual)."""
    def apply(r):
        z = np.zeros_like(r)
        for g in range(gidx.shape[0]):
            idx = gidx[g]
            valid = idx >= 0
            ii = idx[valid]
            z[ii] = P[g][np.ix_(valid, valid)] @ r[ii]
        return z

    x = np.zeros_like(v)
    r = v.copy()
    z = apply(r)
    p = z.copy()
    rz = r @ z
    vn = np.linalg.norm(v)
    it = 0
    while np.linalg.norm(r) > tol * vn and it < max_iters:
        q = S @ p
        alpha = rz / (p @ q)
        x += alpha * p
        r -= alpha * q
        z = apply(r)
        rz_new = r @ z
        p = z + (rz_new / rz) * p
        rz = rz_new
        it += 1
    return x, it, np.linalg.norm(v - S @ x) / vn
