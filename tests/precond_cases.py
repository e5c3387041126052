"""Shared inputs of the learned-preconditioner tests: reduced camera systems of small bundle
adjustment problems built from the oracle's linearization, their camera blocks, and random
network weights with every layer active."""

from __future__ import annotations

import numpy as np

import oracle_lib as O
from oracle import precond_net as PN
from symforce_gb300 import _cabi as A
from symforce_gb300 import synth


def camera_blocks(problem: A.ProblemArrays):
    """[nc, 9] reduced-system scalars (pose 6 + intrinsics 3) and the co-visibility degree."""
    nc = int(problem.meta["num_cameras"])
    gidx = np.zeros((nc, 9), dtype=np.int64)
    for k in range(nc):
        gidx[k, :6] = 6 * k + np.arange(6)
        gidx[k, 6:] = 6 * nc + 3 * k + np.arange(3)
    keys = problem.batches[0].keys
    cams_of_point = {}
    for c, _, pt in keys:
        cams_of_point.setdefault(int(pt), set()).add(int(c))
    nbr = [set() for _ in range(nc)]
    for cams in cams_of_point.values():
        for a in cams:
            nbr[a] |= cams - {a}
    degree = np.array([len(s) for s in nbr], dtype=np.float64)
    return gidx, degree


def reduced_system(problem: A.ProblemArrays, lam: float = 1.0, values=None):
    """S = (B + lam I) - E (C + lam I)^-1 E^T and v = g_B - E (C + lam I)^-1 g_C from the oracle's
    linearization (unit damping lam, the LM default), dense."""
    lin = O.linearize(problem, values)
    N = lin["rhs"].size
    H = np.zeros((N, N))
    cp, ri, hv = lin["colptr"], lin["rowidx"], lin["hvals"]
    for j in range(N):
        for q in range(cp[j], cp[j + 1]):
            H[ri[q], j] = hv[q]
            H[j, ri[q]] = hv[q]
    H += lam * np.eye(N)
    nB = N - 3 * problem.num_schur_keys
    B, E, Cm = H[:nB, :nB], H[nB:, :nB], H[nB:, nB:]
    g = lin["rhs"]
    Ci = np.linalg.inv(Cm)
    S = B - E.T @ Ci @ E
    v = g[:nB] - E.T @ Ci @ g[nB:]
    return 0.5 * (S + S.T), v


def small_ba(seed: int = 3):
    return synth.bundle_adjustment(num_cameras=8, num_points=240, num_observations=1000, seed=seed)


def random_weights(seed: int = 0, out_scale: float = 0.05) -> np.ndarray:
    rng = np.random.Generator(np.random.PCG64(seed))
    F, H, O_ = PN.FEATURES, PN.HIDDEN, PN.OUTPUTS
    parts = [rng.normal(0, np.sqrt(2.0 / F), F * H), rng.normal(0, 0.1, H),
             rng.normal(0, np.sqrt(2.0 / H), H * H), rng.normal(0, 0.1, H),
             rng.normal(0, out_scale, H * O_), rng.normal(0, out_scale, O_)]
    return np.concatenate(parts).astype(np.float32)


def oracle_samples(seeds=(3, 5)) -> np.ndarray:
    out = []
    for s in seeds:
        p = small_ba(s)
        S, v = reduced_system(p)
        gidx, degree = camera_blocks(p)
        out.append(PN.samples_of_system(S, v, gidx, degree))
    return np.concatenate(out, 0)
