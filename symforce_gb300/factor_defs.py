"""Symbolic definitions of the generated factor kinds.

Each entry is a residual written in sympy over the storage of its keys and the factor's constants,
restating a factor of the reference (cited per definition).  `python -m symforce_gb300.codegen
--write` turns them into symforce_gb300/csrc/generated_factors.cuh (residual in FP64 and tangent
Jacobian through the keys' retractions, shared subexpressions) and generated_factor_specs.h (the
dimension table the host code reads); the library registers every kind listed here as a factor
kind of its linearization kernel.
"""

from __future__ import annotations

from dataclasses import dataclass
from typing import Callable, List

import sympy as sp

from . import _cabi as A


@dataclass(frozen=True)
class FactorDef:
    name: str            # struct name in the generated header
    kind: int            # SFG_FACTOR_* id
    enum: str            # SFG_FACTOR_* name
    key_types: tuple
    num_consts: int
    residual: Callable[[List[sp.Matrix], List[sp.Symbol]], sp.Matrix]
    doc: str


def _sign_no_zero(x):
    return sp.Piecewise((1, x >= 0), (-1, True))


def _abs(x):
    return sp.Piecewise((x, x >= 0), (-x, True))


def quat_mul(p, q):
    """Hamilton product p ⊗ q of [x, y, z, w] quaternions."""
    px, py, pz, pw = p
    qx, qy, qz, qw = q
    return [pw * qx + px * qw + py * qz - pz * qy,
            pw * qy - px * qz + py * qw + pz * qx,
            pw * qz + px * qy - py * qx + pz * qw,
            pw * qw - px * qx - py * qy - pz * qz]


def quat_conj(q):
    return [-q[0], -q[1], -q[2], q[3]]


def rot3_log(q, eps):
    """Rot3.to_tangent (symforce/geo/rot3.py:89-100, to_tangent_norm :152-163): the quaternion's
    sign flipped to w >= 0, w clamped below 1 - eps, tangent = xyz / sqrt(1 - w^2) * 2 acos(w)."""
    w_pos = _abs(q[3])
    w_safe = sp.Piecewise((1 - eps, w_pos > 1 - eps), (w_pos, True))
    s = _sign_no_zero(q[3])
    k = 2 * sp.acos(w_safe) / sp.sqrt(1 - w_safe ** 2)
    return [s * q[i] * k for i in range(3)]


def prior_rot3(keys, c):
    """prior_factor (symforce/codegen/geo_factors_codegen.py:75-86) for Rot3 with a diagonal
    sqrt_info: diag(s) local_coordinates(prior, value) = diag(s) Log(prior^-1 value).
    consts [prior q (4), s (3), eps]."""
    x = list(keys[0])
    w = rot3_log(quat_mul(quat_conj(c[0:4]), x), c[7])
    return sp.Matrix([c[4 + i] * w[i] for i in range(3)])


def between_rot3(keys, c):
    """between_factor (symforce/codegen/geo_factors_codegen.py:53-72) for Rot3 with a diagonal
    sqrt_info: diag(s) local_coordinates(a_T_b, a^-1 b).  consts [a_T_b q (4), s (3), eps]."""
    a, b = list(keys[0]), list(keys[1])
    est = quat_mul(quat_conj(a), b)
    w = rot3_log(quat_mul(quat_conj(c[0:4]), est), c[7])
    return sp.Matrix([c[4 + i] * w[i] for i in range(3)])


def barron_vec5(keys, c):
    """The GNC test factor of the reference (test/symforce_gnc_codegen_test.py:24-31): the Barron
    noise model (symforce/opt/noise_models.py:318-428, delta 1, scalar_information 1,
    x_epsilon = alpha_epsilon = eps) with alpha = 2 - 1 / (1 - mu + eps)
    (BarronNoiseModel.compute_alpha_from_mu) whitening x - y element by element.
    consts [y (5), mu, eps]; mu is the convexity parameter a GNC schedule changes between stages."""
    x = keys[0]
    mu, eps = c[5], c[6]
    alpha = 2 - 1 / (1 - mu + eps)
    b = _abs(alpha - 2) + eps
    d = alpha + _sign_no_zero(alpha) * eps
    out = []
    for i in range(5):
        e = x[i] - c[i]
        barron = (b / d) * ((e ** 2 / b + 1) ** (d / 2) - 1)
        out.append(sp.sqrt(2 * barron + eps) - sp.sqrt(eps))
    return sp.Matrix(out)


def linear_vec5(keys, c):
    """r = J x + b for a 5-vector key, J 9 x 5 (row-major) and b 9 in the constants: the linear
    least-squares residual of test/symforce_levenberg_marquardt_test.cc:17-88 (b = 0 there)."""
    x = keys[0]
    return sp.Matrix([sum(c[5 * i + j] * x[j] for j in range(5)) + c[45 + i] for i in range(9)])


def linear_scalar2(keys, c):
    """r = J [x, y] + b over two scalar keys, J 2 x 2 (row-major) and b 2 in the constants: the
    factors of test/symforce_linearizer_test.cc:16-43 (b = 0 there)."""
    x, y = keys[0][0], keys[1][0]
    return sp.Matrix([c[0] * x + c[1] * y + c[4], c[2] * x + c[3] * y + c[5]])


GENERATED = [
    FactorDef("GenPriorRot3", A.SFG_FACTOR_PRIOR_ROT3, "SFG_FACTOR_PRIOR_ROT3", (A.SFG_KEY_ROT3,), 8,
              prior_rot3, "diag(s) Log(prior^-1 x)"),
    FactorDef("GenBetweenRot3", A.SFG_FACTOR_BETWEEN_ROT3, "SFG_FACTOR_BETWEEN_ROT3",
              (A.SFG_KEY_ROT3, A.SFG_KEY_ROT3), 8, between_rot3, "diag(s) Log(a_T_b^-1 a^-1 b)"),
    FactorDef("GenBarronVec5", A.SFG_FACTOR_BARRON_VEC5, "SFG_FACTOR_BARRON_VEC5", (A.SFG_KEY_VEC5,), 7,
              barron_vec5, "Barron-whitened x - y, alpha from mu"),
    FactorDef("GenLinearVec5", A.SFG_FACTOR_LINEAR_VEC5, "SFG_FACTOR_LINEAR_VEC5", (A.SFG_KEY_VEC5,), 54,
              linear_vec5, "J x + b, J 9 x 5"),
    FactorDef("GenLinearScalar2", A.SFG_FACTOR_LINEAR_SCALAR2, "SFG_FACTOR_LINEAR_SCALAR2",
              (A.SFG_KEY_VEC1, A.SFG_KEY_VEC1), 6, linear_scalar2, "J [x, y] + b, J 2 x 2"),
]
