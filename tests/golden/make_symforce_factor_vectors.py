"""Generate tests/golden/factor_vectors.json from the reference's own symbolic factor definitions.

Imports symforce (sympy back end) from the reference checkout given as argv[1] (required), builds each residual exactly as the reference
defines it, differentiates it with symforce's tangent-space Jacobian helper (the same helper the
reference's `with_linearization` codegen uses), and evaluates residual and Jacobian at seeded random
inputs with 60-digit arithmetic.  Run once from the repository root; the JSON is committed and the
tests read only the JSON.

    python tests/golden/make_symforce_factor_vectors.py /path/to/symforce
"""

from __future__ import annotations

import json
import math
import sys
from pathlib import Path

import numpy as np

if len(sys.argv) < 2:
    sys.exit("usage: make_symforce_factor_vectors.py /path/to/symforce  (the reference checkout)")
REF = Path(sys.argv[1])
sys.path.insert(0, str(REF))
sys.path.insert(0, str(REF / "gen" / "python"))

import types  # noqa: E402

# symforce.opt.factor imports graphviz only for plotting; it is not installed here
sys.modules.setdefault("graphviz", types.ModuleType("graphviz"))
import symforce  # noqa: E402


symforce.set_symbolic_api("sympy")
symforce.set_epsilon_to_symbol()
import ast  # noqa: E402

import mpmath  # noqa: E402
import sympy  # noqa: E402

import symforce.symbolic as sf  # noqa: E402
from symforce import jacobian_helpers  # noqa: E402
from symforce.codegen import geo_factors_codegen  # noqa: E402
from symforce.opt.noise_models import BarronNoiseModel  # noqa: E402



def load_functions(path: Path, names: list) -> dict:
    """Compile only the named top-level functions of a reference example file (its module-level
    code needs the compiled optimizer bindings, which are not built here)."""
    tree = ast.parse(path.read_text())
    keep = [n for n in tree.body if isinstance(n, ast.FunctionDef) and n.name in names]
    ns = {"sf": sf, "T": __import__("symforce.typing", fromlist=["typing"])}
    exec(compile(ast.Module(body=keep, type_ignores=[]), str(path), "exec"), ns)
    return {n: ns[n] for n in names}


_ex = REF / "symforce" / "examples"
_r2d = load_functions(_ex / "robot_2d_localization" / "robot_2d_localization.py",
                      ["bearing_residual", "odometry_residual"])
bearing_residual, odometry_residual = _r2d["bearing_residual"], _r2d["odometry_residual"]
snavely_reprojection_residual = load_functions(
    _ex / "bundle_adjustment_in_the_large" / "bundle_adjustment_in_the_large.py",
    ["snavely_reprojection_residual"])["snavely_reprojection_residual"]

OUT = Path(__file__).resolve().parent / "factor_vectors.json"
DIGITS = 60
rng = np.random.Generator(np.random.PCG64(1234))
EPS = 10 * np.finfo(np.float64).eps


def rand_quat() -> list:
    q = rng.normal(size=4)
    q /= np.linalg.norm(q)
    return list(q)


def evaluate(res, args, subs):
    """Residual and tangent Jacobian at `subs`, evaluated with mpmath at DIGITS significant digits
    (inputs converted exactly from their double values)."""
    J = jacobian_helpers.tangent_jacobians(res, args)
    Jfull = sf.Matrix.block_matrix([J]) if len(J) > 1 else J[0]
    syms = list(subs.keys())
    mpmath.mp.dps = DIGITS
    vals = [mpmath.mpf(float(subs[k])) for k in syms]
    # symforce's sign helpers (symforce/internal/symbolic.py: SignNoZero, CopysignNoZero)
    custom = {"SignNoZero": lambda x: 1 if x >= 0 else -1,
              "CopysignNoZero": lambda x, y: abs(x) * (1 if y >= 0 else -1)}
    mods = [custom, "mpmath"]
    fr = sympy.lambdify(syms, sympy.Matrix(res.to_flat_list()), modules=mods)
    Jm = sympy.Matrix([[Jfull[i, j] for j in range(Jfull.shape[1])] for i in range(Jfull.shape[0])])
    fj = sympy.lambdify(syms, Jm, modules=mods)
    R = fr(*vals)
    JJ = fj(*vals)
    r = [float(mpmath.re(R[i])) for i in range(len(res.to_flat_list()))]
    Jv = [[float(mpmath.re(JJ[i, j])) for j in range(Jfull.shape[1])] for i in range(Jfull.shape[0])]
    return r, Jv


def subs_for(obj, values):
    return dict(zip(obj.to_storage(), values))


def pose2_storage(theta, x, y):
    return [math.cos(theta), math.sin(theta), x, y]


vectors = []

# ---- bearing (robot_2d_localization.py:53-61), whitened by a scalar sqrt_info
for k in range(4):
    pose = sf.Pose2.symbolic("pose")
    lm = sf.V2.symbolic("lm")
    angle, eps, w = sf.symbols("angle eps w")
    res = sf.V1(w * bearing_residual(pose, lm, angle, eps))
    st = pose2_storage(rng.uniform(-3, 3), rng.uniform(-5, 5), rng.uniform(-5, 5))
    L = list(rng.uniform(-10, 10, size=2))
    a = float(rng.uniform(-3, 3))
    wt = float(rng.uniform(0.5, 20))
    subs = {**subs_for(pose, st), **subs_for(lm, L), angle: a, eps: EPS, w: wt}
    r, J = evaluate(res, [pose], subs)
    vectors.append(dict(kind=1, key_types=[4], storage=st, consts=L + [a, EPS, wt], residual=r, jacobian=J))

# ---- odometry distance (robot_2d_localization.py:64-70)
for k in range(4):
    pa, pb = sf.Pose2.symbolic("a"), sf.Pose2.symbolic("b")
    dist, eps, w = sf.symbols("dist eps w")
    res = sf.V1(w * odometry_residual(pa, pb, dist, eps))
    sa = pose2_storage(rng.uniform(-3, 3), rng.uniform(-5, 5), rng.uniform(-5, 5))
    sb = pose2_storage(rng.uniform(-3, 3), rng.uniform(-5, 5), rng.uniform(-5, 5))
    d = float(rng.uniform(0.5, 3))
    wt = float(rng.uniform(0.5, 20))
    subs = {**subs_for(pa, sa), **subs_for(pb, sb), dist: d, eps: EPS, w: wt}
    r, J = evaluate(res, [pa, pb], subs)
    vectors.append(dict(kind=2, key_types=[4, 4], storage=sa + sb, consts=[d, EPS, wt], residual=r, jacobian=J))

# ---- Snavely reprojection (bundle_adjustment_in_the_large.py:18-63) with / without the Cauchy
# norm whitening (noise_models.py BarronNoiseModel, alpha = 0, whiten_norm)
for k in range(6):
    cam = sf.Pose3.symbolic("c")
    intr = sf.V3.symbolic("i")
    pt = sf.V3.symbolic("p")
    pix = sf.V2.symbolic("px")
    eps = sf.Symbol("eps")
    e = snavely_reprojection_residual(cam, intr, pt, pix, eps)
    delta = 1.0 if k % 2 == 0 else 0.0
    if delta > 0:
        # alpha_epsilon small enough (and the 60-digit arithmetic wide enough for its cancellation) that the
        # evaluated expression is the alpha -> 0 (Cauchy) limit of the reference's Barron loss
        nm = BarronNoiseModel(alpha=0, scalar_information=1, x_epsilon=eps,
                              delta=sympy.Integer(int(delta)), alpha_epsilon=sympy.Rational(1, 10**25))
        res = nm.whiten_norm(e, epsilon=eps)
    else:
        res = e
    q = rand_quat()
    t = list(rng.uniform(-2, 2, size=3))
    X = list(rng.uniform(-3, 3, size=3))
    # keep the point in front of the camera (pc.z < 0)
    Rm = np.array(sf.Rot3(sf.Quaternion(xyz=sf.V3(q[:3]), w=q[3])).to_rotation_matrix().evalf().to_list(),
                  dtype=float)
    pc = Rm @ np.array(X) + np.array(t)
    t[2] -= pc[2] + float(rng.uniform(5, 15))
    intr_v = [float(rng.uniform(400, 600)), float(rng.normal(0, 1e-2)), float(rng.normal(0, 1e-2))]
    # pixel near the projection plus noise, sometimes an outlier
    pcn = Rm @ np.array(X) + np.array(t)
    uv = pcn[:2] / -pcn[2]
    g = 1 + intr_v[1] * uv.dot(uv) + intr_v[2] * uv.dot(uv) ** 2
    px = list(intr_v[0] * g * uv + rng.normal(0, 3 if k < 4 else 40, size=2))
    subs = {**subs_for(cam, q + t), **subs_for(intr, intr_v), **subs_for(pt, X), **subs_for(pix, px),
            eps: EPS}
    r, J = evaluate(res, [cam, intr, pt], subs)
    vectors.append(dict(kind=3, key_types=[5, 3, 3], storage=q + t + intr_v + X,
                        consts=px + [EPS, delta], residual=r, jacobian=J))

# ---- between / prior Pose3 (codegen/geo_factors_codegen.py:53-86), diagonal sqrt_info
for k in range(4):
    a, b, m = sf.Pose3.symbolic("a"), sf.Pose3.symbolic("b"), sf.Pose3.symbolic("m")
    s = sf.V6.symbolic("s")
    eps = sf.Symbol("eps")
    res = geo_factors_codegen.between_factor(a, b, m, sf.Matrix.diag(s.to_flat_list()), eps)
    sa = rand_quat() + list(rng.uniform(-3, 3, size=3))
    sb = rand_quat() + list(rng.uniform(-3, 3, size=3))
    sm = rand_quat() + list(rng.uniform(-3, 3, size=3))
    sv = list(rng.uniform(1, 20, size=6))
    e_val = 1e-10
    subs = {**subs_for(a, sa), **subs_for(b, sb), **subs_for(m, sm), **dict(zip(s.to_flat_list(), sv)),
            eps: e_val}
    r, J = evaluate(res, [a, b], subs)
    vectors.append(dict(kind=4, key_types=[5, 5], storage=sa + sb, consts=sm + sv + [e_val], residual=r,
                        jacobian=J))
for k in range(4):
    v, p = sf.Pose3.symbolic("v"), sf.Pose3.symbolic("p")
    s = sf.V6.symbolic("s")
    eps = sf.Symbol("eps")
    res = geo_factors_codegen.prior_factor(v, p, sf.Matrix.diag(s.to_flat_list()), eps)
    sv_ = rand_quat() + list(rng.uniform(-3, 3, size=3))
    sp = rand_quat() + list(rng.uniform(-3, 3, size=3))
    sq = list(rng.uniform(1, 20, size=6))
    e_val = 1e-10
    subs = {**subs_for(v, sv_), **subs_for(p, sp), **dict(zip(s.to_flat_list(), sq)), eps: e_val}
    r, J = evaluate(res, [v], subs)
    vectors.append(dict(kind=5, key_types=[5], storage=sv_, consts=sp + sq + [e_val], residual=r, jacobian=J))

# ---- kinds the library generates from symbolic definitions: between / prior Rot3
# (geo_factors_codegen.py:53-86 with sf.Rot3), diagonal sqrt_info
for k in range(3):
    a, b, m = sf.Rot3.symbolic("a"), sf.Rot3.symbolic("b"), sf.Rot3.symbolic("m")
    s = sf.V3.symbolic("s")
    eps = sf.Symbol("eps")
    res = geo_factors_codegen.between_factor(a, b, m, sf.Matrix.diag(s.to_flat_list()), eps)
    sa, sb, sm = rand_quat(), rand_quat(), rand_quat()
    sv = list(rng.uniform(1, 20, size=3))
    e_val = 1e-10
    subs = {**subs_for(a, sa), **subs_for(b, sb), **subs_for(m, sm), **dict(zip(s.to_flat_list(), sv)),
            eps: e_val}
    r, J = evaluate(res, [a, b], subs)
    vectors.append(dict(kind=8, key_types=[6, 6], storage=sa + sb, consts=sm + sv + [e_val], residual=r,
                        jacobian=J))
for k in range(3):
    v, p = sf.Rot3.symbolic("v"), sf.Rot3.symbolic("p")
    s = sf.V3.symbolic("s")
    eps = sf.Symbol("eps")
    res = geo_factors_codegen.prior_factor(v, p, sf.Matrix.diag(s.to_flat_list()), eps)
    sv_, sp_ = rand_quat(), rand_quat()
    sq = list(rng.uniform(1, 20, size=3))
    e_val = 1e-10
    subs = {**subs_for(v, sv_), **subs_for(p, sp_), **dict(zip(s.to_flat_list(), sq)), eps: e_val}
    r, J = evaluate(res, [v], subs)
    vectors.append(dict(kind=7, key_types=[6], storage=sv_, consts=sp_ + sq + [e_val], residual=r, jacobian=J))

# ---- the GNC test factor (test/symforce_gnc_codegen_test.py:24-31): Barron whitening of x - y with
# alpha from the convexity parameter mu (noise_models.py BarronNoiseModel.compute_alpha_from_mu)
for mu_val in (0.0, 0.33, 0.66, 0.99):
    x, y = sf.V5.symbolic("x"), sf.V5.symbolic("y")
    mu, eps = sf.symbols("mu eps")
    alpha = BarronNoiseModel.compute_alpha_from_mu(mu, eps)
    nm = BarronNoiseModel(alpha=alpha, delta=1, scalar_information=1, x_epsilon=eps)
    res = nm.whiten(x - y)
    xv = list(rng.normal(0, 1, size=5))
    yv = list(rng.normal(0, 1, size=5) + (10.0 if mu_val > 0.5 else 0.0))
    e_val = 2.220446049250313e-15
    subs = {**subs_for(x, xv), **subs_for(y, yv), mu: mu_val, eps: e_val}
    r, J = evaluate(res, [x], subs)
    vectors.append(dict(kind=9, key_types=[8], storage=xv, consts=yv + [mu_val, e_val], residual=r,
                        jacobian=J))

OUT.write_text(json.dumps(dict(generator="tests/golden/make_symforce_factor_vectors.py",
                               digits=DIGITS, vectors=vectors), indent=1))
print(f"wrote {len(vectors)} vectors to {OUT}")
