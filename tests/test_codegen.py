"""Typed-factor code generation (symforce_gb300/codegen.py): functors generated from sympy
residuals compile with g++ beside the library's hand-written factor math (factor_math.cuh) and give
the same residuals and tangent Jacobians on random inputs — so the generator's retractions and
Jacobian convention are the library's (and the reference's: symforce/jacobian_helpers.py)."""

from __future__ import annotations

import ctypes as C
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

sp = pytest.importorskip("sympy")

from symforce_gb300 import _cabi as A  # noqa: E402
from symforce_gb300 import codegen  # noqa: E402

ROOT = Path(__file__).resolve().parents[1]
CSRC = ROOT / "symforce_gb300" / "csrc"


def _qmul(p, q):
    """Quaternion product p ⊗ q, storage [x, y, z, w]."""
    px, py, pz, pw = p
    qx, qy, qz, qw = q
    return [pw * qx + px * qw + py * qz - pz * qy,
            pw * qy - px * qz + py * qw + pz * qx,
            pw * qz + px * qy - py * qx + pz * qw,
            pw * qw - px * qx - py * qy - pz * qz]


def prior_pose3_residual(keys, c):
    """diag(s) local_coordinates(prior, x) (symforce/codegen/geo_factors_codegen.py:74-86), without
    the eps clamp of the rotation log (random inputs stay away from it); consts: prior (7), s (6),
    eps."""
    x = keys[0]
    qe = _qmul([-c[0], -c[1], -c[2], c[3]], [x[0], x[1], x[2], x[3]])
    w = qe[3]
    sgn = sp.Piecewise((1, w >= 0), (-1, True))
    aw = sp.Piecewise((w, w >= 0), (-w, True))
    k = 2 * sgn * sp.acos(aw) / sp.sqrt(1 - aw * aw)
    rot = [c[7 + i] * k * qe[i] for i in range(3)]
    trans = [c[10 + i] * (x[4 + i] - c[4 + i]) for i in range(3)]
    return sp.Matrix(rot + trans)


def odometry_pose2_residual(keys, c):
    """w (sqrt(|t_b - t_a|^2 + eps) - distance) between two Pose2 (consts: distance, eps, w)."""
    a, b = keys
    dx, dy = b[2] - a[2], b[3] - a[3]
    return sp.Matrix([c[2] * (sp.sqrt(dx * dx + dy * dy + c[1]) - c[0])])


def snavely_residual(keys, c):
    """The bundle-adjustment reprojection with Cauchy whitening (symforce/examples/
    bundle_adjustment_in_the_large/bundle_adjustment_in_the_large.py:18-63, symforce/opt/
    noise_models.py:318-428 at alpha -> 0); consts: pixel (2), eps, delta."""
    cam, intr, X = keys
    qx, qy, qz, qw = cam[0], cam[1], cam[2], cam[3]
    R = sp.Matrix([[1 - 2 * (qy * qy + qz * qz), 2 * (qx * qy - qz * qw), 2 * (qx * qz + qy * qw)],
                   [2 * (qx * qy + qz * qw), 1 - 2 * (qx * qx + qz * qz), 2 * (qy * qz - qx * qw)],
                   [2 * (qx * qz - qy * qw), 2 * (qy * qz + qx * qw), 1 - 2 * (qx * qx + qy * qy)]])
    pc = R * sp.Matrix(X[0:3, 0]) + sp.Matrix(cam[4:7, 0])
    u, v = -pc[0] / pc[2], -pc[1] / pc[2]
    r2 = u * u + v * v
    g = 1 + intr[1] * r2 + intr[2] * r2 * r2
    e0, e1 = intr[0] * g * u - c[0], intr[0] * g * v - c[1]
    n2 = e0 * e0 + e1 * e1 + c[2]
    rho2 = 2 * c[3] ** 2 * sp.log(1 + n2 / (2 * c[3] ** 2))
    s = sp.sqrt(rho2) / sp.sqrt(n2)
    return sp.Matrix([s * e0, s * e1])


CASES = {
    # name: (kind, key types, consts, residual)
    "range": (A.SFG_FACTOR_RANGE_POSE3, [A.SFG_KEY_POSE3], 6, codegen.range_pose3_residual),
    "prior": (A.SFG_FACTOR_PRIOR_POSE3, [A.SFG_KEY_POSE3], 14, prior_pose3_residual),
    "odometry": (A.SFG_FACTOR_ODOMETRY_POSE2, [A.SFG_KEY_POSE2] * 2, 3, odometry_pose2_residual),
    "snavely": (A.SFG_FACTOR_SNAVELY_REPROJECTION, [A.SFG_KEY_POSE3, A.SFG_KEY_VEC3, A.SFG_KEY_VEC3], 4,
                snavely_residual),
}


@pytest.fixture(scope="module")
def lib(tmp_path_factory):
    gxx = shutil.which("g++")
    cuda_inc = Path("/usr/local/cuda/include")
    if gxx is None or not (cuda_inc / "cuda_runtime.h").exists():
        pytest.skip("g++ or the CUDA headers are not available")
    src = ['#include <cmath>', '#include "factor_math.cuh"', "namespace gen {"]
    for name, (_, kt, nc, fn) in CASES.items():
        src.append(codegen.factor_source(f"Gen_{name}", kt, nc, fn))
    src.append("}  // namespace gen")
    src.append('extern "C" {')
    for name, (kind, kt, _, _) in CASES.items():
        nk = len(kt)
        args = ", ".join(f"const double* x{k}" for k in range(nk))
        xs = ", ".join(f"x{k}" for k in range(nk))
        src.append(f"void gen_{name}({args}, const double* c, double* r, double* J) "
                   f"{{ const double* xp[{nk}] = {{{xs}}}; gen::Gen_{name}::Run<double>(xp, c, r, J); }}")
        src.append(f"void ref_{name}({args}, const double* c, double* r, double* J) "
                   f"{{ const double* xp[3] = {{{xs}}}; sfg::FactorEval<{kind}, double>::Run(xp, c, r, J); }}")
    src.append("}")
    d = tmp_path_factory.mktemp("codegen")
    (d / "gen.cpp").write_text("\n".join(src))
    out = d / "libgen.so"
    subprocess.run([gxx, "-O1", "-std=c++17", "-shared", "-fPIC", f"-I{cuda_inc}", f"-I{ROOT / 'include'}",
                    f"-I{CSRC}", str(d / "gen.cpp"), "-o", str(out)], check=True)
    return C.CDLL(str(out))


def _quat(rng):
    q = rng.normal(size=4)
    q /= np.linalg.norm(q)
    return q if q[3] > 0 else -q


def _inputs(name, rng):
    if name == "range":
        x = [np.concatenate([_quat(rng), rng.normal(size=3) * 5])]
        c = np.concatenate([rng.normal(size=3) * 5, [abs(rng.normal()) * 3, 1 / 0.1, 1e-9]])
    elif name == "prior":
        x0 = np.concatenate([_quat(rng), rng.normal(size=3)])
        dq = np.concatenate([rng.normal(size=3) * 0.2, [1.0]])
        dq /= np.linalg.norm(dq)
        prior_q = np.array(_qmul(list(x0[:4]), list(dq)), dtype=float)
        c = np.concatenate([prior_q, x0[4:] + rng.normal(size=3) * 0.1, 1 / (0.05 + rng.random(6)), [1e-9]])
        x = [x0]
    elif name == "snavely":
        q = _quat(rng)
        X = rng.uniform(-5, 5, size=3)
        qx, qy, qz, qw = q
        R = np.array([[1 - 2 * (qy * qy + qz * qz), 2 * (qx * qy - qz * qw), 2 * (qx * qz + qy * qw)],
                      [2 * (qx * qy + qz * qw), 1 - 2 * (qx * qx + qz * qz), 2 * (qy * qz - qx * qw)],
                      [2 * (qx * qz - qy * qw), 2 * (qy * qz + qx * qw), 1 - 2 * (qx * qx + qy * qy)]])
        t = -R @ X + np.array([rng.normal(), rng.normal(), -20.0])  # the point 20 m in front
        intr = np.array([rng.uniform(400, 600), rng.normal() * 1e-3, rng.normal() * 1e-3])
        pc = R @ X + t
        uv = -pc[:2] / pc[2]
        g = 1 + intr[1] * uv @ uv + intr[2] * (uv @ uv) ** 2
        pix = intr[0] * g * uv + rng.normal(size=2) * 3
        x = [np.concatenate([q, t]), intr, X]
        c = np.array([pix[0], pix[1], 1e-9, 1.0])
    else:
        x = []
        for _ in range(2):
            th = rng.uniform(-np.pi, np.pi)
            x.append(np.array([np.cos(th), np.sin(th), *(rng.normal(size=2) * 3)]))
        c = np.array([abs(rng.normal()) + 0.5, 1e-9, 1 / 0.1])
    return x, c


@pytest.mark.parametrize("name", list(CASES))
def test_generated_functor_matches_library_factor(lib, name):
    kind, kt, nc, _ = CASES[name]
    rd = A.FACTOR_DIMS[kind][2]
    td = sum(A.KEY_DIMS[t][1] for t in kt)
    rng = np.random.default_rng(11)
    ptr = lambda a: a.ctypes.data_as(C.c_void_p)  # noqa: E731
    for _ in range(20):
        x, c = _inputs(name, rng)
        assert c.size == nc
        out = {}
        for which in ("gen", "ref"):
            r, J = np.zeros(rd), np.zeros(rd * td)
            getattr(lib, f"{which}_{name}")(*[ptr(np.ascontiguousarray(v)) for v in x], ptr(c), ptr(r), ptr(J))
            out[which] = (r, J)
        np.testing.assert_allclose(out["gen"][0], out["ref"][0], rtol=1e-10, atol=1e-12)
        np.testing.assert_allclose(out["gen"][1], out["ref"][1], rtol=1e-8, atol=1e-9)


# ---- the generated factor kinds the library registers (symforce_gb300/factor_defs.py) ----------

def test_committed_generated_headers_are_current(tmp_path):
    """generated_factors.cuh / generated_factor_specs.h are what the generator writes from
    factor_defs.py today."""
    p_dev, p_spec = codegen.write_generated(tmp_path)
    assert p_dev.read_text() == (CSRC / "generated_factors.cuh").read_text()
    assert p_spec.read_text() == (CSRC / "generated_factor_specs.h").read_text()


@pytest.fixture(scope="module")
def genlib(tmp_path_factory):
    gxx = shutil.which("g++")
    cuda_inc = Path("/usr/local/cuda/include")
    if gxx is None or not (cuda_inc / "cuda_runtime.h").exists():
        pytest.skip("g++ or the CUDA headers are not available")
    src = ['#include <cmath>', '#include "factor_math.cuh"', 'extern "C" {']
    from symforce_gb300 import factor_defs
    for fd in factor_defs.GENERATED:
        nk = len(fd.key_types)
        src.append(f"void eval_{fd.kind}(const double* const* x, const double* c, double* r, double* J) "
                   f"{{ sfg::FactorEval<{fd.kind}, double>::Run(x, c, r, J); }}")
    src.append("}")
    d = tmp_path_factory.mktemp("genkinds")
    (d / "gen.cpp").write_text("\n".join(src))
    out = d / "libgenkinds.so"
    subprocess.run([gxx, "-O1", "-std=c++17", "-shared", "-fPIC", f"-I{cuda_inc}", f"-I{ROOT / 'include'}",
                    f"-I{CSRC}", str(d / "gen.cpp"), "-o", str(out)], check=True)
    return C.CDLL(str(out))


def _golden_generated():
    import json
    from symforce_gb300 import factor_defs
    kinds = {fd.kind for fd in factor_defs.GENERATED}
    vecs = json.loads((ROOT / "tests" / "golden" / "factor_vectors.json").read_text())["vectors"]
    return [v for v in vecs if v["kind"] in kinds]


@pytest.mark.parametrize("vec", _golden_generated(), ids=lambda v: f"kind{v['kind']}")
def test_generated_kind_matches_symforce_symbolic(genlib, vec):
    """The registered generated kinds (compiled here with g++) against the golden vectors evaluated
    from the reference's own symbolic definitions."""
    kind = vec["kind"]
    nk, _, rd, kt = A.FACTOR_DIMS[kind]
    td = sum(A.KEY_DIMS[t][1] for t in kt)
    st = np.array(vec["storage"])
    offs = np.cumsum([0] + [A.KEY_DIMS[t][0] for t in kt])
    keys = [np.ascontiguousarray(st[offs[k]:offs[k + 1]]) for k in range(nk)]
    xp = (C.c_void_p * nk)(*[k.ctypes.data_as(C.c_void_p) for k in keys])
    c = np.array(vec["consts"])
    r, J = np.zeros(rd), np.zeros(rd * td)
    getattr(genlib, f"eval_{kind}")(xp, c.ctypes.data_as(C.c_void_p), r.ctypes.data_as(C.c_void_p),
                                   J.ctypes.data_as(C.c_void_p))
    np.testing.assert_allclose(r, vec["residual"], rtol=1e-10, atol=1e-12)
    Jg = np.array(vec["jacobian"])
    np.testing.assert_allclose(J.reshape(rd, td), Jg, rtol=1e-8, atol=1e-9 * max(1.0, np.abs(Jg).max()))


def test_generated_linear_kinds_against_numpy(genlib):
    """LINEAR_VEC5 / LINEAR_SCALAR2: residual J x + b and Jacobian J."""
    rng = np.random.default_rng(4)
    for kind, rows, cols, kt in [(A.SFG_FACTOR_LINEAR_VEC5, 9, 5, [5]), (A.SFG_FACTOR_LINEAR_SCALAR2, 2, 2, [1, 1])]:
        Jm = rng.normal(size=(rows, cols))
        b = rng.normal(size=rows)
        x = rng.normal(size=cols)
        keys = [np.ascontiguousarray(x)] if len(kt) == 1 else [np.ascontiguousarray(x[:1]), np.ascontiguousarray(x[1:])]
        xp = (C.c_void_p * len(keys))(*[k.ctypes.data_as(C.c_void_p) for k in keys])
        c = np.concatenate([Jm.ravel(), b])
        r, J = np.zeros(rows), np.zeros(rows * cols)
        getattr(genlib, f"eval_{kind}")(xp, c.ctypes.data_as(C.c_void_p), r.ctypes.data_as(C.c_void_p),
                                       J.ctypes.data_as(C.c_void_p))
        np.testing.assert_allclose(r, Jm @ x + b, rtol=1e-13, atol=1e-13)
        np.testing.assert_allclose(J.reshape(rows, cols), Jm, rtol=0, atol=0)
