"""Typed-factor code generation: from a residual written in sympy to the device functor the
linearization kernel evaluates.

The reference generates each factor's residual and tangent-space Jacobian from a symbolic function
(symforce/codegen/codegen.py, `with_linearization`; the Jacobians by
symforce/jacobian_helpers.py:tangent_jacobians, i.e. d r(x ⊞ δ) / dδ at δ = 0).  This module does
the same for the key types the library knows, with plain sympy, and emits C++ that compiles for the
host and for sm_103a:

- the key count, constant count, residual and tangent dimensions and the per-slot tangent /
  storage sizes as constants of the struct (the fields of `FactorTraits<KIND>` in factor_math.cuh);
- `template <typename T> static void Run(const double* const* x, const double* c, double* r, T* J)`:
  the residual in FP64 and the row-major RD x TD tangent Jacobian in T, common subexpressions
  shared (the calling convention of `FactorEval<KIND, T>::Run`).

Retractions follow the reference's Lie group ops: Pose3 storage [qx, qy, qz, qw, x, y, z], tangent
[ω, δt] with q ← q ⊗ exp(ω), t ← t + δt (gen/cpp/sym/ops/pose3/lie_group_ops.cc:69-102); Pose2
storage [re, im, x, y], tangent [θ, δt] with the rotation multiplied by exp(iθ) and t ← t + δt
(gen/cpp/sym/ops/pose2/lie_group_ops.cc:58-82); vectors add.  A generated functor becomes a factor
kind by adding its id to include/sfgpu.h, a `FactorTraits` / `FactorEval` specialization that
forwards to the generated struct, and a case in `LaunchLinearize` (kernels_lin.cu).

    python -m symforce_gb300.codegen   # prints the generated range factor as an example
"""

from __future__ import annotations

from pathlib import Path
from typing import Callable, List, Sequence

import sympy as sp

from . import _cabi as A


def _key_symbols(k: int, key_type: int):
    sdim = A.KEY_DIMS[key_type][0]
    return sp.Matrix(sp.symbols(f"x{k}_0:{sdim}", real=True))


def _retract_first_order(key_type: int, x: sp.Matrix, d: sp.Matrix) -> sp.Matrix:
    """x ⊞ δ to first order in δ (enough for the Jacobian at δ = 0)."""
    if key_type == A.SFG_KEY_ROT3:
        qx, qy, qz, qw = x[0], x[1], x[2], x[3]
        hx, hy, hz = d[0] / 2, d[1] / 2, d[2] / 2
        return sp.Matrix([qw * hx + qx + qy * hz - qz * hy,
                          qw * hy - qx * hz + qy + qz * hx,
                          qw * hz + qx * hy - qy * hx + qz,
                          qw - qx * hx - qy * hy - qz * hz])
    if key_type == A.SFG_KEY_POSE3:
        qx, qy, qz, qw = x[0], x[1], x[2], x[3]
        # q ⊗ [ω / 2, 1]
        hx, hy, hz = d[0] / 2, d[1] / 2, d[2] / 2
        q = sp.Matrix([qw * hx + qx + qy * hz - qz * hy,
                       qw * hy - qx * hz + qy + qz * hx,
                       qw * hz + qx * hy - qy * hx + qz,
                       qw - qx * hx - qy * hy - qz * hz])
        return sp.Matrix.vstack(q, sp.Matrix([x[4] + d[3], x[5] + d[4], x[6] + d[5]]))
    if key_type == A.SFG_KEY_POSE2:
        re, im = x[0], x[1]
        # (re + i im)(1 + i θ)
        return sp.Matrix([re - im * d[0], im + re * d[0], x[2] + d[1], x[3] + d[2]])
    return x + d


def factor_source(name: str, key_types: Sequence[int], num_consts: int,
                  residual: Callable[[List[sp.Matrix], List[sp.Symbol]], sp.Matrix]) -> str:
    """C++ source of struct `name` (traits + templated Run) for `residual(keys, consts)`, where
    `keys[k]` is the storage vector of key slot k and `consts` the factor's constants."""
    xs = [_key_symbols(k, t) for k, t in enumerate(key_types)]
    cs = list(sp.symbols(f"c0:{num_consts}", real=True)) if num_consts else []
    r = sp.Matrix(residual(xs, cs))
    rd = r.shape[0]
    tdims = [A.KEY_DIMS[t][1] for t in key_types]
    cols = []
    for k, t in enumerate(key_types):
        d = sp.Matrix(sp.symbols(f"d{k}_0:{tdims[k]}", real=True))
        xp = _retract_first_order(t, xs[k], d)
        rk = r.subs({xs[k][i]: xp[i] for i in range(xs[k].shape[0])}, simultaneous=True)
        jk = rk.jacobian(d).subs({di: 0 for di in d})
        cols.append(jk)
    J = sp.Matrix.hstack(*cols)
    td = J.shape[1]
    exprs = list(r) + list(J)
    temps, reduced = sp.cse(exprs, symbols=sp.numbered_symbols("t"), optimizations="basic")
    # storage and constant symbols map to the Run arguments
    names = {}
    for k, x in enumerate(xs):
        for i, s in enumerate(x):
            names[s] = sp.Symbol(f"x[{k}][{i}]")
    for i, s in enumerate(cs):
        names[s] = sp.Symbol(f"c[{i}]")

    def code(e):
        return sp.ccode(e.xreplace(names), standard="c99")

    kt = ", ".join(str(v) for v in tdims)
    ks = ", ".join(str(A.KEY_DIMS[t][0]) for t in key_types)

    def slot_fn(fn, dims):
        expr = "0"
        for k in reversed(range(len(dims))):
            expr = f"(k == {k} ? {dims[k]} : {expr})"
        return f"  static constexpr SFG_HD int {fn}(int k) {{ return {expr}; }}"

    lines = [
        f"// Generated by symforce_gb300.codegen from a sympy residual: {rd} residual rows, tangent",
        f"// dimension {td}; residual in FP64, Jacobian (row-major) in T.",
        f"struct {name} {{",
        f"  static constexpr int NK = {len(key_types)}, NC = {num_consts}, RD = {rd}, TD = {td}, MK = 0;",
        f"  static constexpr int kTangent[NK] = {{{kt}}};",
        f"  static constexpr int kStorage[NK] = {{{ks}}};",
        slot_fn("KT", tdims),
        slot_fn("KS", [A.KEY_DIMS[t][0] for t in key_types]),
        "  template <typename T>",
        "  static SFG_HD void Run(const double* const* x, const double* c, double* r, T* J) {",
    ]
    for s, e in temps:
        lines.append(f"    const double {s} = {code(e)};")
    for i in range(rd):
        lines.append(f"    r[{i}] = {code(reduced[i])};")
    for i in range(rd):
        for j in range(td):
            lines.append(f"    J[{i * td + j}] = T({code(reduced[rd + i * td + j])});")
    lines += ["  }", "};", ""]
    return "\n".join(lines)


def range_pose3_residual(keys, c):
    """w (sqrt(|t - l|^2 + eps) - range): the range factor of the batched 3D localization
    workloads (consts: landmark l (3), range, w, eps)."""
    t = keys[0][4:7, 0]
    d = t - sp.Matrix(c[0:3])
    return sp.Matrix([c[4] * (sp.sqrt(d.dot(d) + c[5]) - c[3])])


def write_generated(csrc: Path | None = None) -> tuple[Path, Path]:
    """Write generated_factors.cuh (device functors) and generated_factor_specs.h (the kinds'
    dimensions, for host code) from the definitions in factor_defs.GENERATED."""
    from . import factor_defs
    csrc = csrc or Path(__file__).resolve().parent / "csrc"
    head = ["// Generated by `python -m symforce_gb300.codegen --write` from the sympy residuals in",
            "// symforce_gb300/factor_defs.py; do not edit by hand."]
    dev = head + ["#pragma once", "", "namespace sfg {", ""]
    specs = head + ["#pragma once", "",
                    "// X(kind, num_keys, num_consts, residual_dim, key type 0, key type 1, key type 2, struct)",
                    "#define SFG_GENERATED_FACTORS(X) \\"]
    rows = []
    for fd in factor_defs.GENERATED:
        dev.append(f"// {fd.enum}: {fd.doc}")
        dev.append(factor_source(fd.name, list(fd.key_types), fd.num_consts, fd.residual))
        kts = list(fd.key_types) + [0] * (3 - len(fd.key_types))
        xs = [_key_symbols(k, t) for k, t in enumerate(fd.key_types)]
        cs = list(sp.symbols(f"c0:{fd.num_consts}", real=True))
        rd = sp.Matrix(fd.residual(xs, cs)).shape[0]
        rows.append(f"  X({fd.enum}, {len(fd.key_types)}, {fd.num_consts}, {rd}, {kts[0]}, {kts[1]}, {kts[2]}, "
                    f"{fd.name})")
    dev += ["}  // namespace sfg", ""]
    specs += [r + " \\" for r in rows[:-1]] + [rows[-1], ""]
    p_dev, p_spec = csrc / "generated_factors.cuh", csrc / "generated_factor_specs.h"
    p_dev.write_text("\n".join(dev))
    p_spec.write_text("\n".join(specs))
    return p_dev, p_spec


if __name__ == "__main__":
    import sys
    if "--write" in sys.argv:
        for p in write_generated():
            print("wrote", p)
    else:
        print(factor_source("GenRangePose3", [A.SFG_KEY_POSE3], 6, range_pose3_residual))
