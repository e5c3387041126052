"""ctypes loader for the CPU oracle (oracle/_build/liboracle.so).

Test infrastructure: the oracle is the checker, never the thing measured or shipped.
"""

from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

from symforce_gb300 import _cabi as A

ROOT = Path(__file__).resolve().parents[1]
ORACLE_DIR = ROOT / "oracle"
LIB_PATH = ORACLE_DIR / "_build" / "liboracle.so"
# timed CPU baselines (bench.py): the same source at -O3, and at -O3 -ffast-math
VARIANTS = {"o2": "liboracle.so", "o3": "liboracle_o3.so", "o3_fast": "liboracle_o3_fast.so"}

_lib = None


def use_variant(name: str) -> None:
    """Load another build of the oracle (VARIANTS) for the calls that follow (bench timing only)."""
    global _lib
    path = ORACLE_DIR / "_build" / VARIANTS[name]
    if not path.exists():
        build()
    L = C.CDLL(str(path))
    L.orc_last_error.restype = C.c_char_p
    _lib = L


def build() -> Path:
    subprocess.run(["make", "-s", "-j3", "-C", str(ORACLE_DIR)], check=True)
    return LIB_PATH


def lib() -> C.CDLL:
    """The oracle library; SFG_ORACLE_VARIANT (o2 | o3 | o3_fast) picks the build (default o2, the
    parity reference)."""
    global _lib
    if _lib is None:
        path = ORACLE_DIR / "_build" / VARIANTS[os.environ.get("SFG_ORACLE_VARIANT", "o2")]
        if not path.exists() or os.environ.get("SFG_REBUILD_ORACLE"):
            build()
        L = C.CDLL(str(path))
        L.orc_last_error.restype = C.c_char_p
        _lib = L
    return _lib


def _check(rc: int) -> None:
    if rc != 0:
        raise RuntimeError("oracle: " + lib().orc_last_error().decode())


def factor_linearize(kind: int, key_types, storage, consts, epsilon=A.DEFAULT_EPSILON):
    nk, nc, rdim, _ = A.FACTOR_DIMS[kind]
    kt = np.ascontiguousarray(key_types, dtype=np.int32)
    st = np.ascontiguousarray(storage, dtype=np.float64)
    cs = np.ascontiguousarray(consts, dtype=np.float64)
    tdim = sum(A.KEY_DIMS[int(t)][1] for t in kt)
    res = np.zeros(rdim)
    J = np.zeros((rdim, tdim))
    _check(lib().orc_factor_linearize(C.c_int32(kind), A.iptr(kt), A.dptr(st), A.dptr(cs),
                                      C.c_double(epsilon), A.dptr(res), A.dptr(J)))
    return res, J


def linearize(problem: A.ProblemArrays, values=None, epsilon=A.DEFAULT_EPSILON):
    pc = problem.to_c()
    v = problem.values if values is None else np.ascontiguousarray(values, dtype=np.float64)
    M, N, nnz = C.c_int64(), C.c_int64(), C.c_int64()
    null = C.POINTER(C.c_double)()
    _check(lib().orc_linearize(C.byref(pc), A.dptr(v), C.c_double(epsilon), C.byref(M), C.byref(N),
                               C.byref(nnz), null, null, C.POINTER(C.c_int64)(),
                               C.POINTER(C.c_int32)(), null))
    res = np.zeros(M.value)
    rhs = np.zeros(N.value)
    colptr = np.zeros(N.value + 1, dtype=np.int64)
    rowidx = np.zeros(nnz.value, dtype=np.int32)
    hv = np.zeros(nnz.value)
    _check(lib().orc_linearize(C.byref(pc), A.dptr(v), C.c_double(epsilon), C.byref(M), C.byref(N),
                               C.byref(nnz), A.dptr(res), A.dptr(rhs), A.lptr(colptr),
                               A.iptr(rowidx), A.dptr(hv)))
    return dict(residual=res, rhs=rhs, colptr=colptr, rowidx=rowidx, hvals=hv)


def optimize(problem: A.ProblemArrays, params=None, num_iterations=-1, epsilon=A.DEFAULT_EPSILON,
             linear_solver=A.SFG_LINEAR_SOLVER_SPARSE_LDLT, ordering=A.SFG_ORDERING_MIN_DEGREE,
             values=None):
    params = params or A.default_optimizer_params()
    pc = problem.to_c()
    v = problem.values if values is None else np.ascontiguousarray(values, dtype=np.float64)
    out = np.zeros_like(v)
    cap = max(params.iterations, num_iterations) + 2
    iters = (A.IterationC * cap)()
    n, best, status, reason = C.c_int32(), C.c_int32(), C.c_int32(), C.c_int32()
    secs = np.zeros(3)
    _check(lib().orc_optimize(C.byref(pc), A.dptr(v), C.byref(params), C.c_int32(num_iterations),
                              C.c_double(epsilon), C.c_int32(linear_solver), C.c_int32(ordering),
                              A.dptr(out), iters, C.c_int32(cap), C.byref(n), C.byref(best),
                              C.byref(status), C.byref(reason), A.dptr(secs)))
    recs = [iters[i] for i in range(n.value)]
    return dict(values=out, iterations=recs, best_index=best.value, status=status.value,
                failure_reason=reason.value, seconds=float(secs[0]),
                seconds_linearize=float(secs[1]), seconds_solve=float(secs[2]))


def ldlt_solve(n, colptr, rowidx, vals, b, ordering=A.SFG_ORDERING_MIN_DEGREE, order=None):
    colptr = np.ascontiguousarray(colptr, dtype=np.int64)
    rowidx = np.ascontiguousarray(rowidx, dtype=np.int32)
    vals = np.ascontiguousarray(vals, dtype=np.float64)
    b = np.ascontiguousarray(b, dtype=np.float64)
    x = np.zeros(n)
    D = np.zeros(n)
    perm = np.zeros(n, dtype=np.int32)
    ordp = A.iptr(np.ascontiguousarray(order, dtype=np.int32)) if order is not None else C.POINTER(C.c_int32)()
    _check(lib().orc_ldlt_solve(C.c_int64(n), A.lptr(colptr), A.iptr(rowidx), A.dptr(vals),
                                C.c_int32(ordering), ordp, A.dptr(b), A.dptr(x), A.dptr(D),
                                A.iptr(perm)))
    return x, D, perm


def schur_solve(n, colptr, rowidx, vals, c_dim, b):
    colptr = np.ascontiguousarray(colptr, dtype=np.int64)
    rowidx = np.ascontiguousarray(rowidx, dtype=np.int32)
    vals = np.ascontiguousarray(vals, dtype=np.float64)
    b = np.ascontiguousarray(b, dtype=np.float64)
    x = np.zeros(n)
    _check(lib().orc_schur_solve(C.c_int64(n), A.lptr(colptr), A.iptr(rowidx), A.dptr(vals),
                                 C.c_int64(c_dim), A.dptr(b), A.dptr(x)))
    return x


def retract(key_type, storage, delta, epsilon=A.DEFAULT_EPSILON):
    sd, _ = A.KEY_DIMS[key_type]
    out = np.zeros(sd)
    st = np.ascontiguousarray(storage, dtype=np.float64)
    d = np.ascontiguousarray(delta, dtype=np.float64)
    _check(lib().orc_retract(C.c_int32(key_type), A.dptr(st), A.dptr(d), C.c_double(epsilon),
                             A.dptr(out)))
    return out


def pose_smoothing_initial_values(num_keys=10, epsilon=A.DEFAULT_EPSILON):
    out = np.zeros(7 * num_keys)
    _check(lib().orc_pose_smoothing_initial_values(C.c_int32(num_keys), C.c_double(epsilon),
                                                   A.dptr(out)))
    return out


def optimize_carry(problem: A.ProblemArrays, params, num_iterations, carry, continue_state,
                   epsilon=A.DEFAULT_EPSILON, values=None):
    """orc_optimize_carry: a fresh run (continue_state False) or OptimizeContinue from `carry`
    ([lambda, nu, iteration], updated in place)."""
    pc = problem.to_c()
    v = problem.values if values is None else np.ascontiguousarray(values, dtype=np.float64)
    out = np.zeros_like(v)
    cap = num_iterations + 2
    iters = (A.IterationC * cap)()
    n, best, status, reason = C.c_int32(), C.c_int32(), C.c_int32(), C.c_int32()
    _check(lib().orc_optimize_carry(C.byref(pc), A.dptr(v), C.byref(params), C.c_int32(num_iterations),
                                    C.c_double(epsilon), C.c_int32(A.SFG_LINEAR_SOLVER_SPARSE_LDLT),
                                    C.c_int32(A.SFG_ORDERING_MIN_DEGREE), A.dptr(out), iters,
                                    C.c_int32(cap), C.byref(n), C.byref(best), C.byref(status),
                                    C.byref(reason), A.dptr(carry), C.c_int32(1 if continue_state else 0)))
    return dict(values=out, iterations=[iters[i] for i in range(n.value)], best_index=best.value,
                status=status.value, failure_reason=reason.value)


def gnc_optimize(problem: A.ProblemArrays, params, gnc_params, mu_slots, epsilon=A.DEFAULT_EPSILON,
                 num_iterations=-1):
    """The GNC schedule (symforce_gb300.gnc.run_gnc) over the oracle's LM loop."""
    from symforce_gb300 import gnc
    state = dict(values=problem.values.copy(), carry=np.zeros(3))
    consts = {b: np.array(problem.batches[b].consts, dtype=np.float64, copy=True) for b, _ in mu_slots}

    def set_mu(mu):
        for b, ci in mu_slots:
            consts[b][:, ci] = mu
            problem.batches[b].consts = consts[b]

    def run(p, n, cont, relax):
        if relax:
            state["carry"][0] = min(state["carry"][0], p.initial_lambda)
            state["carry"][1] = p.dynamic_lambda_update_beta
        r = optimize_carry(problem, p, n, state["carry"], cont, epsilon=epsilon, values=state["values"])
        state["values"] = r["values"]
        return r["iterations"], r["best_index"], r["status"], r["failure_reason"]

    r = gnc.run_gnc(params, gnc_params, set_mu, run, num_iterations)
    r["values"] = state["values"]
    return r


def mt19937_normal_vectors(seed, num_vectors, dim):
    out = np.zeros((num_vectors, dim))
    _check(lib().orc_mt19937_normal_vectors(C.c_uint32(seed), C.c_int32(num_vectors), C.c_int32(dim),
                                            A.dptr(out)))
    return out


def rot3_smoothing_initial_values(num_keys=10, epsilon=A.DEFAULT_EPSILON):
    out = np.zeros(4 * num_keys)
    _check(lib().orc_rot3_smoothing_initial_values(C.c_int32(num_keys), C.c_double(epsilon), A.dptr(out)))
    return out
