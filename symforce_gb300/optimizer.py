"""Python mirror of the sym::Optimizer interface over the C ABI of libsfgpu.so.

`Optimizer(params, problem, form)` corresponds to `sym::Optimizer<double>(params, factors, ...)`
(symforce/opt/optimizer.h:86-111) and `optimize()` to `Optimizer::Optimize(values, num_iterations,
populate_best_linearization, stats)` (symforce/opt/optimizer.tcc:79-89): it runs the whole
Levenberg-Marquardt loop on the GPU and returns `OptimizationStats` with the same per-iteration
records, best index, status and failure reason.  `LinearSolver`-concept objects `SparseLdlt` and
`SparseSchur` mirror SparseCholeskySolver / SparseSchurSolver.

There is no CPU fallback: constructing any of these without a CUDA device raises.
"""

from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from . import _build
from . import _cabi as A

_lib = None


class SfgError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"sfgpu error {code}: {msg}")
        self.code = code


def lib() -> C.CDLL:
    """Load (building first if needed) the in-tree libsfgpu.so."""
    global _lib
    if _lib is None:
        path = _build.build()
        L = C.CDLL(str(path))
        L.sfg_last_error.restype = C.c_char_p
        L.sfg_create.argtypes = [C.POINTER(A.ProblemC), C.POINTER(A.FormParams), C.POINTER(C.c_void_p)]
        L.sfg_destroy.argtypes = [C.c_void_p]
        L.sfg_set_values.argtypes = [C.c_void_p, C.POINTER(C.c_double), C.c_int64]
        L.sfg_get_values.argtypes = [C.c_void_p, C.POINTER(C.c_double), C.c_int64]
        L.sfg_optimize.argtypes = [C.c_void_p, C.POINTER(A.OptimizerParams), C.c_int32, C.POINTER(A.StatsC)]
        L.sfg_optimize_continue.argtypes = [C.c_void_p, C.POINTER(A.OptimizerParams), C.c_int32, C.c_int32,
                                            C.POINTER(A.StatsC)]
        L.sfg_set_factor_consts.argtypes = [C.c_void_p, C.c_int32, C.POINTER(C.c_double), C.c_int64]
        L.sfg_linearize.argtypes = [C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_double),
                                    C.POINTER(C.c_double)]
        L.sfg_hessian_lower.argtypes = [C.c_void_p, C.POINTER(C.c_int64), C.POINTER(C.c_int32),
                                        C.POINTER(C.c_int32), C.POINTER(C.c_double)]
        L.sfg_permutation.argtypes = [C.c_void_p, C.POINTER(C.c_int32), C.c_int64]
        L.sfg_fronts.argtypes = [C.c_void_p, C.POINTER(C.c_int32), C.POINTER(C.c_int32), C.POINTER(C.c_int32)]
        L.sfg_time_stage.argtypes = [C.c_void_p, C.c_int32, C.c_int32, C.POINTER(C.c_double),
                                     C.POINTER(C.c_double), C.POINTER(C.c_double)]
        L.sfg_storage_dim.argtypes = [C.c_void_p, C.POINTER(C.c_int64), C.POINTER(C.c_int64),
                                      C.POINTER(C.c_int64)]
        L.sfg_fp64_diag_tiles.argtypes = [C.c_void_p, C.POINTER(C.c_int64)]
        L.sfg_ldlt_create.argtypes = [C.c_int32, C.POINTER(C.c_int32), C.POINTER(C.c_int32), C.c_int32,
                                      C.c_int32, C.POINTER(C.c_void_p)]
        L.sfg_ldlt_factorize.argtypes = [C.c_void_p, C.POINTER(C.c_double)]
        L.sfg_ldlt_solve.argtypes = [C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_double), C.c_int32]
        L.sfg_ldlt_diagonal.argtypes = [C.c_void_p, C.POINTER(C.c_double)]
        L.sfg_ldlt_permutation.argtypes = [C.c_void_p, C.POINTER(C.c_int32)]
        L.sfg_ldlt_destroy.argtypes = [C.c_void_p]
        L.sfg_ldlt_lower.argtypes = [C.c_void_p, C.POINTER(C.c_int64), C.POINTER(C.c_int32),
                                     C.POINTER(C.c_int32), C.POINTER(C.c_double)]
        L.sfg_factor_lower.argtypes = [C.c_void_p, C.POINTER(C.c_int64), C.POINTER(C.c_int32),
                                       C.POINTER(C.c_int32), C.POINTER(C.c_double)]
        L.sfg_schur_create.argtypes = [C.c_int32, C.POINTER(C.c_int32), C.POINTER(C.c_int32), C.c_int32,
                                       C.c_int32, C.POINTER(C.c_void_p)]
        L.sfg_schur_factorize.argtypes = [C.c_void_p, C.POINTER(C.c_double)]
        L.sfg_schur_solve.argtypes = [C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_double), C.c_int32]
        L.sfg_schur_destroy.argtypes = [C.c_void_p]
        L.sfg_get_pcg_stats.argtypes = [C.c_void_p, C.POINTER(A.PcgStatsC)]
        L.sfg_pcg_step_error.argtypes = [C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_int32),
                                         C.POINTER(C.c_double)]
        L.sfg_set_preconditioner_weights.argtypes = [C.c_void_p, C.POINTER(C.c_float), C.c_int64]
        L.sfg_collect_samples.argtypes = [C.c_void_p, C.c_int32]
        L.sfg_get_samples.argtypes = [C.c_void_p, C.POINTER(C.c_float), C.c_int64, C.POINTER(C.c_int64)]
        L.sfg_precond_train.argtypes = [C.POINTER(C.c_float), C.c_int64, C.POINTER(A.TrainParamsC),
                                        C.POINTER(C.c_float), C.POINTER(C.c_float)]
        L.sfg_precond_loss_grad.argtypes = [C.POINTER(C.c_float), C.c_int64, C.POINTER(C.c_float),
                                            C.c_float, C.POINTER(C.c_double), C.POINTER(C.c_float),
                                            C.c_int32]
        L.sfg_precond_infer.argtypes = [C.POINTER(C.c_float), C.c_int64, C.POINTER(C.c_float),
                                        C.POINTER(C.c_float), C.c_int32]
        _lib = L
    return _lib


def _check(rc: int) -> None:
    if rc != 0:
        raise SfgError(rc, lib().sfg_last_error().decode())


@dataclass
class OptimizationStats:
    """optimization_stats_t (lcmtypes/symforce.lcm:302-336) plus per-iteration device times."""

    iterations: list = field(default_factory=list)
    best_index: int = 0
    status: int = 0
    failure_reason: int = 0
    kernel_launches: int = 0
    device_ms: float = 0.0
    best_linearization: dict | None = None       # populate_best_linearization
    linear_solver_ordering: np.ndarray | None = None  # debug_stats
    cholesky_factor_sparsity: dict | None = None  # debug_stats

    @property
    def best_error(self) -> float:
        return self.iterations[self.best_index].new_error


def _lower_csc(fn, handle, n: int, with_values: bool = True) -> dict:
    """Two-phase query of a compressed-column strict-lower factor (sfg_ldlt_lower /
    sfg_factor_lower)."""
    nnz = C.c_int64()
    _check(fn(handle, C.byref(nnz), None, None, None))
    colptr = np.zeros(n + 1, dtype=np.int32)
    rowidx = np.zeros(nnz.value, dtype=np.int32)
    vals = np.zeros(nnz.value) if with_values else None
    _check(fn(handle, C.byref(nnz), A.iptr(colptr), A.iptr(rowidx), A.dptr(vals) if with_values else None))
    out = dict(colptr=colptr, rowidx=rowidx, shape=(n, n))
    if with_values:
        out["values"] = vals
    return out


def csc_lower_to_dense(colptr: np.ndarray, rowidx: np.ndarray, vals: np.ndarray, n: int) -> np.ndarray:
    """The dense lower triangle (upper part zero) of a compressed-column lower matrix."""
    H = np.zeros((n, n))
    cols = np.repeat(np.arange(n), np.diff(np.asarray(colptr, dtype=np.int64)))
    H[np.asarray(rowidx, dtype=np.int64), cols] = vals
    return H


class Optimizer:
    """GPU Levenberg-Marquardt optimizer for one problem structure (create once, optimize many)."""

    def __init__(self, problem: A.ProblemArrays, params: A.OptimizerParams | None = None,
                 form: A.FormParams | None = None, weights: np.ndarray | None = None):
        """`weights`: preconditioner network weights of the learned PCG form (default: the trained
        weights shipped with the package)."""
        self.problem = problem
        self.params = params or A.default_optimizer_params()
        self.form = form or A.default_form_params()
        self._h = C.c_void_p()
        pc = problem.to_c()
        _check(lib().sfg_create(C.byref(pc), C.byref(self.form), C.byref(self._h)))
        S, N, M = C.c_int64(), C.c_int64(), C.c_int64()
        _check(lib().sfg_storage_dim(self._h, C.byref(S), C.byref(N), C.byref(M)))
        self.storage_dim, self.tangent_dim, self.residual_dim = S.value, N.value, M.value
        if self.form.linear_solver == A.SFG_LINEAR_SOLVER_PCG_LEARNED:
            if weights is None:
                from . import learned
                weights = learned.load_weights()
            self.set_preconditioner_weights(weights)

    def set_preconditioner_weights(self, weights: np.ndarray) -> None:
        w = np.ascontiguousarray(weights, dtype=np.float32)
        _check(lib().sfg_set_preconditioner_weights(self._h, A.fptr(w), w.size))

    def pcg_stats(self) -> dict:
        """Reduced-system PCG solves of the last optimize call (PCG forms)."""
        s = A.PcgStatsC()
        _check(lib().sfg_get_pcg_stats(self._h, C.byref(s)))
        return {k: getattr(s, k) for k, _ in A.PcgStatsC._fields_}

    def fp64_diag_tiles(self) -> int:
        """Mixed form: FP32 diagonal tiles factored again in FP64 (near-singular pivots) so far."""
        n = C.c_int64()
        _check(lib().sfg_fp64_diag_tiles(self._h, C.byref(n)))
        return n.value

    def pcg_step_error(self) -> dict:
        """The exact LDL^T as judge of one PCG step at the last accepted state."""
        e, it, res = C.c_double(), C.c_int32(), C.c_double()
        _check(lib().sfg_pcg_step_error(self._h, C.byref(e), C.byref(it), C.byref(res)))
        return dict(rel_step_error=e.value, iterations=it.value, rel_residual=res.value)

    def collect_samples(self, max_systems: int) -> None:
        """Record preconditioner training samples during the following optimize calls."""
        _check(lib().sfg_collect_samples(self._h, max_systems))

    def samples(self) -> np.ndarray:
        n = C.c_int64()
        _check(lib().sfg_get_samples(self._h, None, 0, C.byref(n)))
        out = np.zeros((n.value, A.PRECOND_SAMPLE_FLOATS), dtype=np.float32)
        if n.value:
            _check(lib().sfg_get_samples(self._h, A.fptr(out), n.value, C.byref(n)))
        return out

    def close(self) -> None:
        if self._h:
            lib().sfg_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self) -> None:
        try:
            self.close()
        except Exception:
            pass

    def set_values(self, values: np.ndarray) -> None:
        v = np.ascontiguousarray(values, dtype=np.float64)
        _check(lib().sfg_set_values(self._h, A.dptr(v), v.size))

    def get_values(self) -> np.ndarray:
        out = np.zeros(self.storage_dim)
        _check(lib().sfg_get_values(self._h, A.dptr(out), out.size))
        return out

    def optimize(self, values: np.ndarray | None = None, num_iterations: int = -1,
                 params: A.OptimizerParams | None = None,
                 out: np.ndarray | None = None,
                 populate_best_linearization: bool = False) -> tuple[np.ndarray, OptimizationStats]:
        """Optimizer::Optimize(values, num_iterations, populate_best_linearization, stats): returns
        (best values, stats).  `out` (float64, storage size), if given, receives the best values
        (e.g. a pinned buffer).  With populate_best_linearization the stats carry the linearization
        at the best values (symforce/opt/internal/optimizer_utils.h:69-75); with params.debug_stats
        the linear solver's ordering and the sparsity of its factor L
        (symforce/opt/levenberg_marquardt_solver.tcc:209-211)."""
        if values is not None:
            self.set_values(values)
        p = params or self.params
        cap = (p.iterations if num_iterations < 0 else num_iterations) + 1
        recs = (A.IterationC * cap)()
        st = A.StatsC(recs, cap, 0, 0, 0, 0, 0, 0.0)
        _check(lib().sfg_optimize(self._h, C.byref(p), num_iterations, C.byref(st)))
        stats = OptimizationStats([recs[i] for i in range(st.num_iterations)], st.best_index,
                                  st.status, st.failure_reason, st.kernel_launches, st.device_ms)
        if out is None:
            out = np.zeros(self.storage_dim)
        _check(lib().sfg_get_values(self._h, A.dptr(out), out.size))
        if populate_best_linearization:
            lin = self.linearize(out)
            stats.best_linearization = dict(residual=lin["residual"], rhs=lin["rhs"], error=lin["error"],
                                            hessian_lower=dict(colptr=lin["colptr"], rowidx=lin["rowidx"],
                                                               values=lin["hvals"]))
        if p.debug_stats and self.form.linear_solver in (A.SFG_LINEAR_SOLVER_SPARSE_LDLT,
                                                          A.SFG_LINEAR_SOLVER_SCHUR):
            stats.linear_solver_ordering = self.permutation()
            stats.cholesky_factor_sparsity = self.factor_lower(with_values=False)
        return out, stats

    def factor_lower(self, with_values: bool = True) -> dict:
        """The unit lower factor L of the last exact factorization (strict lower CSC, solver order)."""
        n = self.tangent_dim - (3 * self.problem.num_schur_keys
                                if self.form.linear_solver in A.SCHUR_SOLVERS else 0)
        return _lower_csc(lib().sfg_factor_lower, self._h, n, with_values)

    def optimize_continue(self, num_iterations: int, params: A.OptimizerParams | None = None,
                          relax_damping: bool = True) -> OptimizationStats:
        """The loop of GncOptimizer::OptimizeContinue (symforce/opt/gnc_optimizer.h:113-121): ResetState
        on the best values of the last call (lambda, nu and the iteration counter carry over), with
        RelaxDampingToInitial first when `relax_damping`.  Returns only the new records; best_index is
        -1 when none of them improved on the starting state."""
        p = params or self.params
        cap = num_iterations + 1
        recs = (A.IterationC * cap)()
        st = A.StatsC(recs, cap, 0, 0, 0, 0, 0, 0.0)
        _check(lib().sfg_optimize_continue(self._h, C.byref(p), num_iterations, int(relax_damping), C.byref(st)))
        return OptimizationStats([recs[i] for i in range(st.num_iterations)], st.best_index, st.status,
                                 st.failure_reason, st.kernel_launches, st.device_ms)

    def set_factor_consts(self, batch: int, consts: np.ndarray) -> None:
        """Replace the constants of one factor batch (the caller's factor order)."""
        c = np.ascontiguousarray(consts, dtype=np.float64)
        _check(lib().sfg_set_factor_consts(self._h, batch, A.dptr(c), c.size))

    def time_stage(self, stage: int, reps: int = 20) -> dict:
        """CUDA-event time of one stage of the LM iteration (after an optimize call)."""
        ms, by, fm = C.c_double(), C.c_double(), C.c_double()
        _check(lib().sfg_time_stage(self._h, stage, reps, C.byref(ms), C.byref(by), C.byref(fm)))
        return dict(ms=ms.value, bytes=by.value, fmas=fm.value)

    def linearize(self, values: np.ndarray | None = None):
        """Linearization at the given (or current) values: residual, rhs, error, CSC hessian_lower."""
        if values is not None:
            self.set_values(values)
        res = np.zeros(self.residual_dim)
        rhs = np.zeros(self.tangent_dim)
        err = C.c_double()
        _check(lib().sfg_linearize(self._h, A.dptr(res), A.dptr(rhs), C.byref(err)))
        nnz = C.c_int64()
        _check(lib().sfg_hessian_lower(self._h, C.byref(nnz), None, None, None))
        colptr = np.zeros(self.tangent_dim + 1, dtype=np.int32)
        rowidx = np.zeros(nnz.value, dtype=np.int32)
        hv = np.zeros(nnz.value)
        _check(lib().sfg_hessian_lower(self._h, C.byref(nnz), A.iptr(colptr), A.iptr(rowidx), A.dptr(hv)))
        return dict(residual=res, rhs=rhs, error=err.value, colptr=colptr, rowidx=rowidx, hvals=hv)

    def linearize_dense(self, values: np.ndarray | None = None) -> dict:
        """DenseLinearizer's linearization (symforce/opt/dense_linearizer.h, DenseLinearization in
        symforce/opt/linearization.h:27-73): residual, dense hessian_lower (lower triangle filled,
        upper zero), rhs and error, from the device linearization.  The Jacobian is not formed on the
        device (the kernels accumulate J^T J per factor), so include_jacobians has no counterpart."""
        lin = self.linearize(values)
        return dict(residual=lin["residual"], rhs=lin["rhs"], error=lin["error"],
                    hessian_lower=csc_lower_to_dense(lin["colptr"], lin["rowidx"], lin["hvals"],
                                                     self.tangent_dim))

    def compute_covariances(self, values: np.ndarray, num_keys: int) -> dict:
        """Optimizer::ComputeCovariances with a block-diagonal C (symforce/opt/optimizer.tcc:176-199,
        symforce/opt/internal/covariance_utils.h:116-140): the marginal covariance of the first
        `num_keys` keys of the key order at `values`.  The trailing block C of the undamped Hessian
        is damped by the optimizer's epsilon, the reduced system S = B - E C^-1 E^T is factored on
        the GPU (SparseSchurSolver: point inverses, S, LDL^T) and S^-1 = (H^-1)_BB is formed by one
        solve with the identity on B as right-hand sides.  Returns {key index: covariance block}."""
        if not 0 < num_keys < len(self.problem.key_types):
            raise ValueError("num_keys must leave a non-empty trailing block to eliminate")
        dims = [A.KEY_DIMS[int(t)][1] for t in self.problem.key_types]
        offs = np.concatenate([[0], np.cumsum(dims)])
        block_dim = int(offs[num_keys])
        n = int(offs[-1])
        lin = self.linearize(values)
        colptr, rowidx, hv = lin["colptr"], lin["rowidx"], lin["hvals"].copy()
        for j in range(block_dim, n):  # damp the diagonal of C
            q = np.searchsorted(rowidx[colptr[j]:colptr[j + 1]], j) + colptr[j]
            if q >= colptr[j + 1] or rowidx[q] != j:
                raise SfgError(A.SFG_ERR_STRUCTURE, f"Hessian column {j} has no diagonal entry")
            hv[q] += self.form.epsilon
        solver = SparseSchur(n, colptr, rowidx, n - block_dim, device=self.form.device)
        solver.factorize(hv)
        rhs = np.zeros((n, block_dim))
        rhs[:block_dim, :block_dim] = np.eye(block_dim)
        cov = solver.solve(rhs)[:block_dim]
        return {k: cov[offs[k]:offs[k + 1], offs[k]:offs[k + 1]].copy() for k in range(num_keys)}

    def permutation(self) -> np.ndarray:
        n = self.form.linear_solver in A.SCHUR_SOLVERS
        size = self.tangent_dim - (3 * self.problem.num_schur_keys if n else 0)
        perm = np.zeros(size, dtype=np.int32)
        _check(lib().sfg_permutation(self._h, A.iptr(perm), size))
        return perm

    def fronts(self) -> tuple[np.ndarray, np.ndarray]:
        """Pivot widths and sizes of the exact factorization's fronts (supernodes), postorder."""
        count = C.c_int32(0)
        _check(lib().sfg_fronts(self._h, C.byref(count), None, None))
        width = np.zeros(count.value, dtype=np.int32)
        size = np.zeros(count.value, dtype=np.int32)
        _check(lib().sfg_fronts(self._h, C.byref(count), A.iptr(width), A.iptr(size)))
        return width, size


class GncOptimizer:
    """sym::GncOptimizer<Optimizer> (symforce/opt/gnc_optimizer.h:22-110) over the device loop.

    The reference keeps mu as a Values entry that the robust factors read; here it is a constant of
    the factors that take it, named by (batch index, constant index) pairs in `mu_slots`, which the
    schedule rewrites on the device (sfg_set_factor_consts) before every stage."""

    def __init__(self, problem: A.ProblemArrays, params: A.OptimizerParams, gnc_params,
                 mu_slots, form: A.FormParams | None = None):
        self.problem = problem
        self.params = params
        self.gnc_params = gnc_params
        self.mu_slots = list(mu_slots)
        self.optimizer = Optimizer(problem, params, form)
        self._consts = {b: np.array(problem.batches[b].consts, dtype=np.float64, copy=True)
                        for b, _ in self.mu_slots}

    def _set_mu(self, mu: float) -> None:
        for b, ci in self.mu_slots:
            self._consts[b][:, ci] = mu
        for b in self._consts:
            self.optimizer.set_factor_consts(b, self._consts[b])

    def optimize(self, values: np.ndarray, num_iterations: int = -1):
        """GncOptimizer::Optimize: returns (best values, OptimizationStats) with the records of every
        stage, and the final mu in stats.mu."""
        from . import gnc

        def run(p, n, cont, relax):
            if not cont:
                _, st = self.optimizer.optimize(values, num_iterations=n, params=p)
            else:
                st = self.optimizer.optimize_continue(n, params=p, relax_damping=relax)
            return st.iterations, st.best_index, st.status, st.failure_reason

        r = gnc.run_gnc(self.params, self.gnc_params, self._set_mu, run, num_iterations)
        stats = OptimizationStats(r["iterations"], r["best_index"], r["status"], r["failure_reason"])
        stats.mu = r["mu"]
        return self.optimizer.get_values(), stats

    def close(self) -> None:
        self.optimizer.close()


class SparseLdlt:
    """SparseCholeskySolver concept on a CSC lower matrix: factorize(values), solve(b)."""

    def __init__(self, n: int, colptr, rowidx, ordering: int = A.SFG_ORDERING_NESTED_DISSECTION,
                 device: int = 0):
        self.n = n
        self._colptr = np.ascontiguousarray(colptr, dtype=np.int32)
        self._rowidx = np.ascontiguousarray(rowidx, dtype=np.int32)
        self._h = C.c_void_p()
        _check(lib().sfg_ldlt_create(n, A.iptr(self._colptr), A.iptr(self._rowidx), ordering, device,
                                     C.byref(self._h)))

    def factorize(self, values) -> None:
        v = np.ascontiguousarray(values, dtype=np.float64)
        _check(lib().sfg_ldlt_factorize(self._h, A.dptr(v)))

    def solve(self, b) -> np.ndarray:
        b = np.ascontiguousarray(np.asarray(b, dtype=np.float64).T)  # column-major rhs
        nrhs = 1 if b.ndim == 1 else b.shape[0]
        x = np.zeros_like(b)
        _check(lib().sfg_ldlt_solve(self._h, A.dptr(b), A.dptr(x), nrhs))
        return x.T if b.ndim > 1 else x

    def diagonal(self) -> np.ndarray:
        d = np.zeros(self.n)
        _check(lib().sfg_ldlt_diagonal(self._h, A.dptr(d)))
        return d

    def permutation(self) -> np.ndarray:
        p = np.zeros(self.n, dtype=np.int32)
        _check(lib().sfg_ldlt_permutation(self._h, A.iptr(p)))
        return p

    def lower(self) -> dict:
        """L(): the unit lower factor (strict lower CSC in the solver's ordering) with its values."""
        return _lower_csc(lib().sfg_ldlt_lower, self._h, self.n)

    def __del__(self) -> None:
        try:
            if self._h:
                lib().sfg_ldlt_destroy(self._h)
        except Exception:
            pass


class SparseSchur:
    """SparseSchurSolver concept: A = [[B, E^T], [E, C]] with 3x3 block-diagonal C."""

    def __init__(self, n: int, colptr, rowidx, c_dim: int, device: int = 0):
        self.n = n
        self._colptr = np.ascontiguousarray(colptr, dtype=np.int32)
        self._rowidx = np.ascontiguousarray(rowidx, dtype=np.int32)
        self._h = C.c_void_p()
        _check(lib().sfg_schur_create(n, A.iptr(self._colptr), A.iptr(self._rowidx), c_dim, device,
                                      C.byref(self._h)))

    def factorize(self, values) -> None:
        v = np.ascontiguousarray(values, dtype=np.float64)
        _check(lib().sfg_schur_factorize(self._h, A.dptr(v)))

    def solve(self, b) -> np.ndarray:
        b = np.ascontiguousarray(np.asarray(b, dtype=np.float64).T)
        nrhs = 1 if b.ndim == 1 else b.shape[0]
        x = np.zeros_like(b)
        _check(lib().sfg_schur_solve(self._h, A.dptr(b), A.dptr(x), nrhs))
        return x.T if b.ndim > 1 else x

    def __del__(self) -> None:
        try:
            if self._h:
                lib().sfg_schur_destroy(self._h)
        except Exception:
            pass
