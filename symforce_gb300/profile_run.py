"""Run a few optimize calls of a named workload, for profilers.

    python -m symforce_gb300.profile_run --workload ba_50_7800 --form plain --runs 2

Set SFG_EAGER=1 so that each kernel is an individual launch (profilers do not attribute kernels
inside graphs with conditional nodes).
"""

from __future__ import annotations

import argparse

from . import _cabi as A
from . import workloads
from .optimizer import Optimizer


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--workload", default="ba_50_7800")
    ap.add_argument("--form", default="plain", choices=["plain", "mixed", "jacobi", "learned"])
    ap.add_argument("--pcg-tol", type=float, default=1e-8)
    ap.add_argument("--runs", type=int, default=2)
    ap.add_argument("--iterations", type=int, default=-1, help="LM iteration cap (default: the workload's)")
    args = ap.parse_args()
    w = workloads.get(args.workload)
    p = w.problem()
    prec = A.SFG_PRECISION_FP64 if args.form == "plain" else A.SFG_PRECISION_MIXED
    form = w.form(prec)
    if args.form in ("jacobi", "learned"):
        form.linear_solver = (A.SFG_LINEAR_SOLVER_PCG_BLOCK_JACOBI if args.form == "jacobi"
                              else A.SFG_LINEAR_SOLVER_PCG_LEARNED)
        form.pcg_tol = args.pcg_tol
    params = w.params()
    if args.iterations > 0:
        params.iterations = args.iterations
    opt = Optimizer(p, params, form)
    for _ in range(args.runs):
        _, stats = opt.optimize(p.values)
        print(f"{args.workload} {args.form}: {len(stats.iterations)} records, best {stats.best_error:.10g}, "
              f"{stats.device_ms:.3f} ms, {stats.kernel_launches} kernels", flush=True)


if __name__ == "__main__":
    main()
