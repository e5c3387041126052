"""Generate tests/golden/oracle_costs.json: the CPU oracle's best cost on the benchmark workloads.

The benchmark's target cost ("time to FP64-oracle cost") is read from this file, so the timed GPU
run never executes the oracle.  Run from the repository root:

    python tests/golden/make_oracle_costs.py [workload ...]

With names, only those workloads are (re)computed and merged into the existing file.  The
1,000-camera workload runs the oracle's Schur path (the full-Hessian LDL^T would take hours); it
takes about 40 minutes on one core.
"""

from __future__ import annotations

import json
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "tests"))

import oracle_lib as O  # noqa: E402
from symforce_gb300 import _cabi as A  # noqa: E402
from symforce_gb300 import workloads  # noqa: E402


SOLVER = {"ba_1000_200k": A.SFG_LINEAR_SOLVER_SCHUR}


def main() -> None:
    path = ROOT / "tests" / "golden" / "oracle_costs.json"
    names = sys.argv[1:] or ["ba_50_7800", "robot2d_1000"]
    out = json.loads(path.read_text()) if sys.argv[1:] and path.exists() else {}
    for name in names:
        w = workloads.get(name)
        p = w.problem()
        solver = SOLVER.get(name, A.SFG_LINEAR_SOLVER_SPARSE_LDLT)
        r = O.optimize(p, w.params(), linear_solver=solver, ordering=A.SFG_ORDERING_MIN_DEGREE)
        best = r["iterations"][r["best_index"]]
        out[name] = dict(
            seed=w.seed,
            best_error=best.new_error,
            initial_error=r["iterations"][0].new_error,
            num_records=len(r["iterations"]),
            best_index=r["best_index"],
            status=r["status"],
            oracle_seconds=r["seconds"],
            oracle_linear_solver="schur" if solver == A.SFG_LINEAR_SOLVER_SCHUR else "sparse_ldlt",
            errors=[it.new_error for it in r["iterations"]],
            accepted=[it.update_accepted for it in r["iterations"]],
        )
        print(name, out[name]["best_error"], out[name]["num_records"], r["seconds"])
    path.write_text(json.dumps(out, indent=1))


if __name__ == "__main__":
    main()
