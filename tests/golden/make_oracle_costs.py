"""Generate tests/golden/oracle_costs.json: the CPU oracle's best cost on the benchmark workloads.

The benchmark's target cost ("time to FP64-oracle cost") is read from this file, so the timed GPU
run never executes the oracle.  Run from the repository root:

    python tests/golden/make_oracle_costs.py
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


def main() -> None:
    out = {}
    for name in ["ba_50_7800", "robot2d_1000"]:
        w = workloads.get(name)
        p = w.problem()
        r = O.optimize(p, w.params(), linear_solver=A.SFG_LINEAR_SOLVER_SPARSE_LDLT,
                       ordering=A.SFG_ORDERING_MIN_DEGREE)
        best = r["iterations"][r["best_index"]]
        out[name] = dict(
            seed=w.seed,
            best_error=best.new_error,
            initial_error=r["iterations"][0].new_error,
            num_records=len(r["iterations"]),
            best_index=r["best_index"],
            status=r["status"],
            oracle_seconds=r["seconds"],
            errors=[it.new_error for it in r["iterations"]],
            accepted=[it.update_accepted for it in r["iterations"]],
        )
        print(name, out[name]["best_error"], out[name]["num_records"], r["seconds"])
    (ROOT / "tests" / "golden" / "oracle_costs.json").write_text(json.dumps(out, indent=1))


if __name__ == "__main__":
    main()
