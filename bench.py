#!/usr/bin/env python3
"""Benchmark: bundle-adjustment time to the FP64-oracle cost on one GB300.

Headline (one step = one full Optimizer::Optimize call): the 50-camera / 7,800-point / ~32k
observation synthetic bundle adjustment with Cauchy-whitened Snavely reprojection factors, plain FP64
form (Schur elimination of the points and a device multifrontal LDL^T of the reduced camera system),
DYNAMIC lambda.  Metric: milliseconds until the best cost is within 1e-6 (relative) of the CPU
oracle's final cost (committed in tests/golden/oracle_costs.json), read from the per-iteration
device timestamps of the run; lower is better.  The same line reports:
  forms    - mixed precision, block-Jacobi PCG and learned-preconditioner PCG on the same workload;
  scale    - every form on the 1,000-camera / 200k-point / ~1.2M-observation workload;
  scale_10k - every form on the 10,000-camera / 1M-point / ~5M-observation workload;
  batched  - 4,096 independent Pose3-chain problems in one persistent launch (problems/s);
  batched_dense - 4,096 small 2D localization, loop-closed Pose3 and Rot3 smoothing problems
             (the batched form's dense path);
  roofline - the linearization stage against the measured HBM copy bandwidth.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
                    [--no-scale] [--no-scale-10k] [--no-batched] [--no-cpu-baseline]

Profiling mode (no JSON line; the command the ncu summaries under profiles/ give):

    SFG_EAGER=1 python bench.py --profile-workload ba_50_7800 --profile-form plain --profile-runs 2
                                [--profile-iterations N]

runs `--profile-runs` optimize calls of one form on one workload and prints one line per call.
SFG_EAGER=1 launches each kernel on its own (profilers do not attribute the kernels inside graphs
with conditional nodes).

`--impl reference` times the CPU restatement of the reference's sym::Optimizer (the reference
itself cannot be compiled here: its Eigen / METIS dependencies are absent) on the host cores.
"""

from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

from symforce_gb300 import _cabi as A  # noqa: E402
from symforce_gb300 import workloads  # noqa: E402

METRIC = "BA time to FP64-oracle cost (rel 1e-6): plain vs mixed/learned; linearize GB/s"
WORKLOAD = "ba_50_7800"
FP64_PEAK_GFLOPS = 1208.0  # FP64 FMA throughput measured on GB300 (profiles/gb300_fp64_latency.md)
TOL = 1e-6


def _oracle_cost(name: str) -> dict:
    return json.loads((ROOT / "tests" / "golden" / "oracle_costs.json").read_text())[name]


def _measured_peaks() -> tuple[dict, str]:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        return json.loads(p.read_text()), "measured"
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines: list[str] = []

    def start(self) -> None:
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except FileNotFoundError:
            self.proc = None

    def _read(self) -> None:
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def _dist_init():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
    return world, rank, local


def _allreduce_max(x: float, world: int) -> float:
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def _barrier(world: int) -> None:
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def _cpu_solve(problem, params, max_iterations: int, variant: str = "o3") -> dict:
    """The oracle port (CPU restatement of the reference optimizer), single-threaded; `variant`
    picks its build: "o3" (the timed baseline), "o3_fast" (-O3 -ffast-math), "o2" (the parity
    build the tests use)."""
    sys.path.insert(0, str(ROOT / "tests"))
    import oracle_lib as O
    O.use_variant(variant)
    p = A.default_optimizer_params()
    for f, _ in A.OptimizerParams._fields_:
        setattr(p, f, getattr(params, f))
    p.iterations = max_iterations
    r = O.optimize(problem, p, linear_solver=A.SFG_LINEAR_SOLVER_SPARSE_LDLT,
                   ordering=A.SFG_ORDERING_MIN_DEGREE)
    return r


def run_reference(args) -> None:
    world, rank, _ = _dist_init()
    if rank != 0:
        return
    w = workloads.get(WORKLOAD)
    problem = w.problem()
    params = w.params()
    oracle = _oracle_cost(WORKLOAD)
    target = oracle["best_error"] * (1 + TOL)
    # bounded sample: the full 50-iteration solve takes ~10-15 s on one core; cap the whole run
    budget_s = float(os.environ.get("SFG_REFERENCE_BUDGET_S", "200"))
    t0 = time.perf_counter()
    probe = _cpu_solve(problem, params, params.iterations)
    est = time.perf_counter() - t0
    total_steps = args.warmup + args.steps
    iters = params.iterations
    if est * total_steps > budget_s:
        iters = max(5, int(params.iterations * budget_s / (est * total_steps)))
    times = []
    for k in range(total_steps):
        t0 = time.perf_counter()
        r = _cpu_solve(problem, params, iters)
        dt = time.perf_counter() - t0
        if k >= args.warmup:
            times.append(dt * params.iterations / iters)
    ttc_iters = next((i for i, e in enumerate(probe["iterations"]) if e.best_error <= target),
                     len(probe["iterations"]) - 1)
    frac = ttc_iters / max(len(probe["iterations"]) - 1, 1)
    ms_step = 1e3 * statistics.median(times)
    value = ms_step * frac
    sample = (f"{iters} of {params.iterations} LM iterations per step, scaled to the full solve"
              if iters < params.iterations else "full 50-iteration solve per step")
    line = {
        "metric": METRIC, "impl": "reference", "value": round(value, 3), "unit": "ms",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(ms_step, 3), "higher_is_better": False, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded PCG64)",
        "config": {"workload": WORKLOAD, "form": "plain FP64, CPU restatement of sym::Optimizer "
                   "(up-looking sparse LDL^T on the full Hessian, block minimum-degree ordering), "
                   "built g++ -O3",
                   "cores": 1},
        "cpu_baseline": {"value": round(value, 3), "unit": "ms", "cores": 1, "kind": "port",
                         "sample": sample},
        "e2e": {"value": round(value, 3), "unit": "ms", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
        "time_to_cost_fraction_of_solve": round(frac, 4),
    }
    print(json.dumps(line), flush=True)


# The forms beside the plain FP64 drop-in.  "pcg_learned" is the learned-preconditioned
# mixed-precision solve (FP32 linearization / Schur, PCG with the trained camera-block network on the
# band preconditioner, exact LDL^T as fallback, FP64 cost and gain ratio); "pcg_band" is the same
# band preconditioner without the network (Lambda = I), "pcg_block_jacobi" the block-diagonal one.
PCG_BAND = 4  # neighbouring camera blocks of a band preconditioner row (form parameter pcg_band)
FORMS = {
    "plain": (A.SFG_PRECISION_FP64, A.SFG_LINEAR_SOLVER_SCHUR, 0),
    "mixed": (A.SFG_PRECISION_MIXED, A.SFG_LINEAR_SOLVER_SCHUR, 0),
    "pcg_block_jacobi": (A.SFG_PRECISION_MIXED, A.SFG_LINEAR_SOLVER_PCG_BLOCK_JACOBI, 0),
    "pcg_band": (A.SFG_PRECISION_MIXED, A.SFG_LINEAR_SOLVER_PCG_BLOCK_JACOBI, PCG_BAND),
    "pcg_learned": (A.SFG_PRECISION_MIXED, A.SFG_LINEAR_SOLVER_PCG_LEARNED, PCG_BAND),
}
SCALE_WORKLOAD = "ba_1000_200k"
SCALE_10K_WORKLOAD = "ba_10k_1m"  # the learned form's named configuration, in the default run too
BATCH_PROBLEMS = 4096


def _form_params(params: A.OptimizerParams, name: str) -> A.OptimizerParams:
    """The plain form stops where the oracle does (the reference's early-exit rule, relative
    reduction < 1e-6); the other forms follow other LM paths, whose early exit can land up to ~1e-6
    above the oracle's cost, so they run on (relative reduction < 1e-9, same iteration cap) and the
    time is read when their best cost first reaches the target."""
    if name == "plain":
        return params
    q = A.default_optimizer_params()
    for f, _ in A.OptimizerParams._fields_:
        setattr(q, f, getattr(params, f))
    q.early_exit_min_reduction = 1e-9
    return q


def _make_form(w, name: str, device: int) -> A.FormParams:
    prec, solver, band = FORMS[name]
    form = w.form(prec)
    form.linear_solver = solver
    form.pcg_band = band
    form.device = device
    return form


def _time_form(opt, vin_np, vout_np, flush, steps, warmup, target, target9):
    """Warm up, then time `steps` full optimize calls through the public API (pinned host values in
    and out).  Returns per-step e2e ms, device ms, time-to-target ms, launches and the last stats."""
    import torch

    def step():
        flush.zero_()  # L2 flush: 256 MB > 129 MB L2
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        vals, stats = opt.optimize(vin_np, out=vout_np)
        t1 = time.perf_counter()
        recs = stats.iterations
        ttc = next((r.elapsed_ms for r in recs if r.best_error <= target), float("nan"))
        ttc9 = next((r.elapsed_ms for r in recs if r.best_error <= target9), float("nan"))
        last_values[0] = vals
        return (t1 - t0) * 1e3, stats, ttc, ttc9

    last_values = [None]

    for _ in range(warmup):
        step()
    out = dict(e2e=[], dev=[], ttc=[], ttc9=[], launches=[], stats=None)
    for _ in range(steps):
        e, stats, ttc, ttc9 = step()
        out["e2e"].append(e)
        out["dev"].append(stats.device_ms)
        out["ttc"].append(ttc)
        out["ttc9"].append(ttc9)
        out["launches"].append(stats.kernel_launches)
        out["stats"] = stats
    out["values"] = np.array(last_values[0], copy=True)
    return out


def _quat_to_rot(q: np.ndarray) -> np.ndarray:
    """Rotation matrices of [n, 4] unit quaternions [x, y, z, w]."""
    x, y, z, w = q[:, 0], q[:, 1], q[:, 2], q[:, 3]
    return np.stack([np.stack([1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)], -1),
                     np.stack([2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)], -1),
                     np.stack([2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)], -1)], 1)


def _state_errors(problem, x: np.ndarray, ref: np.ndarray) -> dict:
    """Per-state differences of a bundle-adjustment solution from a reference one, after the
    similarity transform (scale, rotation, translation of the world) that best maps its points onto
    the reference's (Umeyama): the cost is invariant to that 7-dof gauge, so solutions from different
    LM paths differ by it.  Camera rotation angle (rad), camera centre and point position (m),
    relative focal length, and the gauge scale."""
    nc = int(problem.meta["num_cameras"])
    cam, cam_r = x[:7 * nc].reshape(nc, 7), ref[:7 * nc].reshape(nc, 7)
    pts, pts_r = x[10 * nc:].reshape(-1, 3), ref[10 * nc:].reshape(-1, 3)
    mu, mu_r = pts.mean(0), pts_r.mean(0)
    a, b = pts - mu, pts_r - mu_r
    U, D, Vt = np.linalg.svd(b.T @ a / len(a))
    sgn = np.diag([1.0, 1.0, np.sign(np.linalg.det(U @ Vt))])
    R = U @ sgn @ Vt                                   # world rotation: x -> reference
    scale = float(np.trace(np.diag(D) @ sgn) / (a * a).sum(1).mean())
    t = mu_r - scale * R @ mu
    pts_al = scale * pts @ R.T + t
    Rc, Rc_r = _quat_to_rot(cam[:, :4]), _quat_to_rot(cam_r[:, :4])   # camera-from-world
    centres = -np.einsum("nji,nj->ni", Rc, cam[:, 4:])                # world position of a camera
    centres_r = -np.einsum("nji,nj->ni", Rc_r, cam_r[:, 4:])
    centres_al = scale * centres @ R.T + t
    Rc_al = Rc @ R.T                                                 # camera-from-reference-world
    dR = np.einsum("nij,nkj->nik", Rc_al, Rc_r)
    sin = 0.5 * np.linalg.norm(np.stack([dR[:, 2, 1] - dR[:, 1, 2], dR[:, 0, 2] - dR[:, 2, 0],
                                         dR[:, 1, 0] - dR[:, 0, 1]], -1), axis=1)
    ang = np.arctan2(sin, (np.trace(dR, axis1=1, axis2=2) - 1) / 2)
    intr, intr_r = x[7 * nc:10 * nc].reshape(nc, 3), ref[7 * nc:10 * nc].reshape(nc, 3)
    return {"rotation_rad": float(ang.max()),
            "camera_centre_m": float(np.linalg.norm(centres_al - centres_r, axis=1).max()),
            "point_m": float(np.linalg.norm(pts_al - pts_r, axis=1).max()),
            "focal_rel": float((np.abs(intr[:, 0] - intr_r[:, 0]) / np.abs(intr_r[:, 0])).max()),
            "gauge_scale": scale}


def _med(x):
    return round(statistics.median(x), 4)


def _form_summary(r: dict, opt, oracle_cost: float) -> dict:
    st = r["stats"]
    out = {
        "time_to_cost_ms": _med(r["ttc"]),
        "time_to_cost_1e-9_ms": _med(r["ttc9"]),
        "solve_ms": _med(r["dev"]),
        "e2e_ms": _med(r["e2e"]),
        "lm_iterations": len(st.iterations) - 1,
        "status": st.status,
        "final_cost_rel_err_vs_oracle": (st.best_error - oracle_cost) / oracle_cost,
    }
    if opt.form.linear_solver in (A.SFG_LINEAR_SOLVER_PCG_BLOCK_JACOBI, A.SFG_LINEAR_SOLVER_PCG_LEARNED):
        ps = opt.pcg_stats()
        out["pcg"] = {"solves": ps["solves"], "fallbacks": ps["fallbacks"],
                      "iterations_per_solve": round(ps["iterations"] / max(ps["solves"], 1), 1),
                      "max_rel_residual": ps["max_rel_residual"]}
    return out


def _scale_section(device: int, flush, workload: str = SCALE_WORKLOAD) -> dict:
    """A large workload (default the 1,000-camera / 200k-point / ~1.2M-observation one; the
    10,000-camera one with --scale-workload ba_10k_1m): every form once after one
    warm-up call, time to the FP64 oracle's cost (the CPU oracle's committed cost when present,
    else the plain FP64 form's own best cost, which the oracle pins at the smaller sizes)."""
    w = workloads.get(workload)
    problem = w.problem()
    params = w.params()
    costs = json.loads((ROOT / "tests" / "golden" / "oracle_costs.json").read_text())
    vin = problem.values.copy()
    res, launches, create_s = {}, 0, {}
    from symforce_gb300.optimizer import Optimizer
    for name in FORMS:
        t0 = time.perf_counter()
        opt = Optimizer(problem, _form_params(params, name), _make_form(w, name, device))
        create_s[name] = round(time.perf_counter() - t0, 2)
        r = _time_form(opt, vin, None, flush, 1, 1, -1.0, -1.0)
        launches += sum(r["launches"])
        res[name] = (r, opt)
    if workload in costs:
        oracle_cost, kind = costs[workload]["best_error"], "CPU oracle (Schur path)"
    else:
        oracle_cost, kind = res["plain"][0]["stats"].best_error, "plain FP64 GPU form"
    target = oracle_cost * (1 + TOL)
    out = {"workload": workload, "num_cameras": problem.meta["num_cameras"],
           "num_points": problem.meta["num_points"],
           "num_observations": problem.meta["num_observations"], "lm_iteration_cap": params.iterations,
           "oracle_cost": oracle_cost, "oracle": kind, "target_rel": TOL, "forms": {},
           "host_analysis_s": create_s}
    for name, (r, opt) in res.items():
        st = r["stats"]
        r["ttc"] = [next((x.elapsed_ms for x in st.iterations if x.best_error <= target), float("nan"))]
        out["forms"][name] = _form_summary(r, opt, oracle_cost)
        out["forms"][name]["max_state_err_vs_plain"] = _state_errors(problem, r["values"],
                                                                     res["plain"][0]["values"])
        opt.close()
    plain_t = out["forms"]["plain"]["time_to_cost_ms"]
    for name in FORMS:
        t = out["forms"][name]["time_to_cost_ms"]
        out["forms"][name]["speedup_vs_plain"] = round(plain_t / t, 3) if t == t and t > 0 else None
    return out, launches


def _batched_section(device: int, steps: int, cpu_budget_s: float, mixed: bool = False) -> dict:
    """4,096 independent problems in one persistent launch (device time per batch and problems/s),
    next to the CPU oracle on a bounded sample of the same problems, one optimizer per host thread:
    Pose3 chains (the block-tridiagonal path) or, with `mixed`, small 2D localization,
    loop-closed Pose3 and Rot3 smoothing problems (the dense path)."""
    from concurrent.futures import ThreadPoolExecutor

    from symforce_gb300 import synth
    from symforce_gb300.batch import BatchOptimizer
    problems = synth.mixed_small_problems(BATCH_PROBLEMS, seed=0) if mixed else synth.pose3_chains(BATCH_PROBLEMS, seed=0)
    params = A.default_optimizer_params(iterations=50)
    form = A.default_form_params()
    form.device = device
    t0 = time.perf_counter()
    opt = BatchOptimizer(problems, params, form)
    create_s = time.perf_counter() - t0
    v0 = opt.initial_values()
    opt.set_values(v0)
    shape = opt.autotune()
    opt.optimize(v0)  # warm-up (graph build)
    dev, e2e = [], []
    for _ in range(max(1, steps)):
        t0 = time.perf_counter()
        res = opt.optimize(v0)
        vals = opt.get_values()
        e2e.append((time.perf_counter() - t0) * 1e3)
        dev.append(res.device_ms)
    del vals
    ms = statistics.median(dev)
    out = {"workload": f"{'mixed_small_problems' if mixed else 'pose3_chains'}_{BATCH_PROBLEMS}",
           "problems": BATCH_PROBLEMS,
           "keys": int(sum(len(p.key_types) for p in problems)),
           "batch_ms": round(ms, 3), "problems_per_s": round(BATCH_PROBLEMS / (ms * 1e-3), 1),
           "e2e_ms": round(statistics.median(e2e), 3), "autotuned_shape": list(shape),
           "host_create_s": round(create_s, 2),
           "status_success": int((res.status == A.SFG_STATUS_SUCCESS).sum()),
           "lm_iterations_mean": round(float(res.num_iterations.mean()), 2)}
    opt.close()
    # CPU oracle: one optimizer per thread (ctypes releases the GIL), bounded sample
    sys.path.insert(0, str(ROOT / "tests"))
    import oracle_lib as O
    threads = os.cpu_count() or 1
    done, t0 = 0, time.perf_counter()
    ref_best, ref_status = [], []
    with ThreadPoolExecutor(threads) as ex:
        while time.perf_counter() - t0 < cpu_budget_s and done < BATCH_PROBLEMS:
            chunk = problems[done:done + 4 * threads]
            for r in ex.map(lambda p: O.optimize(p, params), chunk):
                ref_best.append(r["iterations"][r["best_index"]].new_error)
                ref_status.append(r["status"])
            done += len(chunk)
    cpu_s = time.perf_counter() - t0
    out["cpu_baseline"] = {"problems_per_s": round(done / cpu_s, 1), "cores": threads, "kind": "port",
                           "sample": f"the first {done} of the {BATCH_PROBLEMS} problems"}
    # per-problem parity on the same sample: best cost within 1e-9 and the same status
    if done:
        gb, rb = res.best_error[:done], np.array(ref_best)
        rel = np.abs(gb - rb) / np.maximum(np.abs(rb), 1e-300)
        out["parity_vs_oracle"] = {"problems": done, "within_1e-9": int((rel <= 1e-9).sum()),
                                   "same_status": int((res.status[:done] == np.array(ref_status)).sum()),
                                   "max_rel_cost_diff": float(rel.max())}
    return out, len(dev) + 2


def run_gb300(args) -> None:
    world, rank, local = _dist_init()
    import torch
    torch.cuda.set_device(local)
    from symforce_gb300.optimizer import Optimizer
    w = workloads.get(WORKLOAD)
    problem = w.problem()
    params = w.params()
    oracle = _oracle_cost(WORKLOAD)
    target = oracle["best_error"] * (1 + TOL)
    target9 = oracle["best_error"] * (1 + 1e-9)
    S = problem.storage_dim
    vin = torch.from_numpy(problem.values.copy()).pin_memory()
    vout = torch.empty(S, dtype=torch.float64).pin_memory()
    vin_np, vout_np = vin.numpy(), vout.numpy()
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=f"cuda:{local}")

    opts = {name: Optimizer(problem, _form_params(params, name), _make_form(w, name, local))
            for name in FORMS}
    # the plain form is the headline; clocks are sampled during its timed region
    clocks = ClockSampler(torch.cuda.current_device()) if rank == 0 else None
    _barrier(world)
    torch.cuda.synchronize()
    if clocks:
        clocks.start()
    res = {}
    for name in FORMS:
        res[name] = _time_form(opts[name], vin_np, vout_np, flush, args.steps, args.warmup, target, target9)
    torch.cuda.synchronize()
    _barrier(world)
    clk = clocks.stop() if clocks else None
    plain = res["plain"]
    value = _allreduce_max(statistics.median(plain["ttc"]), world)
    ms_step = _allreduce_max(statistics.median(plain["dev"]), world)
    e2e_ms = _allreduce_max(statistics.median(plain["e2e"]), world)
    forms = {name: _form_summary(res[name], opts[name], oracle["best_error"]) for name in FORMS}
    for name in FORMS:
        forms[name]["max_state_err_vs_plain"] = _state_errors(problem, res[name]["values"],
                                                              res["plain"]["values"])
    for name in FORMS:
        t = forms[name]["time_to_cost_ms"]
        forms[name]["speedup_vs_plain"] = round(forms["plain"]["time_to_cost_ms"] / t, 3) if t == t else None
    # live roofline of the plain form's linearization stage (CUDA events on the library's stream)
    opt = opts["plain"]
    lin = opt.time_stage(A.SFG_STAGE_LINEARIZE, reps=50)
    stages = {}
    factor_fmas = {}
    for fname in ["plain", "mixed"]:
        stages[fname] = {}
        for name, sid in [("linearize", A.SFG_STAGE_LINEARIZE), ("schur", A.SFG_STAGE_SCHUR),
                          ("factor", A.SFG_STAGE_FACTOR), ("solve", A.SFG_STAGE_SOLVE)]:
            t = opts[fname].time_stage(sid, reps=20)
            stages[fname][name] = {"ms": round(t["ms"], 5),
                                   "gfma_s": round(t["fmas"] / t["ms"] / 1e6, 2)}
            if name == "factor":
                factor_fmas[fname] = t
    for o in opts.values():
        o.close()
    peaks, peak_kind = _measured_peaks()
    achieved = lin["bytes"] / (lin["ms"] * 1e-3) / 1e9
    traffic = None
    tp = ROOT / "profiles" / "traffic.json"
    if tp.exists():
        traffic = json.loads(tp.read_text()).get(f"linearize_{WORKLOAD}")
    launches = int(sum(sum(r["launches"]) for r in res.values()))
    scale = scale_10k = batched = batched_dense = None
    # the secondary sections report an error in the line instead of losing the headline
    if not args.no_scale:
        try:
            scale, n = _scale_section(local, flush, args.scale_workload)
            launches += n
        except Exception as e:  # noqa: BLE001
            scale = {"error": f"{type(e).__name__}: {e}"}
        if args.scale_workload != SCALE_10K_WORKLOAD and not args.no_scale_10k:
            try:
                scale_10k, n = _scale_section(local, flush, SCALE_10K_WORKLOAD)
                launches += n
            except Exception as e:  # noqa: BLE001
                scale_10k = {"error": f"{type(e).__name__}: {e}"}
    if not args.no_batched:
        try:
            batched, n = _batched_section(local, min(args.steps, 5),
                                          cpu_budget_s=10.0 if rank == 0 else 0.0)
            launches += n
        except Exception as e:  # noqa: BLE001
            batched = {"error": f"{type(e).__name__}: {e}"}
        try:
            batched_dense, n = _batched_section(local, min(args.steps, 5),
                                                cpu_budget_s=10.0 if rank == 0 else 0.0, mixed=True)
            launches += n
        except Exception as e:  # noqa: BLE001
            batched_dense = {"error": f"{type(e).__name__}: {e}"}
    if rank != 0:
        return
    cpu = None
    if not args.no_cpu_baseline:
        timed = {}
        for variant in ("o3", "o3_fast", "o2"):
            t0 = time.perf_counter()
            r = _cpu_solve(problem, params, params.iterations, variant)
            cpu_s = time.perf_counter() - t0
            frac = next((i for i, e in enumerate(r["iterations"]) if e.best_error <= target),
                        len(r["iterations"]) - 1) / max(len(r["iterations"]) - 1, 1)
            timed[variant] = round(cpu_s * 1e3 * frac, 3)
        cpu = {"value": timed["o3"], "unit": "ms", "cores": 1, "kind": "port", "build": "g++ -O3",
               "variants_ms": {"-O3 -ffast-math": timed["o3_fast"], "-O2 (the parity build)": timed["o2"]},
               "sample": "one full solve (to convergence) of the same workload on one host core "
                         "(CPU restatement of sym::Optimizer, full-Hessian sparse LDL^T)"}
    line = {
        "metric": METRIC, "value": round(value, 4), "unit": "ms", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms_step, 4),
        "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded PCG64, no dataset)",
        "config": {"workload": WORKLOAD, "form": "plain FP64 (Schur over points + multifrontal "
                   "LDL^T of the reduced camera system)",
                   "parallelism": "replicas" if world > 1 else "1 GPU",
                   "l2": "flushed (256 MB write) before every step",
                   "num_cameras": problem.meta["num_cameras"], "num_points": problem.meta["num_points"],
                   "num_observations": problem.meta["num_observations"],
                   "oracle_cost": oracle["best_error"], "target_rel": TOL},
        "forms": forms,
        "roofline": {"kernel": "linearize (Snavely FP64 factor kernel + staged reduction + cost)",
                     "bound": "hbm", "achieved": round(achieved, 2),
                     "peak": peaks.get("hbm_gbs"), "unit": "GB/s",
                     "frac": round(achieved / peaks.get("hbm_gbs"), 5),
                     "traffic": traffic, "peak_kind": peak_kind,
                     "algorithmic_bytes": lin["bytes"], "ms_per_launch": round(lin["ms"], 5)},
        "stages_ms_per_launch": stages,
        # the kernel that sets the plain form's time: the FP64 multifrontal LDL^T of the reduced
        # camera system, flops from the symbolic factor (2 per multiply-add) against the FP64 rate
        # measured on this GPU (profiles/gb300_fp64_latency.md; MEASURED_PEAKS.json has no FP64 entry)
        "roofline_factor": {
            "kernel": "FactorKernel<double, 16> (persistent tile-task LDL^T)", "bound": "fp64",
            "achieved": round(2 * factor_fmas["plain"]["fmas"] / (factor_fmas["plain"]["ms"] * 1e-3) / 1e9, 2),
            "peak": FP64_PEAK_GFLOPS, "unit": "GFLOP/s", "peak_kind": "measured (FP64 FMA loop, all SMs)",
            "frac": round(2 * factor_fmas["plain"]["fmas"] / (factor_fmas["plain"]["ms"] * 1e-3) / 1e9
                          / FP64_PEAK_GFLOPS, 5),
            "multiply_adds": factor_fmas["plain"]["fmas"], "ms_per_launch": round(factor_fmas["plain"]["ms"], 5)},
        "scale": scale,
        "scale_10k": scale_10k,
        "batched": batched,
        "batched_dense": batched_dense,
        "cpu_baseline": cpu,
        "e2e": {"value": round(e2e_ms, 4), "unit": "ms", "h2d_bytes_per_step": 8 * S + 8 * 24,
                "d2h_bytes_per_step": 8 * S + 64 * len(plain["stats"].iterations)},
        "gpu_launches": launches,
        "clocks": clk,
    }
    print(json.dumps(line), flush=True)


def run_profile(args) -> None:
    """A few optimize calls of one form on one workload, for profilers."""
    from symforce_gb300.optimizer import Optimizer
    if args.profile_workload in ("pose3_chains", "mixed_small_problems"):
        # the batched form on 1,024 problems of the bench's batched sections (one launch a run)
        from symforce_gb300 import synth
        from symforce_gb300.batch import BatchOptimizer
        probs = (synth.pose3_chains(1024, seed=0) if args.profile_workload == "pose3_chains"
                 else synth.mixed_small_problems(1024, seed=0))
        params = A.default_optimizer_params(iterations=50 if args.profile_iterations <= 0 else args.profile_iterations)
        opt = BatchOptimizer(probs, params)
        v0 = opt.initial_values()
        for _ in range(args.profile_runs):
            res = opt.optimize(v0)
            print(f"{args.profile_workload} batched: 1024 problems, {res.device_ms:.3f} ms, "
                  f"{int((res.status == A.SFG_STATUS_SUCCESS).sum())} SUCCESS", flush=True)
        opt.close()
        return
    w = workloads.get(args.profile_workload)
    p = w.problem()
    params = w.params()
    if args.profile_iterations > 0:
        params.iterations = args.profile_iterations
    trace_path = None
    if args.profile_pcg_trace:
        # iteration trace of the PCG kernel's CTA 0 (read back after the runs)
        trace_path = os.path.join(tempfile.mkdtemp(), "pcg_trace.bin")
        os.environ["SFG_TRACE_PCG"] = "1"
        os.environ["SFG_TRACE_PCG_FILE"] = trace_path
    opt = Optimizer(p, _form_params(params, args.profile_form), _make_form(w, args.profile_form, 0))
    if args.profile_fronts:
        width, size = opt.fronts()
        edges = [0, 16, 64, 128, 256, 512, 1024, 2048, 4096, 1 << 30]
        hist = np.histogram(size, bins=edges)[0]
        madd = sum(int(m) ** 3 - (int(m) - int(wd)) ** 3 for wd, m in zip(width, size)) / 6
        print(f"{args.profile_workload} {args.profile_form}: {len(size)} fronts, size max {size.max()}, median "
              f"{int(np.median(size))}, pivot columns {int(width.sum())}; sizes: "
              + ", ".join(f"[{edges[q]}, {edges[q + 1]}): {int(h)}" for q, h in enumerate(hist) if h)
              + f"; dense LDL^T multiply-adds ~{madd / 1e6:.1f} M", flush=True)
    for _ in range(args.profile_runs):
        _, stats = opt.optimize(p.values)
        print(f"{args.profile_workload} {args.profile_form}: {len(stats.iterations)} records, best "
              f"{stats.best_error:.10g}, {stats.device_ms:.3f} ms, {stats.kernel_launches} kernels",
              flush=True)
    if trace_path:
        opt.pcg_stats()  # writes the trace of the last solve
        tr = np.fromfile(trace_path, dtype=np.uint64)
        n = min(int(tr[0]), (len(tr) - 1) // 4)
        st = tr[1:1 + 4 * n].astype(np.int64).reshape(n, 4)
        if n > 1:
            ph = np.empty((n - 1, 4))
            ph[:, 0] = st[1:, 0] - st[:-1, 3]  # product with S (from the previous iteration's end)
            ph[:, 1:] = np.diff(st[1:], axis=1)  # first reduction, preconditioner + update, second reduction
            med = np.median(ph, axis=0) / 1e3
            print(f"{args.profile_workload} {args.profile_form}: last solve {n} CG iterations, "
                  f"{(st[-1, 3] - st[0, 0]) / 1e3 / (n - 1):.2f} us each (CTA 0); median us: product with S "
                  f"{med[0]:.2f}, grid reduction p.Sp {med[1]:.2f}, update + preconditioner {med[2]:.2f}, "
                  f"grid reduction r.z {med[3]:.2f}", flush=True)
    opt.close()


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-scale", action="store_true", help="skip the large workload")
    ap.add_argument("--scale-workload", default=SCALE_WORKLOAD,
                    help="large workload of the scale section (ba_1000_200k or ba_10k_1m)")
    ap.add_argument("--no-scale-10k", action="store_true", help="skip the 10,000-camera workload")
    ap.add_argument("--no-batched", action="store_true", help="skip the batched sections")
    ap.add_argument("--profile-workload", default=None,
                    help="profiling mode: run --profile-runs optimize calls of one form on this workload")
    ap.add_argument("--profile-form", default="plain", choices=list(FORMS))
    ap.add_argument("--profile-runs", type=int, default=2)
    ap.add_argument("--profile-iterations", type=int, default=-1,
                    help="LM iteration cap in profiling mode (default: the workload's)")
    ap.add_argument("--profile-pcg-trace", action="store_true",
                    help="profiling mode (PCG forms): per-phase times of the last solve's CG iterations")
    ap.add_argument("--profile-fronts", action="store_true",
                    help="profiling mode: print the sizes of the factorization's fronts")
    args = ap.parse_args()
    if args.profile_workload:
        run_profile(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_gb300(args)


if __name__ == "__main__":
    main()
