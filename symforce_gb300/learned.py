"""The learned camera-block preconditioner of the PCG form: training data, training, weights.

Training data come from the plain FP64 solver itself: every reduced camera system S y = v that the
exact Schur + LDL^T path forms during LM on seeded small bundle-adjustment instances, recorded on
the device as one sample per camera block (network inputs, whitened rhs and whitened exact
solution; include/sfgpu.h describes the layout and the loss).  Training runs on the GPU through
the library's own forward / backward / Adam kernels (`sfg_precond_train`).

    python -m symforce_gb300.learned train --instances 200 --out symforce_gb300/weights/precond_net.npy
    (defaults: 4000 Adam steps, batch 1024, lr 1e-3, seed 0, Kaporin weight 10: the shipped weights)
    python -m symforce_gb300.learned evaluate
"""

from __future__ import annotations

import argparse
import ctypes as C
import json
import time
from pathlib import Path

import numpy as np

from . import _cabi as A
from . import synth
from .optimizer import Optimizer, _check, lib

WEIGHTS = Path(__file__).resolve().parent / "weights" / "precond_net.npy"
TRAIN_SEED_BASE = 10_000  # training instances use seeds TRAIN_SEED_BASE + k, disjoint from tests
# Weight of the Kaporin term of the shipped weights.  Block Jacobi minimizes Kaporin's condition
# number over block-diagonal preconditioners, so the regression term alone (weight 0) moves the
# network to blocks that need 15-35 % more PCG iterations than block Jacobi on held-out problems;
# weight 10 keeps it beside block Jacobi, where it saves ~1 % (the FP64 PCG comparison in
# tests/test_gpu_pcg.py).
KAPORIN = 10.0


def init_weights(seed: int = 0) -> np.ndarray:
    """He-initialised hidden layers, zero output layer (the untrained network is block Jacobi)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    F, H, O = A.PRECOND_FEATURES, A.PRECOND_HIDDEN, A.PRECOND_OUTPUTS
    parts = [rng.normal(0, np.sqrt(2.0 / F), size=F * H), np.zeros(H),
             rng.normal(0, np.sqrt(2.0 / H), size=H * H), np.zeros(H),
             np.zeros(H * O), np.zeros(O)]
    w = np.concatenate(parts).astype(np.float32)
    assert w.size == A.PRECOND_NET_PARAMS
    return w


def load_weights(path: Path | str | None = None) -> np.ndarray:
    p = Path(path) if path else WEIGHTS
    if not p.exists():
        raise FileNotFoundError(f"no preconditioner weights at {p}; train them with "
                                f"`python -m symforce_gb300.learned train`")
    w = np.load(p).astype(np.float32)
    if w.size != A.PRECOND_NET_PARAMS:
        raise ValueError(f"{p} holds {w.size} weights, expected {A.PRECOND_NET_PARAMS}")
    return w


def save_weights(w: np.ndarray, path: Path | str | None = None) -> Path:
    p = Path(path) if path else WEIGHTS
    p.parent.mkdir(parents=True, exist_ok=True)
    np.save(p, np.ascontiguousarray(w, dtype=np.float32))
    return p


def training_instance(k: int) -> A.ProblemArrays:
    """The k-th seeded training instance: 12-60 cameras, 150 points per camera, 3-5.5 views per
    point on average (the benchmark generator at smaller sizes)."""
    nc = 12 + (7 * k) % 49
    npt = 150 * nc
    views = 3.0 + 2.5 * ((13 * k) % 11) / 10.0
    return synth.bundle_adjustment(nc, npt, int(views * npt), seed=TRAIN_SEED_BASE + k)


def ba_params(iterations: int = 30) -> A.OptimizerParams:
    return A.default_optimizer_params(lambda_update_type=A.SFG_LAMBDA_UPDATE_DYNAMIC,
                                      iterations=iterations)


def collect(instances, max_systems: int = 24, iterations: int = 30) -> np.ndarray:
    """Samples of every reduced system the plain FP64 Schur solver forms on the given problems."""
    out = []
    for p in instances:
        opt = Optimizer(p, ba_params(iterations),
                        A.default_form_params(linear_solver=A.SFG_LINEAR_SOLVER_SCHUR))
        opt.collect_samples(max_systems)
        opt.optimize(p.values)
        out.append(opt.samples())
        opt.close()
    return np.concatenate(out, 0) if out else np.zeros((0, A.PRECOND_SAMPLE_FLOATS), np.float32)


def train(samples: np.ndarray, steps: int = 4000, batch: int = 1024, lr: float = 1e-3,
          seed: int = 0, weights: np.ndarray | None = None, device: int = 0, kaporin: float = 0.0):
    """Adam on the GPU; returns (weights, per-step batch loss).  `kaporin` weights the loss term
    that keeps the preconditioner near block Jacobi (include/sfgpu.h, learned preconditioner)."""
    s = np.ascontiguousarray(samples, dtype=np.float32)
    w = np.ascontiguousarray(init_weights(seed) if weights is None else weights, dtype=np.float32).copy()
    curve = np.zeros(steps, dtype=np.float32)
    p = A.TrainParamsC(steps, batch, lr, 0.9, 0.999, 1e-8, seed, device, kaporin)
    _check(lib().sfg_precond_train(A.fptr(s), s.shape[0], C.byref(p), A.fptr(w), A.fptr(curve)))
    return w, curve


def loss_grad(samples: np.ndarray, weights: np.ndarray, device: int = 0, kaporin: float = 0.0):
    s = np.ascontiguousarray(samples, dtype=np.float32)
    w = np.ascontiguousarray(weights, dtype=np.float32)
    loss = C.c_double()
    g = np.zeros(A.PRECOND_NET_PARAMS, dtype=np.float32)
    _check(lib().sfg_precond_loss_grad(A.fptr(s), s.shape[0], A.fptr(w), C.c_float(kaporin),
                                       C.byref(loss), A.fptr(g), device))
    return loss.value, g


def infer(features: np.ndarray, weights: np.ndarray, device: int = 0) -> np.ndarray:
    x = np.ascontiguousarray(features, dtype=np.float32)
    w = np.ascontiguousarray(weights, dtype=np.float32)
    z = np.zeros((x.shape[0], A.PRECOND_OUTPUTS), dtype=np.float32)
    _check(lib().sfg_precond_infer(A.fptr(x), x.shape[0], A.fptr(w), A.fptr(z), device))
    return z


def time_to_cost(stats, target: float, rel: float = 1e-6) -> float | None:
    """Device time (ms) of the first LM record whose best error is within `rel` of `target`."""
    for r in stats.iterations:
        if r.best_error <= target * (1 + rel):
            return r.elapsed_ms
    return None


def compare(problem: A.ProblemArrays, weights: np.ndarray, params: A.OptimizerParams,
            precision: int = A.SFG_PRECISION_MIXED, target: float | None = None,
            forms=("block_jacobi", "learned"), **form_overrides) -> dict:
    """Block-Jacobi PCG versus the learned preconditioner (and optionally the exact "plain" /
    "mixed" Schur forms) on one problem: PCG iterations, fallbacks, LM iterations, device time,
    final cost and, given the oracle's cost, the time to reach it within 1e-6."""
    solvers = {"block_jacobi": (A.SFG_LINEAR_SOLVER_PCG_BLOCK_JACOBI, precision),
               "learned": (A.SFG_LINEAR_SOLVER_PCG_LEARNED, precision),
               "plain": (A.SFG_LINEAR_SOLVER_SCHUR, A.SFG_PRECISION_FP64),
               "mixed": (A.SFG_LINEAR_SOLVER_SCHUR, A.SFG_PRECISION_MIXED)}
    out = {}
    for name in forms:
        solver, prec = solvers[name]
        opt = Optimizer(problem, params, A.default_form_params(precision=prec, linear_solver=solver,
                                                               **form_overrides),
                        weights=weights if solver == A.SFG_LINEAR_SOLVER_PCG_LEARNED else None)
        opt.optimize(problem.values)  # warm-up (graph build)
        _, st = opt.optimize(problem.values)
        ps = opt.pcg_stats()
        out[name] = dict(pcg_iterations=int(ps["iterations"]), solves=int(ps["solves"]),
                         fallbacks=int(ps["fallbacks"]), lm_iterations=len(st.iterations) - 1,
                         device_ms=round(st.device_ms, 3), best_error=st.best_error)
        if target is not None:
            out[name]["time_to_cost_ms"] = time_to_cost(st, target)
        opt.close()
    return out


def main(argv=None) -> None:
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    sub = ap.add_subparsers(dest="cmd", required=True)
    t = sub.add_parser("train")
    t.add_argument("--instances", type=int, default=200)
    t.add_argument("--steps", type=int, default=4000)
    t.add_argument("--batch", type=int, default=1024)
    t.add_argument("--lr", type=float, default=1e-3)
    t.add_argument("--seed", type=int, default=0)
    t.add_argument("--kaporin", type=float, default=KAPORIN)
    t.add_argument("--out", default=str(WEIGHTS))
    t.add_argument("--log", default=None, help="write a JSON summary here")
    e = sub.add_parser("evaluate")
    e.add_argument("--weights", default=str(WEIGHTS))
    e.add_argument("--seeds", default="0,1,2")
    e.add_argument("--pcg-tol", type=float, default=1e-8)
    e.add_argument("--pcg-max-iters", type=int, default=500)
    e.add_argument("--forms", default="block_jacobi,learned")
    args = ap.parse_args(argv)
    if args.cmd == "train":
        t0 = time.perf_counter()
        samples = collect(training_instance(k) for k in range(args.instances))
        t1 = time.perf_counter()
        w, curve = train(samples, args.steps, args.batch, args.lr, args.seed, kaporin=args.kaporin)
        t2 = time.perf_counter()
        path = save_weights(w, args.out)
        k = max(1, args.steps // 20)
        summary = dict(samples=int(samples.shape[0]), instances=args.instances, steps=args.steps,
                       batch=args.batch, lr=args.lr, kaporin=args.kaporin,
                       collect_s=round(t1 - t0, 2), train_s=round(t2 - t1, 2),
                       loss_first=float(curve[:k].mean()), loss_last=float(curve[-k:].mean()),
                       weights=str(path))
        print(json.dumps(summary))
        if args.log:
            Path(args.log).write_text(json.dumps(dict(summary, curve=curve[::k].tolist()), indent=1))
    else:
        w = load_weights(args.weights)
        for seed in [int(s) for s in args.seeds.split(",")]:
            p = synth.bundle_adjustment(50, 7800, 32000, seed=seed)
            # the exact FP64 Schur form's converged cost is the target (it matches the oracle's)
            ref = Optimizer(p, ba_params(100), A.default_form_params(linear_solver=A.SFG_LINEAR_SOLVER_SCHUR))
            target = ref.optimize(p.values)[1].best_error
            ref.close()
            r = compare(p, w, ba_params(100), target=target, forms=tuple(args.forms.split(",")),
                        pcg_tol=args.pcg_tol, pcg_max_iters=args.pcg_max_iters)
            print(json.dumps(dict(seed=seed, pcg_tol=args.pcg_tol, **r)))


if __name__ == "__main__":
    main()
