"""Trains the learned 4x-dt stepper and writes its weights.

Training data: trajectories of the 256 batched dam-break scenes (particle
counts log-uniform in [2048, 65536], column heights up to 1 m, rest density
and viscosity varied per scene), one sample per tracked particle per
substep: the 32 neighbour features at substep t and the correction that
makes one 4 dt step from t land on the velocity 4 plain substeps reach, plus
the density change over those substeps.

Stage 1 samples the plain trajectories and trains the network. An optional
stage 2 (--learned-steps > 0) runs that network's learned steps from the
same start, samples the plain outcome of every state they visit (the states
a learned stepper actually reaches) and trains the final network on both
sets; on the large dam break it did not lower the density deviation of
learned runs, so it is off by default. The last `--holdout` fraction of each
stage's substeps is kept for validation. Everything runs through the
engine's own kernels (include/clsph_learned.h); torch is not used.

    python -m libclsph_gb300.train_stepper [--substeps 1000] [--learned-steps 0]
        [--stride 64] [--epochs 10] [--out libclsph_gb300/weights/stepper_4dt.npz]
"""

from __future__ import annotations

import argparse
import json
import time
from pathlib import Path

import numpy as np

from . import learned as Lm
from . import workloads as W
from .gpu import GpuSolver


def collect(solver, col, substeps: int, chunk: int = 50):
    done = 0
    while done < substeps:
        k = min(chunk, substeps - done)
        col.step(k)
        done += k
    return solver.sync()


def collect_learned(solver, col, mlp, steps: int, chunk: int = 25):
    done = 0
    while done < steps:
        k = min(chunk, steps - done)
        col.step_learned(mlp, k)
        done += k
    return solver.sync()


def output_quality(mlp, col, first: int, count: int) -> dict:
    """Per-output R^2 and errors of `mlp` on samples [first, first + count)."""
    xp, _, _ = col.samples()
    _, y = col.copy(first, count)
    pred = mlp.predict(xp + 4 * 32 * first, count)
    resid = pred.astype(np.float64) - y
    var = y.astype(np.float64).var(0)
    out = {
        name: {"r2": float(1 - (resid[:, k] ** 2).mean() / max(var[k], 1e-30)),
               "rms_error": float(np.sqrt((resid[:, k] ** 2).mean())),
               "rms_target": float(np.sqrt((y[:, k].astype(np.float64) ** 2).mean()))}
        for k, name in enumerate(["da_x", "da_y", "da_z", "drho"])}
    out["drho"]["mean_abs_error"] = float(np.abs(resid[:, 3]).mean())
    out["drho"]["mean_abs_target"] = float(np.abs(y[:, 3]).mean())
    return out


def train_on(col, first: int, count: int, args, seed: int):
    """A new network trained on samples [first, first + count) (whole batches)."""
    xp, yp, _ = col.samples()
    count -= count % args.batch
    mlp = Lm.Mlp(seed=seed)
    t = time.perf_counter()
    log = mlp.train(xp + 4 * 32 * first, yp + 4 * 4 * first, count, epochs=args.epochs, batch=args.batch,
                    lr=args.lr, lr_final=args.lr_final, seed=seed, fit_normalisation=True, log_every=50)
    return mlp, count, time.perf_counter() - t, log


def main(argv=None) -> dict:
    ap = argparse.ArgumentParser()
    ap.add_argument("--scenes", type=int, default=256)
    ap.add_argument("--substeps", type=int, default=1000)
    ap.add_argument("--learned-steps", type=int, default=0,
                    help="second stage: learned steps of the first network whose visited states are sampled")
    ap.add_argument("--stride", type=int, default=64)
    ap.add_argument("--epochs", type=int, default=10)
    ap.add_argument("--batch", type=int, default=65536)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--lr-final", type=float, default=3e-5)
    ap.add_argument("--holdout", type=float, default=0.05)
    ap.add_argument("--seed", type=int, default=7)
    ap.add_argument("--out", default=str(Lm.default_weights_path()))
    args = ap.parse_args(argv)
    dt_mult = 4

    t0 = time.perf_counter()
    scenes = W.batched_dam_breaks(args.scenes)
    initial = np.concatenate([s.particles for s in scenes])
    solver = GpuSolver.batched([s.params for s in scenes], [s.terms for s in scenes],
                               [s.n for s in scenes], [s.mesh for s in scenes])
    solver.upload(initial)
    m = (solver.n + args.stride - 1) // args.stride
    cap = m * (max(1, args.substeps - dt_mult) + args.learned_steps)
    col = Lm.Collector(solver, args.stride, cap, dt_mult)
    flags = collect(solver, col, args.substeps)
    n1 = col.samples()[2]
    val1 = m * max(1, int(round(n1 // m * args.holdout)))
    t_collect = time.perf_counter() - t0

    # stage 1: the plain trajectories
    mlp1, n_train1, t_train1, log1 = train_on(col, 0, n1 - val1, args, args.seed)
    report = {
        "scenes": args.scenes, "particles": int(solver.n), "substeps": args.substeps,
        "tracked_per_substep": m, "epochs": args.epochs, "batch": args.batch, "lr": args.lr,
        "lr_final": args.lr_final, "collect_s": t_collect,
        "stage1": {"samples": int(n1), "train_samples": int(n_train1), "val_samples": int(val1),
                   "train_s": t_train1, "val_outputs": output_quality(mlp1, col, n1 - val1, val1),
                   "loss_log": [float(v) for v in log1]},
    }
    final = mlp1
    if args.learned_steps:
        # stage 2: the states the first network's learned steps reach, from the start
        t1 = time.perf_counter()
        solver.upload(initial)
        flags |= collect_learned(solver, col, mlp1, args.learned_steps)
        n2 = col.samples()[2]
        val2 = m * max(1, int(round((n2 - n1) // m * args.holdout)))
        mlp2, n_train2, t_train2, log2 = train_on(col, 0, n2 - val2, args, args.seed + 1)
        report["stage2"] = {"samples": int(n2 - n1), "collect_s": time.perf_counter() - t1 - t_train2,
                            "train_samples": int(n_train2), "val_samples": int(val2), "train_s": t_train2,
                            "val_outputs": output_quality(mlp2, col, n2 - val2, val2),
                            "val_outputs_stage1_net": output_quality(mlp1, col, n2 - val2, val2),
                            "loss_log": [float(v) for v in log2]}
        final = mlp2
        mlp1.close()
    blob = final.blob()
    report["y_sigma"] = [float(v) for v in blob[Lm.OFF_YSIGMA:Lm.BLOB]]
    report["y_mu"] = [float(v) for v in blob[Lm.OFF_YMU:Lm.OFF_YSIGMA]]
    report["device_flags"] = int(flags)
    out = Path(args.out)
    out.parent.mkdir(parents=True, exist_ok=True)
    final.save(out, report=json.dumps(report))
    col.close()
    solver.close()
    final.close()
    brief = {k: v for k, v in report.items() if not k.startswith("stage")}
    for r in ("stage1", "stage2"):
        if r in report:
            brief[r] = {k: v for k, v in report[r].items() if k != "loss_log"}
    print(json.dumps(brief))
    return report


if __name__ == "__main__":
    main()
