"""Trains the learned 4x-dt stepper and writes its weights.

Training data: plain trajectories of the 256 batched dam-break scenes
(particle counts log-uniform in [2048, 65536], rest density and viscosity
varied per scene), one sample per tracked particle per substep: the 32
neighbour features at substep t and the correction that makes one 4 dt step
from t land on the velocity 4 plain substeps reach, plus the density change
over those substeps. The last `--holdout` fraction of the substeps is kept
for validation. Everything runs through the engine's own kernels
(include/clsph_learned.h); torch is not used.

    python -m libclsph_gb300.train_stepper [--substeps 1000] [--stride 64]
        [--epochs 3] [--out libclsph_gb300/weights/stepper_4dt.npz]
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


def collect(scenes, substeps: int, stride: int, dt_mult: int = 4, chunk: int = 50):
    solver = GpuSolver.batched([s.params for s in scenes], [s.terms for s in scenes],
                               [s.n for s in scenes], [s.mesh for s in scenes])
    solver.upload(np.concatenate([s.particles for s in scenes]))
    m = (solver.n + stride - 1) // stride
    cap = m * max(1, substeps - dt_mult)
    col = Lm.Collector(solver, stride, cap, dt_mult)
    done = 0
    while done < substeps:
        k = min(chunk, substeps - done)
        col.step(k)
        done += k
    flags = solver.sync()
    return solver, col, m, flags


def main(argv=None) -> dict:
    ap = argparse.ArgumentParser()
    ap.add_argument("--scenes", type=int, default=256)
    ap.add_argument("--substeps", type=int, default=1000)
    ap.add_argument("--stride", type=int, default=64)
    ap.add_argument("--epochs", type=int, default=3)
    ap.add_argument("--batch", type=int, default=65536)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--lr-final", type=float, default=3e-5)
    ap.add_argument("--holdout", type=float, default=0.05)
    ap.add_argument("--seed", type=int, default=7)
    ap.add_argument("--out", default=str(Lm.default_weights_path()))
    args = ap.parse_args(argv)

    t0 = time.perf_counter()
    scenes = W.batched_dam_breaks(args.scenes)
    solver, col, m, flags = collect(scenes, args.substeps, args.stride)
    xp, yp, count = col.samples()
    t_collect = time.perf_counter() - t0
    per_step = m
    steps_with_samples = count // per_step
    n_val_steps = max(1, int(round(steps_with_samples * args.holdout)))
    n_train = (steps_with_samples - n_val_steps) * per_step
    n_train -= n_train % args.batch
    val_first = (steps_with_samples - n_val_steps) * per_step
    n_val = count - val_first

    mlp = Lm.Mlp(seed=args.seed)
    t1 = time.perf_counter()
    log = mlp.train(xp, yp, n_train, epochs=args.epochs, batch=args.batch, lr=args.lr,
                    lr_final=args.lr_final, seed=args.seed, fit_normalisation=True, log_every=50)
    t_train = time.perf_counter() - t1
    val_loss = mlp.loss(xp + 4 * 32 * val_first, yp + 4 * 4 * val_first, n_val)
    train_loss = mlp.loss(xp, yp, min(n_train, 1 << 22))
    blob = mlp.blob()
    # per-output quality on the held-out substeps
    _, y_val = col.copy(val_first, n_val)
    pred = mlp.predict(xp + 4 * 32 * val_first, n_val)
    resid = pred.astype(np.float64) - y_val
    var = y_val.astype(np.float64).var(0)
    per_output = {
        name: {"r2": float(1 - (resid[:, k] ** 2).mean() / max(var[k], 1e-30)),
               "rms_error": float(np.sqrt((resid[:, k] ** 2).mean())),
               "rms_target": float(np.sqrt((y_val[:, k].astype(np.float64) ** 2).mean()))}
        for k, name in enumerate(["da_x", "da_y", "da_z", "drho"])}
    per_output["drho"]["mean_abs_error"] = float(np.abs(resid[:, 3]).mean())
    per_output["drho"]["mean_abs_target"] = float(np.abs(y_val[:, 3]).mean())
    report = {
        "scenes": args.scenes, "particles": int(solver.n), "substeps": args.substeps,
        "tracked_per_substep": per_step, "samples": int(count), "train_samples": int(n_train),
        "val_samples": int(n_val), "epochs": args.epochs, "batch": args.batch, "lr": args.lr,
        "lr_final": args.lr_final, "collect_s": t_collect, "train_s": t_train,
        "train_loss": train_loss, "val_loss": val_loss, "val_outputs": per_output,
        "loss_log": [float(v) for v in log],
        "y_sigma": [float(v) for v in blob[Lm.OFF_YSIGMA:Lm.BLOB]],
        "y_mu": [float(v) for v in blob[Lm.OFF_YMU:Lm.OFF_YSIGMA]],
        "device_flags": int(flags),
    }
    out = Path(args.out)
    out.parent.mkdir(parents=True, exist_ok=True)
    mlp.save(out, report=json.dumps(report))
    col.close()
    solver.close()
    mlp.close()
    print(json.dumps({k: v for k, v in report.items() if k != "loss_log"}))
    return report


if __name__ == "__main__":
    main()
