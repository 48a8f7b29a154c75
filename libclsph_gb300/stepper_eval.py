"""Judges the learned 4x-dt stepper against the plain solver.

Both runs start from the same state and cover the same simulated time
(`plain_substeps` plain substeps = plain_substeps / dt_mult learned steps).
Timing runs measure simulated seconds per wall second on the GPU; accuracy
runs (the same deterministic trajectories, downloaded at checkpoints) compare
the two states:

  rho_dev_plain/learned  mean |rho / rho0 - 1| of each run (the usual SPH
                     density deviation; the headline `density_dev` is the
                     mean over checkpoints of their difference)
  density_dev_pop    |mean rho_L - mean rho_P| / rho0
  density_dev_particle  mean over particles (by id) of |rho_L - rho_P| / rho0
  pos_rms_h          RMS distance between a particle's two positions, in h
  pos_rms_chaos_h, density_dev_chaos  the same measures between the plain
                     run and a plain run whose initial positions differ by
                     1e-6 h: how far two plain trajectories of this flow
                     separate with no model error at all
  ke_plain/learned   kinetic energy

Densities are those of the checkpoint state itself (one neighbour build and
density pass on a scratch handle). No counterpart in the reference.
"""

from __future__ import annotations

import time

import numpy as np

from . import learned as Lm
from .gpu import STAGE_DENSITY, GpuSolver


def state_density(scratch: GpuSolver, state: np.ndarray) -> np.ndarray:
    """Density of every slot of `state` (the plain density kernel on a scratch handle)."""
    scratch.upload(state)
    scratch.step_until(STAGE_DENSITY)
    rho_sorted = scratch.fields()[0]
    _, perm = scratch.keys()
    rho = np.empty_like(rho_sorted)
    rho[perm] = rho_sorted
    return rho


def by_id(solver: GpuSolver, scratch: GpuSolver):
    state = solver.download()
    ids = solver.ids()
    order = np.argsort(ids)
    rho = state_density(scratch, state)
    return state[order], rho[order]


def compare(p_state, p_rho, l_state, l_rho, params) -> dict:
    rho0 = float(params["fluid_density"])
    h = float(params["h"])
    m = float(params["particle_mass"])
    dpos = l_state["position"][:, :3].astype(np.float64) - p_state["position"][:, :3]
    ke = lambda s: 0.5 * m * float((s["velocity"][:, :3].astype(np.float64) ** 2).sum())
    d_p = float(np.abs(p_rho / rho0 - 1).mean())
    d_l = float(np.abs(l_rho / rho0 - 1).mean())
    return {
        "density_dev": abs(d_l - d_p),
        "density_dev_particle": float(np.abs(l_rho.astype(np.float64) - p_rho).mean() / rho0),
        "density_dev_pop": float(abs(l_rho.astype(np.float64).mean() - p_rho.astype(np.float64).mean()) / rho0),
        "rho_dev_plain": d_p,
        "rho_dev_learned": d_l,
        "pos_rms_h": float(np.sqrt((dpos ** 2).sum(1).mean()) / h),
        "ke_plain": ke(p_state),
        "ke_learned": ke(l_state),
    }


def evaluate(scene, mlp: Lm.Mlp, plain_substeps: int = 2000, dt_mult: int = 4, checkpoints: int = 10,
             threshold: float = 0.01, graph: bool = True, check: bool = True) -> dict:
    import torch

    if plain_substeps % (dt_mult * checkpoints):
        raise ValueError("plain_substeps must be a multiple of dt_mult * checkpoints")
    learned_steps = plain_substeps // dt_mult
    dt = float(np.float32(scene.params["time_delta"]) * np.float32(scene.params["simulation_scale"]))
    sim_time = plain_substeps * dt

    def solver(particles=None):
        s = GpuSolver(scene.params, scene.terms, scene.n, scene.mesh)
        s.upload(scene.particles if particles is None else particles)
        return s

    perturbed = scene.particles.copy()
    rng = np.random.default_rng(12345)
    eps = 1e-6 * float(scene.params["h"])
    perturbed["position"][:, :3] += rng.uniform(-eps, eps, (scene.n, 3)).astype(np.float32)

    # ---- timing: the whole interval, wall clock around synchronised runs
    with solver() as p:
        p.set_graph(graph)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        p.step(plain_substeps)
        p.sync()
        plain_s = time.perf_counter() - t0
    with solver() as lr:
        lr.set_graph(graph)
        stats = Lm.LearnedStats()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        Lm.step_learned(lr, mlp, learned_steps, dt_mult, threshold, stats, check=check)
        lr.sync()
        learned_s = time.perf_counter() - t0
    # ---- accuracy: the same trajectories with checkpoints
    curve = []
    with solver() as p, solver() as lr, solver() as scratch, solver(perturbed) as pc:
        p.set_graph(graph)
        pc.set_graph(graph)
        lr.set_graph(graph)
        chk_stats = Lm.LearnedStats()
        per = plain_substeps // checkpoints
        h = float(scene.params["h"])
        for c in range(checkpoints):
            p.step(per)
            pc.step(per)
            Lm.step_learned(lr, mlp, per // dt_mult, dt_mult, threshold, chk_stats, check=check)
            ps, prho = by_id(p, scratch)
            ls, lrho = by_id(lr, scratch)
            cs, crho = by_id(pc, scratch)
            row = compare(ps, prho, ls, lrho, scene.params)
            chaos = compare(ps, prho, cs, crho, scene.params)
            row["pos_rms_chaos_h"] = chaos["pos_rms_h"]
            row["density_dev_chaos"] = chaos["density_dev"]
            row["t"] = (c + 1) * per * dt
            curve.append(row)
    st = stats.as_dict()
    out = {
        "workload": scene.name,
        "particles": scene.n,
        "dt_mult": dt_mult,
        "threshold": threshold if check else None,
        "plain_substeps": plain_substeps,
        "learned_steps": learned_steps,
        "sim_time_s": sim_time,
        "plain_wall_s": plain_s,
        "learned_wall_s": learned_s,
        "plain_sim_s_per_s": sim_time / plain_s,
        "learned_sim_s_per_s": sim_time / learned_s,
        "speedup": plain_s / learned_s,
        "plain_particle_steps_per_s": scene.n * plain_substeps / plain_s,
        "fallback_fraction": st["fallback_fraction"],
        "accepted_steps": st["learned_steps"],
        "rejected_steps": st["rejected"],
        "check_deviation_mean": st["deviation_mean"],
        "check_deviation_max": st["deviation_max"],
        "density_dev": float(np.mean([r["density_dev"] for r in curve])),
        "density_dev_max": float(np.max([r["density_dev"] for r in curve])),
        "density_dev_pop": float(np.mean([r["density_dev_pop"] for r in curve])),
        "density_dev_particle": float(np.mean([r["density_dev_particle"] for r in curve])),
        "rho_dev_plain": float(np.mean([r["rho_dev_plain"] for r in curve])),
        "rho_dev_learned": float(np.mean([r["rho_dev_learned"] for r in curve])),
        "pos_rms_h_final": curve[-1]["pos_rms_h"],
        "pos_rms_chaos_h_final": curve[-1]["pos_rms_chaos_h"],
        "density_dev_chaos": float(np.mean([r["density_dev_chaos"] for r in curve])),
        "check_particle_deviation_mean": st["particle_deviation_mean"],
        "curve": curve,
    }
    return out


def main(argv=None) -> int:
    """Command line: `--steps K` runs K learned steps of a workload and prints
    their statistics (a short run to profile the stepper's kernels);
    `--evaluate` runs the whole plain-versus-learned comparison instead."""
    import argparse
    import json

    from . import workloads as W

    scenes = {"dam_break_1m": W.dam_break_1m, "dam_break_32k": W.dam_break_32k}
    ap = argparse.ArgumentParser(prog="python -m libclsph_gb300.stepper_eval")
    ap.add_argument("--workload", default="dam_break_1m", choices=sorted(scenes))
    ap.add_argument("--steps", type=int, default=8, help="learned steps (without --evaluate)")
    ap.add_argument("--dt-mult", type=int, default=4)
    ap.add_argument("--threshold", type=float, default=0.01, help="density check; 1e30 disables it")
    ap.add_argument("--evaluate", action="store_true", help="plain vs learned over 2000 plain substeps")
    ap.add_argument("--weights", default=None)
    a = ap.parse_args(argv)

    scene = scenes[a.workload]()
    mlp = Lm.Mlp.load(a.weights)
    try:
        if a.evaluate:
            r = evaluate(scene, mlp, plain_substeps=2000, dt_mult=a.dt_mult, checkpoints=10,
                         threshold=a.threshold)
            r.pop("curve")
        else:
            import torch

            with GpuSolver(scene.params, scene.terms, scene.n, scene.mesh) as s:
                s.upload(scene.particles)
                st = Lm.step_learned(s, mlp, a.steps, a.dt_mult, a.threshold)
                s.sync()
                torch.cuda.synchronize()
            r = {"workload": scene.name, "particles": scene.n, "steps": a.steps,
                 "accepted_steps": st.learned_steps, "rejected": st.rejected}
    finally:
        mlp.close()
    print(json.dumps(r))
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
