"""Batched scenes and CUDA-graph replay (no counterpart in the reference).

Each scene of a batched handle must evolve exactly as the same scene in a
handle of its own: same grid, same sort order, same fields, bit for bit.
Graph replay of the substep must equal launching every kernel."""

import numpy as np
import pytest

from libclsph_gb300 import workloads as W
from libclsph_gb300.gpu import GpuSolver

pytestmark = pytest.mark.gpu


def scene_set(count=5, seed=40):
    rng = np.random.default_rng(seed)
    out = []
    for k in range(count):
        side = int(rng.integers(6, 14))
        sc = W.small_block(side, seed=seed + k, velocity_sigma=float(rng.uniform(0.05, 1.0)),
                           offset=(0.05 + 0.1 * rng.random(), 0.001 + 0.05 * rng.random(), 0.2))
        # per-scene fluid constants, as in the batched benchmark
        st = W.water_settings(sc.n, fluid_density=float(rng.uniform(900, 1200)),
                              dynamic_viscosity=float(3.5 * rng.uniform(0.5, 4.0)))
        sc.params, sc.terms = st.params, st.terms
        out.append(sc)
    return out


def test_batched_scenes_equal_separate_runs(gpu_lib):
    scenes = scene_set()
    steps = 6
    with GpuSolver.batched([s.params for s in scenes], [s.terms for s in scenes],
                           [s.n for s in scenes], [s.mesh for s in scenes]) as b:
        b.upload(np.concatenate([s.particles for s in scenes]))
        b.step(steps)
        assert b.sync() == 0
        out = b.download()
        prm = [b.parameters(k) for k in range(len(scenes))]
        tables = [b.cell_table(k) for k in range(len(scenes))]
    for k, sc in enumerate(scenes):
        with GpuSolver(sc.params, sc.terms, sc.n, sc.mesh) as g:
            g.upload(sc.particles)
            g.step(steps)
            ref = g.download()
            ref_prm = g.parameters()
            ref_table = g.cell_table()
        part = out[b.first[k]:b.first[k + 1]]
        assert np.array_equal(part.view(np.uint8), ref.view(np.uint8)), f"scene {k}"
        assert prm[k]["grid_cell_count"] == ref_prm["grid_cell_count"]
        assert np.array_equal(prm[k]["min_point"], ref_prm["min_point"])
        assert np.array_equal(tables[k], ref_table)


def test_batched_scene_matches_oracle(gpu_lib, oracle):
    scenes = scene_set(3, seed=60)
    with GpuSolver.batched([s.params for s in scenes], [s.terms for s in scenes],
                           [s.n for s in scenes], [s.mesh for s in scenes]) as b:
        b.upload(np.concatenate([s.particles for s in scenes]))
        b.step(1)
        out = b.download()
    for k, sc in enumerate(scenes):
        ref = oracle.step(sc.params, sc.terms, sc.particles, sc.mesh).final
        part = out[b.first[k]:b.first[k + 1]]
        assert np.array_equal(part["position"][:, :3], ref["position"][:, :3])
        assert np.array_equal(part["density"], ref["density"])


def test_batched_256_full_size_matches_oracle_per_scene(gpu_lib, oracle):
    """The batched workload at full size: one substep of the 256 dam breaks
    (4,703,741 particles, per-scene rest density and viscosity, one handle)
    against the oracle's substep of each scene on its own: every scene's
    sorted final state, density and pressure bit for bit."""
    scenes = W.batched_dam_breaks()
    with GpuSolver.batched([s.params for s in scenes], [s.terms for s in scenes],
                           [s.n for s in scenes], [s.mesh for s in scenes]) as b:
        b.upload(np.concatenate([s.particles for s in scenes]))
        b.step(1)
        assert b.sync() == 0
        out = b.download()
    for k, sc in enumerate(scenes):
        ref = oracle.step(sc.params, sc.terms, sc.particles, sc.mesh).final
        part = out[b.first[k]:b.first[k + 1]]
        for f in ("position", "velocity", "intermediate_velocity"):
            assert np.array_equal(part[f][:, :3], ref[f][:, :3]), (k, f)
        assert np.array_equal(part["density"], ref["density"]), k
        assert np.array_equal(part["pressure"], ref["pressure"]), k


@pytest.mark.parametrize("steps", [2, 7, 35])  # 35: two 16-substep replays, one of 2, one launch
def test_graph_replay_equals_launches(gpu_lib, steps):
    sc = W.small_block(14, seed=70, velocity_sigma=0.4)
    results = []
    for graph in (False, True):
        with GpuSolver(sc.params, sc.terms, sc.n, sc.mesh) as g:
            g.set_graph(graph)
            g.upload(sc.particles)
            g.step(steps)
            g.step(steps)
            results.append((g.download(), g.ids(), g.counters()))
    assert np.array_equal(results[0][0].view(np.uint8), results[1][0].view(np.uint8))
    assert np.array_equal(results[0][1], results[1][1])
    assert results[0][2]["substeps"] == results[1][2]["substeps"] == 2 * steps
    assert results[0][2]["launches"] == results[1][2]["launches"]  # replays count their kernels


def test_autotune_keeps_state_and_results(gpu_lib):
    sc = W.small_block(16, seed=80, velocity_sigma=0.3)
    with GpuSolver(sc.params, sc.terms, sc.n, sc.mesh) as g:
        g.upload(sc.particles)
        g.step(2)
        report = g.autotune(2)
        g.step(3)
        tuned = g.download()
        tuned_ids = g.ids()
    assert "chosen:" in report
    with GpuSolver(sc.params, sc.terms, sc.n, sc.mesh) as g:
        g.upload(sc.particles)
        g.step(5)
        plain = g.download()
        plain_ids = g.ids()
    assert np.array_equal(tuned.view(np.uint8), plain.view(np.uint8))
    assert np.array_equal(tuned_ids, plain_ids)


@pytest.mark.parametrize("shape", [(64, 64, 4), (256, 256, 16)])
def test_launch_shapes_do_not_change_results(gpu_lib, shape):
    sc = W.small_block(15, seed=81, velocity_sigma=0.3)
    outs = []
    for sh in (None, shape):
        with GpuSolver(sc.params, sc.terms, sc.n, sc.mesh) as g:
            if sh:
                g.set_launch_shape(*sh)
            g.upload(sc.particles)
            g.step(4)
            outs.append(g.download())
    assert np.array_equal(outs[0].view(np.uint8), outs[1].view(np.uint8))


def _run_mode(scenes, steps, persistent, density_block=None):
    with GpuSolver.batched([s.params for s in scenes], [s.terms for s in scenes],
                           [s.n for s in scenes], [s.mesh for s in scenes]) as b:
        if density_block is not None:
            b.set_launch_shape(density_block, 128, 8)
        b.set_persistent(persistent)
        b.upload(np.concatenate([s.particles for s in scenes]))
        b.step(steps)
        flags = b.sync()
        out = b.download()
        keys, perm = b.keys()
        ids = b.ids()
    return flags, out, keys, perm, ids


@pytest.mark.parametrize("steps", [1, 6, 67])
def test_persistent_substeps_equal_launched(gpu_lib, steps):
    """The persistent cooperative launch (every phase of the substep in one
    kernel, grid barriers between phases) against launched kernels, on
    scenes of uneven sizes: the state, the sort and the particle ids bit for
    bit (67 substeps span two launches of at most 64)."""
    scenes = scene_set(7, seed=70)
    want = _run_mode(scenes, steps, False, density_block=256)  # the same 8-warp density tiles
    got = _run_mode(scenes, steps, True)
    assert got[0] == want[0] == 0
    assert np.array_equal(got[1].view(np.uint8), want[1].view(np.uint8))
    for a, b in zip(got[2:], want[2:]):
        assert np.array_equal(a, b)


def test_persistent_dam_break_1m_equals_launched(gpu_lib):
    sc = W.dam_break_1m()
    want = _run_mode([sc], 4, False, density_block=256)
    got = _run_mode([sc], 4, True)
    assert got[0] == want[0] == 0
    assert np.array_equal(got[1].view(np.uint8), want[1].view(np.uint8))
    assert np.array_equal(got[4], want[4])


def test_persistent_barrier_wait_runs_out_and_reports(gpu_lib):
    """Block 0 leaves at the first grid barrier (a block that never arrives,
    through the barrier test hook), so every other block's bounded wait runs
    out; clsph_gpu_sync reports it and resets the barrier, and the same
    handle then steps exactly like a fresh one."""
    from libclsph_gb300.gpu import ClsphError

    scenes = scene_set(3, seed=75)
    parts = np.concatenate([s.particles for s in scenes])
    want = _run_mode(scenes, 2, True)
    with GpuSolver.batched([s.params for s in scenes], [s.terms for s in scenes],
                           [s.n for s in scenes], [s.mesh for s in scenes]) as b:
        b.set_persistent(True)
        b.set_barrier_limits(barrier_spins=256, withheld_block=0)
        b.upload(parts)
        b.step(1)
        with pytest.raises(ClsphError) as err:
            b.sync()
        assert err.value.code == 512 and "grid barrier" in str(err.value)
        b.set_barrier_limits()
        b.upload(parts)
        b.step(2)
        assert b.sync() == 0
        out = b.download()
    assert np.array_equal(out.view(np.uint8), want[1].view(np.uint8))
