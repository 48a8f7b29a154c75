"""GPU parity: the CUDA substep (through the C ABI) against the CPU oracle.

Bar: bit for bit. Grid keys, sorted order and cell offsets are integer
work; density, pressure, acceleration and the advected state are too,
because the engine evaluates every contributing pair in the reference's
expression order with IEEE round-to-nearest operations (no contraction into
FMAs) and sums them in the reference's visiting order. A mismatch reports
the largest difference relative to the field's largest magnitude.
"""

import numpy as np
import pytest

from libclsph_gb300 import workloads as W
from libclsph_gb300.gpu import STAGE_DENSITY, STAGE_FORCES, STAGE_SORT, GpuSolver

pytestmark = pytest.mark.gpu

def rel_err(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    scale = np.abs(b).max() if b.size else 0.0
    return float(np.abs(a - b).max() / scale) if scale > 0 else float(np.abs(a - b).max())


def assert_same(a, b, what=""):
    """a and b equal bit for bit (NaN nowhere); on a mismatch the message
    gives the largest difference relative to b's largest magnitude."""
    a, b = np.asarray(a), np.asarray(b)
    assert a.shape == b.shape, (what, a.shape, b.shape)
    assert np.array_equal(a, b), f"{what}: max rel diff {rel_err(a, b):.3g}"


def scenes():
    yield W.small_block(16, seed=1, velocity_sigma=0.05)          # 4096, free fall
    yield W.small_block(10, seed=2, velocity_sigma=0.5,            # 1000, near the floor
                        offset=(0.2, 0.0005, 0.2))
    yield W.small_block(12, seed=3, velocity_sigma=2.0,            # fast, wall contacts
                        offset=(0.0005, 0.0005, 0.0005), spacing_frac=0.45)


@pytest.mark.parametrize("scene", list(scenes()), ids=lambda s: s.name)
def test_single_substep_matches_oracle(gpu_lib, oracle, scene):
    ref = oracle.step(scene.params, scene.terms, scene.particles, scene.mesh)
    with GpuSolver(scene.params, scene.terms, scene.n, scene.mesh) as g:
        g.upload(scene.particles)
        g.step(1)
        assert g.sync() == 0
        keys, perm = g.keys()
        table = g.cell_table()
        out = g.download()
        prm = g.parameters()
    assert np.array_equal(keys, ref.sorted["grid_index"])
    assert np.array_equal(perm, ref.perm)
    assert np.array_equal(table, ref.table)
    for f in ("grid_size_x", "grid_size_y", "grid_size_z", "grid_cell_count"):
        assert prm[f] == ref.params[f]
    assert np.array_equal(prm["min_point"][:3], ref.params["min_point"][:3])
    for f in ("position", "velocity", "intermediate_velocity"):
        assert_same(out[f][:, :3], ref.final[f][:, :3], f)
    for f in ("density", "pressure"):
        assert_same(out[f], ref.final[f], f)
    assert np.array_equal(out["grid_index"], ref.final["grid_index"])
    assert not out["acceleration"].any()


@pytest.mark.parametrize("scene", list(scenes())[:2], ids=lambda s: s.name)
def test_stages_match_oracle(gpu_lib, oracle, scene):
    ref = oracle.step(scene.params, scene.terms, scene.particles, scene.mesh)
    with GpuSolver(scene.params, scene.terms, scene.n, scene.mesh) as g:
        g.upload(scene.particles)
        g.step_until(STAGE_SORT)
        keys, perm = g.keys()
        assert np.array_equal(perm, ref.perm)
        g.upload(scene.particles)
        g.step_until(STAGE_DENSITY)
        rho, prs, _ = g.fields()
        g.upload(scene.particles)
        g.step_until(STAGE_FORCES)
        _, _, acc = g.fields()
    assert_same(rho, ref.density["density"], "density")
    assert_same(prs, ref.density["pressure"], "pressure")
    assert_same(acc, ref.forces["acceleration"][:, :3], "acceleration")


def test_fields_bit_exact(gpu_lib, oracle):
    scene = W.small_block(16, seed=4, velocity_sigma=0.3)
    ref = oracle.step(scene.params, scene.terms, scene.particles, scene.mesh)
    with GpuSolver(scene.params, scene.terms, scene.n, scene.mesh) as g:
        g.upload(scene.particles)
        g.step_until(STAGE_FORCES)
        rho, prs, acc = g.fields()
    assert np.array_equal(rho, ref.forces["density"])
    assert np.array_equal(prs, ref.forces["pressure"])
    assert np.array_equal(acc, ref.forces["acceleration"][:, :3])


def test_multi_substep_trajectory(gpu_lib, oracle):
    scene = W.small_block(12, seed=5, velocity_sigma=0.2)
    steps = 20
    with GpuSolver(scene.params, scene.terms, scene.n, scene.mesh) as g:
        g.upload(scene.particles)
        g.step(steps)
        assert g.sync() == 0
        out = g.download()
        ids = g.ids()
    ref = oracle.run(scene.params, scene.terms, scene.particles, steps, scene.mesh)
    # identical arithmetic keeps the chaotic trajectory on the oracle's
    assert_same(out["position"][:, :3], ref["position"][:, :3], "position")
    assert_same(out["velocity"][:, :3], ref["velocity"][:, :3], "velocity")
    # ids are a permutation that follows the particles
    assert np.array_equal(np.sort(ids), np.arange(scene.n, dtype=np.uint32))


@pytest.mark.parametrize("n_side", [1, 2, 5, 7])
def test_tiny_and_ragged_counts(gpu_lib, oracle, n_side):
    scene = W.small_block(n_side, seed=6, velocity_sigma=0.1)
    ref = oracle.step(scene.params, scene.terms, scene.particles, scene.mesh)
    with GpuSolver(scene.params, scene.terms, scene.n, scene.mesh) as g:
        g.upload(scene.particles)
        g.step(1)
        keys, perm = g.keys()
        out = g.download()
    assert np.array_equal(perm, ref.perm)
    assert_same(out["position"][:, :3], ref.final["position"][:, :3], "position")
    assert_same(out["density"], ref.final["density"], "density")


def test_no_mesh(gpu_lib, oracle):
    scene = W.small_block(8, seed=8, velocity_sigma=0.1)
    empty = {"vertices": np.zeros(0, np.float32), "indices": np.zeros(0, np.uint32),
             "face_normals": np.zeros(0, np.float32)}
    ref = oracle.step(scene.params, scene.terms, scene.particles, None)
    with GpuSolver(scene.params, scene.terms, scene.n, empty) as g:
        g.upload(scene.particles)
        g.step(1)
        out = g.download()
    assert_same(out["position"][:, :3], ref.final["position"][:, :3], "position")


def test_wide_grid_four_radix_passes(gpu_lib, oracle):
    # two blobs about 260 cells apart along x: Morton keys above 2^24, so the
    # sort takes all four 8-bit passes; sparse grid, no mesh
    st = W.water_settings(2 * 216)
    h = float(st.params["h"])
    rng = np.random.default_rng(41)
    a = W.lattice((6, 6, 6), 0.5 * h, (0.0, 0.0, 0.0), 0.01, rng)
    b = W.lattice((6, 6, 6), 0.5 * h, (260 * 2 * h, 0.0, 0.0), 0.01, rng)
    vel = rng.normal(0.0, 0.2, (2 * 216, 3)).astype(np.float32)
    parts = W.particles_from_arrays(np.concatenate([a, b]), vel, vel)
    scene = W.Scene("wide_432", st.params, st.terms, parts, None, 10, {"h": h})
    ref = oracle.step(scene.params, scene.terms, scene.particles, None)
    empty = {"vertices": np.zeros(0, np.float32), "indices": np.zeros(0, np.uint32),
             "face_normals": np.zeros(0, np.float32)}
    with GpuSolver(scene.params, scene.terms, scene.n, empty) as g:
        g.upload(scene.particles)
        g.step(1)
        assert g.sync() == 0
        keys, perm = g.keys()
        table = g.cell_table()
        out = g.download()
    assert int(keys.max()) >= 1 << 24  # the fourth pass ran
    assert np.array_equal(keys, ref.sorted["grid_index"])
    assert np.array_equal(perm, ref.perm)
    assert np.array_equal(table, ref.table)
    for f in ("position", "velocity", "intermediate_velocity"):
        assert np.array_equal(out[f][:, :3], ref.final[f][:, :3]), f
    assert np.array_equal(out["density"], ref.final["density"])
