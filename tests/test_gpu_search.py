"""GPU parity of the density kernel's neighbour search modes.

Both modes (one thread per particle over its window; one warp per cell with
the neighbour cells staged in shared memory) must give the oracle's fields
bit for bit, including scenes that exercise the rare paths: particles on the
cells' mid-planes (both half bits set), candidate buffer overflow and a cell
too crowded for the cell-warp buffers (both take the in-order rescan).
"""

import numpy as np
import pytest

from libclsph_gb300 import workloads as W
from libclsph_gb300.gpu import SEARCH_CELL_WARPS, SEARCH_MODES, STAGE_FORCES, GpuSolver

pytestmark = pytest.mark.gpu


def _fields(scene, mode, stage=STAGE_FORCES):
    with GpuSolver(scene.params, scene.terms, scene.n, scene.mesh) as g:
        g.set_neighbour_search(mode)
        g.upload(scene.particles)
        g.step_until(stage)
        assert g.sync() == 0
        return g.fields()


def _aligned_block(n_side: int) -> W.Scene:
    """A block without jitter at spacing h/2: a quarter of the 2h cell, so one
    lattice plane in four lies on a cell mid-plane (within the rounding margin
    of both halves)."""
    st = W.water_settings(n_side ** 3)
    h = float(st.params["h"])
    pos = W.lattice((n_side,) * 3, h * 0.5, (0.25, 0.25, 0.25), 0.0, np.random.default_rng(0))
    parts = W.particles_from_arrays(pos, None, None)
    return W.Scene(f"aligned_{n_side ** 3}", st.params, st.terms, parts,
                   W.box_mesh((0, 0, 0), (1, 1, 1)), 10, {"h": h})


@pytest.mark.parametrize("mode", SEARCH_MODES)
def test_search_modes_match_oracle(gpu_lib, oracle, mode):
    scene = W.small_block(16, seed=14, velocity_sigma=0.3)
    ref = oracle.step(scene.params, scene.terms, scene.particles, scene.mesh)
    rho, prs, acc = _fields(scene, mode)
    assert np.array_equal(rho, ref.forces["density"])
    assert np.array_equal(prs, ref.forces["pressure"])
    assert np.array_equal(acc, ref.forces["acceleration"][:, :3])


@pytest.mark.parametrize("mode", SEARCH_MODES)
def test_search_modes_mid_plane_particles(gpu_lib, oracle, mode):
    scene = _aligned_block(12)
    ref = oracle.step(scene.params, scene.terms, scene.particles, scene.mesh)
    rho, prs, acc = _fields(scene, mode)
    assert np.array_equal(rho, ref.forces["density"])
    assert np.array_equal(acc, ref.forces["acceleration"][:, :3])


@pytest.mark.parametrize("mode", SEARCH_MODES)
def test_search_modes_compressed_overflow(gpu_lib, oracle, mode):
    # spacing h/4: about 270 neighbours, far beyond the 48-entry candidate buffer
    scene = W.small_block(12, seed=15, velocity_sigma=0.1, spacing_frac=0.25)
    ref = oracle.step(scene.params, scene.terms, scene.particles, scene.mesh)
    rho, prs, acc = _fields(scene, mode)
    assert np.array_equal(rho, ref.forces["density"])
    assert np.array_equal(acc, ref.forces["acceleration"][:, :3])


@pytest.mark.parametrize("mode", SEARCH_MODES)
def test_search_modes_crowded_cell(gpu_lib, oracle, mode):
    # 3,000 particles inside one 2h cell: more than a cell-warp buffer entry can
    # address (2,048), so every particle takes the in-order rescan
    st = W.water_settings(3000)
    h = float(st.params["h"])
    rng = np.random.default_rng(16)
    pos = (0.5 + rng.uniform(0.0, 0.5 * h, (3000, 3))).astype(np.float32)
    parts = W.particles_from_arrays(pos, None, None)
    scene = W.Scene("one_cell", st.params, st.terms, parts, W.box_mesh((0, 0, 0), (1, 1, 1)), 10, {})
    ref = oracle.step(scene.params, scene.terms, scene.particles, scene.mesh)
    rho, prs, acc = _fields(scene, mode)
    assert np.array_equal(rho, ref.forces["density"])
    assert np.array_equal(acc, ref.forces["acceleration"][:, :3])


def _random_cloud(n: int, seed: int, per_cell: float = 64.0) -> W.Scene:
    """n particles placed uniformly at random in a cube sized for a mean of
    per_cell particles per 2h cell (64 is the lattice's): cell counts scatter
    around it, so the cell-warp search packs its tiles across cells of ragged
    sizes and takes second passes for cells above 64."""
    st = W.water_settings(n)
    h = float(st.params["h"])
    side = (n / per_cell) ** (1.0 / 3.0) * 2.0 * h
    rng = np.random.default_rng(seed)
    pos = (0.2 + rng.uniform(0.0, side, (n, 3))).astype(np.float32)
    vel = rng.normal(0.0, 0.2, pos.shape).astype(np.float32)
    parts = W.particles_from_arrays(pos, vel, vel)
    return W.Scene(f"cloud_{n}", st.params, st.terms, parts, W.box_mesh((0, 0, 0), (1, 1, 1)), 10, {"h": h})


CELL_WARP_SCENES = {
    # cells of about 48 to 93 particles, 30 neighbours on average
    "random_cloud": lambda: _random_cloud(8000, seed=17),
    # about 46 neighbours on average: many particles fill the 8-warp block's
    # 40-entry survivor buffer and some the 48-entry one of 2/4-warp blocks
    "dense_cloud": lambda: _random_cloud(8000, seed=18, per_cell=96.0),
    "mid_planes": lambda: _aligned_block(12),
}


@pytest.mark.parametrize("density_block", [64, 128, 256])
@pytest.mark.parametrize("name", sorted(CELL_WARP_SCENES))
def test_cell_warp_blocks_match_oracle(gpu_lib, oracle, name, density_block):
    """The cell-warp search with 2-, 4- and 8-warp blocks (the 8-warp block's
    survivor buffer is shorter) against the oracle, on scenes whose cells are
    ragged, whose particles sit near the buffers' capacity, or on mid-planes."""
    scene = CELL_WARP_SCENES[name]()
    ref = oracle.step(scene.params, scene.terms, scene.particles, scene.mesh)
    with GpuSolver(scene.params, scene.terms, scene.n, scene.mesh) as g:
        g.set_neighbour_search(SEARCH_CELL_WARPS)
        g.set_launch_shape(density_block, 128, 8)
        g.upload(scene.particles)
        g.step_until(STAGE_FORCES)
        assert g.sync() == 0
        rho, prs, acc = g.fields()
    assert np.array_equal(rho, ref.forces["density"])
    assert np.array_equal(prs, ref.forces["pressure"])
    assert np.array_equal(acc, ref.forces["acceleration"][:, :3])
