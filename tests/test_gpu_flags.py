"""GPU tests of the engine's warning flags (CLSPH_WARN_*), which replace the
reference's asserts and its unbounded collision loop:

* a grid axis of 1024 cells or more (sph_simulation.cpp:247-249 asserts);
* non-finite particle coordinates in the uploaded state;
* the advection/collision loop reaching its iteration cap (sph.cl:82-101 has
  no cap).

Every case keeps all device accesses in bounds: coordinates beyond 1023 cells
alias through the 10-bit Morton masks, non-finite positions fail every
distance comparison, and a capped loop simply stops.
"""

import numpy as np
import pytest

from libclsph_gb300 import workloads as W
from libclsph_gb300.gpu import (SEARCH_MODES, WARN_COLLISION_CAP, WARN_GRID_OVERFLOW, WARN_NONFINITE,
                                GpuSolver)

pytestmark = pytest.mark.gpu

EMPTY = {"vertices": np.zeros(0, np.float32), "indices": np.zeros(0, np.uint32),
         "face_normals": np.zeros(0, np.float32)}


def test_grid_overflow_is_flagged(gpu_lib):
    st = W.water_settings(2 * 125)
    h = float(st.params["h"])
    rng = np.random.default_rng(51)
    a = W.lattice((5, 5, 5), 0.5 * h, (0.0, 0.0, 0.0), 0.01, rng)
    b = W.lattice((5, 5, 5), 0.5 * h, (1100 * 2 * h, 0.0, 0.0), 0.01, rng)  # about 1100 cells apart
    parts = W.particles_from_arrays(np.concatenate([a, b]))
    for mode in SEARCH_MODES:
        with GpuSolver(st.params, st.terms, len(parts), EMPTY) as g:
            g.set_neighbour_search(mode)
            g.upload(parts)
            g.step(2)
            flags = g.sync()
            out = g.download()
        assert flags & WARN_GRID_OVERFLOW
        assert np.all(np.isfinite(out["position"][:, :3]))


def test_nonfinite_input_is_flagged(gpu_lib):
    sc = W.small_block(8, seed=52, velocity_sigma=0.1)
    parts = sc.particles.copy()
    parts["position"][17, 0] = np.nan
    with GpuSolver(sc.params, sc.terms, sc.n, sc.mesh) as g:
        g.upload(parts)
        assert g.sync() & WARN_NONFINITE
        g.step(1)
        flags = g.sync()
        out = g.download()
    assert flags & WARN_NONFINITE
    # the other particles still move: one NaN does not poison its neighbours
    assert np.isfinite(out["position"][:, :3]).all(axis=1).sum() == sc.n - 1


def test_collision_cap_is_flagged_and_counted(gpu_lib):
    # a block thrown at the floor of the box: with the loop capped at one pass
    # every particle that hits the wall stops early
    sc = W.small_block(8, seed=53, offset=(0.3, -0.012, 0.3))  # bottom layer 3.5 mm above the floor
    parts = sc.particles.copy()
    parts["velocity"][:, 1] = -5.0
    parts["intermediate_velocity"][:, 1] = -5.0
    with GpuSolver(sc.params, sc.terms, sc.n, sc.mesh) as g:
        g.set_collision_cap(1)
        g.upload(parts)
        g.step(1)
        flags = g.sync()
        capped = g.counters()["collision_capped"]
    assert flags & WARN_COLLISION_CAP
    assert capped > 0
    with GpuSolver(sc.params, sc.terms, sc.n, sc.mesh) as g:  # the default cap is not reached
        g.upload(parts)
        g.step(1)
        assert g.sync() & WARN_COLLISION_CAP == 0


def test_argument_errors_are_reported(gpu_lib):
    from libclsph_gb300.gpu import ClsphError

    sc = W.small_block(4, seed=54)
    with pytest.raises(ClsphError):
        GpuSolver(sc.params, sc.terms, 0, sc.mesh)  # no particles
    with GpuSolver(sc.params, sc.terms, sc.n, sc.mesh) as g:
        with pytest.raises(ClsphError):
            g.set_neighbour_search(99)
        with pytest.raises(ClsphError):
            g.step(1)  # nothing uploaded yet
        with pytest.raises(ValueError):
            g.upload(sc.particles[:-1])  # wrong count
        g.upload(sc.particles)
        g.step(1)
        assert g.sync() == 0
