"""GPU tests at the headline workloads' full sizes.

* One substep of the 1,048,576-particle dam break against the CPU oracle
  (OpenMP over particles; a few seconds): grid keys, sorted order and the
  dense cell table bit-exact, density, pressure, acceleration and the
  advected state bit for bit.
* Every neighbour-search mode gives the same bytes at full size (the 1M dam
  break after a few substeps, and the 4,194,304-particle pour onto a
  131,072-triangle heightfield, whose collisions the oracle cannot run at
  that size).
* Ten substeps of the 1M dam break against ten oracle substeps (chaotic in
  the long run, but bit for bit over ten substeps), and one substep from the
  state the GPU reached after 200 substeps against the oracle's substep from
  that state; the 32,768-particle dam break over 100 substeps in every
  neighbour-search mode.
* The GPU's FP32 density, pressure and acceleration of the 1M dam break
  reported against the FP64 oracle (the same algorithm in double): maximum
  and mean relative error per field, bounded at 1e-5 (density), 1e-4
  (pressure) and 1e-5 of the largest acceleration.
* Size-independent properties after several substeps: keys non-decreasing,
  the sort permutation and the particle ids are permutations, the cell table
  is the lower bound of every cell in the sorted keys, no device flags.
"""

import numpy as np
import pytest

from libclsph_gb300 import workloads as W
from libclsph_gb300.gpu import SEARCH_MODES, STAGE_FORCES, GpuSolver

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def dam_break():
    return W.dam_break_1m()


def test_dam_break_1m_substep_matches_oracle(gpu_lib, oracle, dam_break):
    sc = dam_break
    ref = oracle.step(sc.params, sc.terms, sc.particles, sc.mesh)
    with GpuSolver(sc.params, sc.terms, sc.n, sc.mesh) as g:
        g.upload(sc.particles)
        g.step_until(STAGE_FORCES)
        rho, prs, acc = g.fields()
        keys, perm = g.keys()
        table = g.cell_table()
        g.upload(sc.particles)
        g.step(1)
        assert g.sync() == 0
        out = g.download()
    assert np.array_equal(perm, ref.perm)
    assert np.array_equal(keys, ref.sorted["grid_index"])
    assert np.array_equal(table, ref.table)
    assert np.array_equal(rho, ref.forces["density"])
    assert np.array_equal(prs, ref.forces["pressure"])
    assert np.array_equal(acc, ref.forces["acceleration"][:, :3])
    for f in ("position", "velocity", "intermediate_velocity"):
        assert np.array_equal(out[f][:, :3], ref.final[f][:, :3]), f
    assert np.array_equal(out["density"], ref.final["density"])


def test_dam_break_1m_ten_substeps_match_oracle(gpu_lib, oracle, dam_break):
    sc = dam_break
    want = oracle.run(sc.params, sc.terms, sc.particles, 10, sc.mesh)
    with GpuSolver(sc.params, sc.terms, sc.n, sc.mesh) as g:
        g.upload(sc.particles)
        g.step(10)
        assert g.sync() == 0
        out = g.download()
    for f in ("position", "velocity", "intermediate_velocity"):
        assert np.array_equal(out[f][:, :3], want[f][:, :3]), f
    assert np.array_equal(out["density"], want["density"])
    assert np.array_equal(out["pressure"], want["pressure"])


def test_dam_break_32k_hundred_substeps_match_oracle(gpu_lib, oracle):
    """The 32,768-particle dam break over 100 substeps (the column falling
    onto the floor of its box, with wall and floor collisions) in every
    neighbour-search mode against 100 oracle substeps: state, density and
    pressure bit for bit."""
    sc = W.dam_break_32k()
    want = oracle.run(sc.params, sc.terms, sc.particles, 100, sc.mesh)
    for mode in SEARCH_MODES:
        with GpuSolver(sc.params, sc.terms, sc.n, sc.mesh) as g:
            g.set_neighbour_search(mode)
            g.upload(sc.particles)
            g.step(100)
            assert g.sync() == 0
            out = g.download()
        for f in ("position", "velocity", "intermediate_velocity"):
            assert np.array_equal(out[f][:, :3], want[f][:, :3]), (mode, f)
        assert np.array_equal(out["density"], want["density"]), mode
        assert np.array_equal(out["pressure"], want["pressure"]), mode


@pytest.mark.parametrize("density_block", [128, 256])
def test_dam_break_1m_collapsed_state_substep_matches_oracle(gpu_lib, oracle, dam_break, density_block):
    """One substep from the state the GPU reached after 200 substeps (the
    column collapsing onto the floor: cells of a few to over a hundred
    particles, second passes and tiles across ragged cells in the cell-warp
    search), with 4- and 8-warp density blocks, against the oracle's substep
    from the same state: sort, fields and advected state bit for bit."""
    sc = dam_break
    with GpuSolver(sc.params, sc.terms, sc.n, sc.mesh) as g:
        g.upload(sc.particles)
        g.step(200)
        assert g.sync() == 0
        state = g.download()
    ref = oracle.step(sc.params, sc.terms, state, sc.mesh)
    with GpuSolver(sc.params, sc.terms, sc.n, sc.mesh) as g:
        g.set_launch_shape(density_block, 128, 8)
        g.upload(state)
        g.step_until(STAGE_FORCES)
        rho, prs, acc = g.fields()
        keys, perm = g.keys()
        g.upload(state)
        g.step(1)
        assert g.sync() == 0
        out = g.download()
    assert np.array_equal(perm, ref.perm)
    assert np.array_equal(keys, ref.sorted["grid_index"])
    assert np.array_equal(rho, ref.forces["density"])
    assert np.array_equal(prs, ref.forces["pressure"])
    assert np.array_equal(acc, ref.forces["acceleration"][:, :3])
    for f in ("position", "velocity", "intermediate_velocity"):
        assert np.array_equal(out[f][:, :3], ref.final[f][:, :3]), f
    assert np.array_equal(out["density"], ref.final["density"])


def fp64_report(rho, prs, acc, rho64, prs64, acc64):
    """Relative errors of FP32 fields against FP64 ones: per particle for
    density; for the pressure per particle and against the field's largest
    magnitude (the Tait pressure K((rho/rho0)^7 - 1) passes through zero at
    rho0, where its per-particle relative error is unbounded); per particle as
    |a - a64| / |a64| (median, max) and against the field's largest magnitude
    for the acceleration, whose sums cancel."""
    def rel(x, y):
        e = np.abs(x.astype(np.float64) - y)
        return e / np.maximum(np.abs(y), 1e-30)

    da = np.linalg.norm(acc.astype(np.float64) - acc64, axis=1)
    na = np.linalg.norm(acc64, axis=1)
    r_rho, r_p = rel(rho, rho64), rel(prs, prs64)
    return {
        "density": {"max_rel": float(r_rho.max()), "mean_rel": float(r_rho.mean())},
        "pressure": {"max_rel": float(r_p.max()), "mean_rel": float(r_p.mean()),
                     "max_abs_over_max": float(np.abs(prs.astype(np.float64) - prs64).max() / np.abs(prs64).max())},
        "acceleration": {"max_abs_over_max": float(da.max() / na.max()),
                         "median_rel": float(np.median(da / np.maximum(na, 1e-30))),
                         "max_rel": float((da / np.maximum(na, 1e-30)).max())},
    }


@pytest.mark.parametrize("after", [0, 200])
def test_dam_break_1m_fields_against_fp64_oracle(gpu_lib, oracle, dam_break, after):
    """FP32 density, pressure and acceleration of one substep against the
    FP64 restatement on the same sorted input: from the lattice, and from the
    state the GPU reached after 200 substeps (the column collapsing)."""
    sc = dam_break
    start = sc.particles
    if after:
        with GpuSolver(sc.params, sc.terms, sc.n, sc.mesh) as g:
            g.upload(sc.particles)
            g.step(after)
            assert g.sync() == 0
            start = g.download()
    ref = oracle.step(sc.params, sc.terms, start, sc.mesh)
    rho64, prs64, acc64 = oracle.fields_f64(ref.params, ref.sorted, ref.table)
    with GpuSolver(sc.params, sc.terms, sc.n, sc.mesh) as g:
        g.upload(start)
        g.step_until(STAGE_FORCES)
        rho, prs, acc = g.fields()
        _, perm = g.keys()
    assert np.array_equal(perm, ref.perm)  # the FP64 fields are of the same sorted state
    rep = fp64_report(rho, prs, acc, rho64, prs64, acc64)
    print(f"FP32 GPU fields vs FP64 oracle, 1,048,576-particle dam break after {after} substeps:", rep)
    assert rep["density"]["max_rel"] <= 1e-5
    assert rep["pressure"]["max_abs_over_max"] <= 1e-5
    assert rep["acceleration"]["max_abs_over_max"] <= 1e-5
    assert rep["acceleration"]["median_rel"] <= 1e-4


def _run(sc, mode, substeps):
    with GpuSolver(sc.params, sc.terms, sc.n, sc.mesh) as g:
        g.set_neighbour_search(mode)
        g.upload(sc.particles)
        g.step(substeps)
        flags = g.sync()
        out = g.download()
        keys, perm = g.keys()
        ids = g.ids()
        table = g.cell_table()
    return flags, out, keys, perm, ids, table


def test_dam_break_1m_search_modes_identical_and_consistent(gpu_lib, dam_break):
    sc = dam_break
    runs = [_run(sc, m, 6) for m in SEARCH_MODES]
    base = runs[0]
    for r in runs[1:]:
        assert np.array_equal(r[1].view(np.uint8), base[1].view(np.uint8))
        assert np.array_equal(r[4], base[4])
    flags, out, keys, perm, ids, table = base
    assert flags == 0
    assert np.all(np.diff(keys.astype(np.int64)) >= 0)
    n = sc.n
    assert np.array_equal(np.sort(perm), np.arange(n, dtype=np.uint32))
    assert np.array_equal(np.sort(ids), np.arange(n, dtype=np.uint32))
    # table[c] = first sorted slot with key >= c (sph_simulation.cpp:162-170)
    cells = np.arange(len(table), dtype=np.uint32)
    assert np.array_equal(table, np.searchsorted(keys, cells, side="left").astype(np.uint32))
    assert np.all(np.isfinite(out["position"][:, :3]))


def test_pour_4m_search_modes_identical(gpu_lib):
    sc = W.pour()
    runs = [_run(sc, m, 2) for m in SEARCH_MODES]
    for r in runs[1:]:
        assert np.array_equal(r[1].view(np.uint8), runs[0][1].view(np.uint8))
    assert runs[0][0] == 0
    assert np.all(np.diff(runs[0][2].astype(np.int64)) >= 0)
