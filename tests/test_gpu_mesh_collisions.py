"""Mesh collisions on dense meshes: the GPU's per-cell face lists against the
oracle's scan over every face (libclsph/kernels/collisions.cl:15-129, the
nearest hit over all faces in face order, a later face winning a tie).

* the reference's dense scenes (monkey.obj, shower.obj, labyrinth.obj,
  river.obj; their meshes and aimed particles come from the golden fixtures,
  whose first substep tests/test_gpu_golden.py checks against the reference
  build) over four substeps, in which particles that hit slide along the
  surface and hit again;
* a sample of the 4,194,304-particle pour: 12,288 particles of the pour's
  64 x 64 column cross-section, three layers deep, placed just above the full
  256 x 256-quad heightfield (131,072 triangles plus the 12 of the box) with
  the pour's velocities, over four substeps: keys, order and cell table of the
  first substep and every state bit for bit.

* the per-cell triangle lists themselves, built on the GPU by
  clsph_gpu_set_scene_mesh, against a numpy restatement of their definition
  (every face whose box, grown by pad + tolerance, meets the cell, in
  ascending order) on every one of these meshes: CSR starts and lists equal.

The pour's maximum speed (0.8 h per frame interval, h = 2.7 mm) is 0.13 m/s,
so a particle travels 0.22 mm per substep; the bottom layer starts 0.01 to
0.8 mm above the surface, so it reaches the heightfield within these four
substeps.
"""

from pathlib import Path

import numpy as np
import pytest

from libclsph_gb300 import workloads as W
from libclsph_gb300.gpu import GpuSolver
from libclsph_gb300.layout import particles_from_arrays

pytestmark = pytest.mark.gpu

GOLDEN = Path(__file__).resolve().parent / "golden"
MESH_CASES = ["monkey_hits", "shower_hits", "labyrinth_hits", "river_hits"]


def rel_err(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    scale = np.abs(b).max() if b.size else 0.0
    return float(np.abs(a - b).max() / scale) if scale > 0 else float(np.abs(a - b).max())


def assert_same_state(out, want):
    """Bit for bit; a mismatch reports the largest relative difference."""
    for f in ("position", "velocity", "intermediate_velocity"):
        a, b = out[f][:, :3], want[f][:, :3]
        assert np.array_equal(a, b), f"{f}: max rel diff {rel_err(a, b):.3g}"
    for f in ("density", "pressure"):
        assert np.array_equal(out[f], want[f]), f"{f}: max rel diff {rel_err(out[f], want[f]):.3g}"
    assert np.array_equal(out["grid_index"], want["grid_index"])


@pytest.mark.parametrize("name", MESH_CASES)
def test_reference_scene_collisions_over_substeps(gpu_lib, oracle, name):
    d = np.load(GOLDEN / f"{name}.npz")
    params, terms, parts = d["params"][0], d["terms"][0], d["particles"]
    mesh = {"vertices": d["vertices"], "indices": d["indices"], "face_normals": d["face_normals"]}
    want = oracle.run(params, terms, parts, 4, mesh)
    with GpuSolver(params, terms, len(parts), mesh) as g:
        g.upload(parts)
        g.step(4)
        assert g.sync() == 0
        out = g.download()
    assert_same_state(out, want)


def heightfield_surface(mesh, quads, x, z, extent=4.0):
    """Height of the pour's heightfield triangles at (x, z): quad (i, j) is
    split along the diagonal from vertex (i + 1, j) to (i, j + 1)
    (workloads.heightfield_mesh)."""
    Y = mesh["vertices"].reshape(-1, 3)[: (quads + 1) ** 2, 1].astype(np.float64)
    Y = Y.reshape(quads + 1, quads + 1)
    q = extent / quads
    i = np.clip((x / q).astype(np.int64), 0, quads - 1)
    j = np.clip((z / q).astype(np.int64), 0, quads - 1)
    u = x / q - i
    w = z / q - j
    ya, yb, yc, yd = Y[i, j], Y[i, j + 1], Y[i + 1, j], Y[i + 1, j + 1]
    lower = ya + u * (yc - ya) + w * (yb - ya)
    upper = yd + (1 - u) * (yb - yd) + (1 - w) * (yc - yd)
    return np.where(u + w <= 1.0, lower, upper)


def pour_sample(cross=64, layers=3, seed=3):
    """The pour's column cross-section, `layers` deep, just above the full
    heightfield, with the pour's velocities (2 m/s down, +-5 % per particle)."""
    sc = W.pour(cross=cross, length=1024, seed=seed)
    s = float(sc.info["spacing"])
    rng = np.random.default_rng(seed + 100)
    pos = W.lattice((cross, layers, cross), s, (2.0 - cross * s / 2, 0.0, 2.0 - cross * s / 2),
                    0.01, rng).astype(np.float64)
    layer = np.rint(pos[:, 1] / s - 0.5)
    surface = heightfield_surface(sc.mesh, 256, pos[:, 0], pos[:, 2])
    pos[:, 1] = surface + rng.uniform(1e-5, 8e-4, len(pos)) + layer * s
    n = len(pos)
    vel = np.zeros((n, 3), dtype=np.float32)
    vel[:, 1] = -2.0 * (1.0 + rng.uniform(-0.05, 0.05, n))
    st = W.water_settings(n, mass=float(sc.info["mass"]))
    return st, particles_from_arrays(pos.astype(np.float32), vel, vel), sc.mesh


def test_pour_sample_on_full_heightfield(gpu_lib, oracle):
    st, parts, mesh = pour_sample()
    assert len(mesh["indices"]) // 3 == 131072 + 12
    first = oracle.step(st.params, st.terms, parts, mesh)
    want = oracle.run(st.params, st.terms, parts, 4, mesh)
    with GpuSolver(st.params, st.terms, len(parts), mesh) as g:
        g.upload(parts)
        g.step(1)
        assert g.sync() == 0
        keys, perm = g.keys()
        table = g.cell_table()
        out1 = g.download()
        g.step(3)
        assert g.sync() == 0
        out4 = g.download()
    assert np.array_equal(perm, first.perm)
    assert np.array_equal(keys, first.sorted["grid_index"])
    assert np.array_equal(table, first.table)
    assert_same_state(out1, first.final)
    assert_same_state(out4, want)
    # the sample exercises the collision loop: about 1,000 particles end the
    # first substep away from their free flight x + v' dt
    dt = np.float32(st.params["time_delta"]) * np.float32(st.params["simulation_scale"])
    v = (first.sorted["intermediate_velocity"][:, :3].astype(np.float64)
         + first.forces["acceleration"][:, :3].astype(np.float64) * dt)
    sp = np.linalg.norm(v, axis=1, keepdims=True)
    vmax = float(st.params["max_velocity"])
    v = np.where(sp > vmax, v / np.maximum(sp, 1e-30) * vmax, v)
    free = first.sorted["position"][:, :3].astype(np.float64) + v * dt
    assert np.sum(np.linalg.norm(first.final["position"][:, :3] - free, axis=1) > 1e-5) > 500


def face_lists_numpy(mesh, plan):
    """CSR lists of the plan's grid: face f is in every cell of
    [floor((((min_a - pad) - tol) - glo_a) / cell), the same for max_a + pad
    + tol], clamped to the grid, per axis (float32 operations in that order),
    faces in ascending order."""
    v = np.asarray(mesh["vertices"], np.float32).reshape(-1, 3)
    t = np.asarray(mesh["indices"], np.int64).reshape(-1, 3)
    tri = v[t]  # faces x 3 x 3
    f32 = np.float32
    pad, tol, cell = f32(plan["pad"]), f32(plan["tol"]), f32(plan["cell"])
    glo = plan["glo"].astype(np.float32)
    dims = plan["dims"]
    mn = (tri.min(axis=1) - pad) - tol
    mx = (tri.max(axis=1) + pad) + tol
    c0 = np.floor((mn - glo) / cell).astype(np.int64)
    c1 = np.floor((mx - glo) / cell).astype(np.int64)
    c0 = np.clip(c0, 0, dims - 1)
    c1 = np.clip(c1, 0, dims - 1)
    cells, faces = [], []
    span = c1 - c0 + 1
    for f in range(len(t)):
        zs = np.arange(c0[f, 2], c1[f, 2] + 1)
        ys = np.arange(c0[f, 1], c1[f, 1] + 1)
        xs = np.arange(c0[f, 0], c1[f, 0] + 1)
        z, y, x = np.meshgrid(zs, ys, xs, indexing="ij")
        cells.append(((z * dims[1] + y) * dims[0] + x).ravel())
        faces.append(np.full(int(np.prod(span[f])), f, np.int64))
    cells = np.concatenate(cells)
    faces = np.concatenate(faces)
    order = np.argsort(cells, kind="stable")  # faces stay ascending within a cell
    ncell = int(np.prod(dims))
    start = np.zeros(ncell + 1, np.int64)
    start[1:] = np.cumsum(np.bincount(cells, minlength=ncell))
    return start.astype(np.uint32), faces[order].astype(np.uint32)


def _mesh_cases():
    for name in MESH_CASES:
        d = np.load(GOLDEN / f"{name}.npz")
        yield name, d["params"][0], d["terms"][0], {"vertices": d["vertices"], "indices": d["indices"],
                                                    "face_normals": d["face_normals"]}
    sc = W.pour(cross=8, length=8)
    yield "pour_heightfield", sc.params, sc.terms, sc.mesh
    sc = W.small_block(4)
    yield "box", sc.params, sc.terms, sc.mesh


@pytest.mark.parametrize("case", list(range(6)))
def test_face_lists_built_on_gpu_match_restatement(gpu_lib, case):
    name, params, terms, mesh = list(_mesh_cases())[case]
    with GpuSolver(params, terms, 128, mesh) as g:
        plan, start, faces = g.face_lists()
    assert plan is not None, name
    want_start, want_faces = face_lists_numpy(mesh, plan)
    assert np.array_equal(start, want_start), name
    assert np.array_equal(faces, want_faces), name
