"""Generates the golden fixtures of tests/golden/ from oracle/_ref.

oracle/_ref is the reference's own kernel sources (libclsph/kernels/*.cl,
libclsph/common/*.h) compiled as C++ through oracle/ref_shim, driven by a
restatement of libclsph/sph_simulation.cpp's substep. Each fixture holds the
inputs of one substep (parameter block, kernel constants, particle AoS,
mesh) and every output the reference produces for it: the grid parameters,
the stable-sort permutation, the dense cell table, the AoS after the sort,
after density_pressure, after forces, and after advection_collision.

Run in the development container (needs the reference sources):
    python tests/golden/make_golden.py [fixture name ...]
"""

from __future__ import annotations

import json
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
sys.path.insert(0, str(ROOT))

from libclsph_gb300 import workloads as W  # noqa: E402
from libclsph_gb300.layout import particles_from_arrays  # noqa: E402
from libclsph_gb300.settings import WATER, DEFAULT_SIM, settings_from_dicts  # noqa: E402
from oracle import RefBuild, build_ref  # noqa: E402

from oracle import reference_root  # noqa: E402

REF_ROOT = reference_root()  # CLSPH_REFERENCE_ROOT, else oracle/Makefile's default
MUCUS = {"fluid_density": 1000, "dynamic_viscosity": 36, "restitution": 0.5, "k": 5,
         "surface_tension_threshold": 5, "surface_tension": 6,
         "particles_inside_influence_radius": 40}


def obj_mesh(name: str) -> dict:
    """A scene of the reference's scenes/ folder through the project's OBJ
    reader (same vertex/face order as tinyobj 0.9.6)."""
    from libclsph_gb300.scene import Scene

    sc = Scene()
    if not sc.load(name, base=REF_ROOT / "scenes"):
        raise RuntimeError(f"cannot load {name}")
    return {"vertices": np.asarray(sc.vertices, np.float32),
            "indices": np.asarray(sc.indices, np.uint32),
            "face_normals": np.asarray(sc.face_normals, np.float32)}


def settings(n, fluid=WATER, **sim_overrides):
    sim = dict(DEFAULT_SIM, particles_count=n, **sim_overrides)
    return settings_from_dicts(fluid, sim)


def case_default_lattice():
    """The reference's own initial condition (init_particles cube lattice),
    512 particles, water + default properties, scenes/cube.obj."""
    from oracle import Oracle

    st = settings(512)
    parts = Oracle().init_lattice(512, st.initial_volume)
    return "default_lattice_cube_512", st, parts, obj_mesh("cube.obj"), 1


def case_box_floor():
    """2000 particles with random velocities on the floor of scenes/box.obj."""
    st = settings(2000, constant_acceleration={"x": 0, "y": -9.81, "z": 0})
    h = float(st.params["h"])
    rng = np.random.default_rng(11)
    pos = W.lattice((20, 5, 20), h / 2, (-0.25, -1.9995, -0.25), 0.01, rng)
    vel = rng.normal(0, 1.5, pos.shape).astype(np.float32)
    vel[:, 1] -= 2.0
    return "box_floor_2000", st, particles_from_arrays(pos, vel, vel), obj_mesh("box.obj"), 1


def case_mucus_corner():
    """1000 mucus particles (restitution 0.5) driven into a corner of a unit box."""
    st = settings(1000, fluid=MUCUS, constant_acceleration={"x": 0, "y": -9.81, "z": 0})
    h = float(st.params["h"])
    rng = np.random.default_rng(12)
    pos = W.lattice((10, 10, 10), h / 2, (0.0004, 0.0004, 0.0004), 0.01, rng)
    vel = (-np.abs(rng.normal(0, 3.0, pos.shape))).astype(np.float32)
    return ("mucus_corner_1000", st, particles_from_arrays(pos, vel, vel),
            W.box_mesh((0, 0, 0), (1, 1, 1)), 1)


def case_coincident():
    """Coincident pairs (the r ~ 0 branch of spiky_gradient) and particles on
    exact cell boundaries."""
    st = settings(729)
    h = float(st.params["h"])
    rng = np.random.default_rng(13)
    pos = W.lattice((9, 9, 9), h / 2, (0.3, 0.3, 0.3), 0.0, rng).astype(np.float32)
    pos[1::7] = pos[0::7][: len(pos[1::7])]  # duplicate positions
    vel = rng.normal(0, 0.2, pos.shape).astype(np.float32)
    return ("coincident_729", st, particles_from_arrays(pos, vel, vel),
            W.box_mesh((0, 0, 0), (1, 1, 1)), 1)


def case_trajectory():
    """Five substeps of a 15^3 block dropping onto the floor of a unit box (final AoS)."""
    st = settings(3375, constant_acceleration={"x": 0, "y": -9.81, "z": 0})
    h = float(st.params["h"])
    rng = np.random.default_rng(14)
    pos = W.lattice((15, 15, 15), h / 2, (0.05, 0.0005, 0.05), 0.01, rng)
    vel = rng.normal(0, 0.3, pos.shape).astype(np.float32)
    return ("trajectory_3375_x5", st, particles_from_arrays(pos, vel, vel),
            W.box_mesh((0, 0, 0), (1, 1, 1)), 5)


def case_edge_hits():
    """Particles whose path crosses a mesh edge or vertex exactly in this
    substep, with no gravity and no neighbours, so each moves in a straight
    line: onto the diagonal shared by the two triangles of the z = 0 face
    (x == y there), onto the edges where two faces meet, and into the corners
    where three meet. The hit distances tie between faces, which is where
    "equal distance: the later face wins" decides the response. An interior
    lattice spaced wider than h fills the scene to 216 particles."""
    st = settings(216, constant_acceleration={"x": 0, "y": 0, "z": 0})
    h = float(st.params["h"])
    assert 0.1 > h
    pos, vel = [], []
    for t in np.arange(0.15, 0.9, 0.1, dtype=np.float32):  # the face diagonal
        pos.append((t, t, 0.002))
        vel.append((0.0, 0.0, -3.0))
    for t in (0.25, 0.55, 0.85):  # edges between two faces
        pos.append((0.002, t, 0.002))
        vel.append((-2.0, 0.0, -2.0))
        pos.append((t, 0.998, 0.002))
        vel.append((0.0, 2.0, -2.0))
    for c in [(0.003, 0.003, 0.003), (0.997, 0.003, 0.003), (0.003, 0.997, 0.997),
              (0.997, 0.997, 0.997)]:  # corners
        pos.append(c)
        vel.append(tuple(-2.5 if x < 0.5 else 2.5 for x in c))
    rng = np.random.default_rng(15)
    need = 216 - len(pos)
    fill = W.lattice((6, 6, 6), 0.1, (0.2, 0.2, 0.2), 0.0, rng)[:need]
    pos = np.concatenate([np.array(pos, np.float32), fill.astype(np.float32)])
    vel = np.concatenate([np.array(vel, np.float32),
                          rng.normal(0, 0.2, (need, 3)).astype(np.float32)])
    return ("edge_hits_216", st, particles_from_arrays(pos, vel, vel),
            W.box_mesh((0, 0, 0), (1, 1, 1)), 1)


def aimed_at_mesh(mesh, n, st, rng, region=None):
    """Up to n particles whose paths cross the mesh during the substep: each
    is aimed at a point inside a face, on an edge or at a vertex (in turn), of
    a random face (limited to faces whose centroid lies in `region`), from
    either side, along the face's normal tilted at random, at 30-100 % of the
    maximum speed, and starts 5-95 % of one substep's travel before it.
    Particles start at least 0.6 h apart."""
    h = float(st.params["h"])
    dt = float(st.params["time_delta"]) * float(st.params["simulation_scale"])
    vmax = float(st.params["max_velocity"])
    v = np.asarray(mesh["vertices"], np.float64).reshape(-1, 3)
    tri = np.asarray(mesh["indices"], np.int64).reshape(-1, 3)
    nrm = np.asarray(mesh["face_normals"], np.float64).reshape(-1, 3)[:len(tri)]
    faces = np.arange(len(tri))
    if region is not None:
        cen = v[tri].mean(axis=1)
        faces = faces[np.all((cen >= region[0]) & (cen <= region[1]), axis=1)]
    pos, vel = [], []
    for _ in range(60 * n):
        if len(pos) == n:
            break
        f = int(rng.choice(faces))
        a, b, c = v[tri[f]]
        kind = len(pos) % 3
        if kind == 0:
            r1, r2 = rng.uniform(0.02, 0.98, 2)
            if r1 + r2 > 1.0:
                r1, r2 = 1.0 - r1, 1.0 - r2
            target = a + r1 * (b - a) + r2 * (c - a)
        elif kind == 1:
            p, q = [(a, b), (b, c), (c, a)][int(rng.integers(3))]
            target = p + rng.uniform(0.05, 0.95) * (q - p)
        else:
            target = (a, b, c)[int(rng.integers(3))]
        nf = nrm[f]
        if not np.all(np.isfinite(nf)):
            continue
        into = -nf if rng.random() < 0.5 else nf
        d = into + rng.normal(0.0, 0.35, 3)
        d /= np.linalg.norm(d)
        if np.dot(d, into) < 0.2:
            continue
        speed = rng.uniform(0.3, 1.0) * vmax
        start = target - d * speed * dt * rng.uniform(0.05, 0.95)
        if pos and np.min(np.linalg.norm(np.asarray(pos) - start, axis=1)) < 0.6 * h:
            continue
        pos.append(start)
        vel.append(d * speed)
    pos = np.asarray(pos, np.float32)
    vel = np.asarray(vel, np.float32)
    return particles_from_arrays(pos, vel, vel)


def _mesh_case(name, obj, n, seed, region=None):
    mesh = obj_mesh(obj)
    st = settings(n, constant_acceleration={"x": 0, "y": -9.81, "z": 0})
    parts = aimed_at_mesh(mesh, n, st, np.random.default_rng(seed), region)
    st = settings(len(parts), constant_acceleration={"x": 0, "y": -9.81, "z": 0})
    return name, st, parts, mesh, 1


def case_monkey_hits():
    """Paths through the faces, edges and vertices of scenes/monkey.obj (968 faces)."""
    return _mesh_case("monkey_hits", "monkey.obj", 1500, 16)


def case_shower_hits():
    """Paths through scenes/shower.obj (1,248 faces)."""
    return _mesh_case("shower_hits", "shower.obj", 1500, 17)


def case_labyrinth_hits():
    """Paths through scenes/labyrinth.obj (606 faces)."""
    return _mesh_case("labyrinth_hits", "labyrinth.obj", 1000, 18)


def case_river_hits():
    """Paths through scenes/river.obj (332 faces over 19 x 15 x 17 m: a grid
    of about 157 x 118 x 141 cells, 2^24 dense table entries)."""
    return _mesh_case("river_hits", "river.obj", 1000, 19)


CASES = [case_default_lattice, case_box_floor, case_mucus_corner, case_coincident, case_trajectory,
         case_edge_hits, case_monkey_hits, case_shower_hits, case_labyrinth_hits, case_river_hits]
# fixtures that keep only the sorted and final states (the dense cell table
# follows from the sorted keys): their meshes make the other stages large
COMPACT = {"monkey_hits", "shower_hits", "labyrinth_hits", "river_hits"}


def collided(st, r) -> int:
    """Particles whose substep ended away from their free flight (a collision
    moved them): free flight is x + v' dt with v' = v_half + a dt, clamped to
    the maximum speed."""
    dt = np.float32(st.params["time_delta"]) * np.float32(st.params["simulation_scale"])
    x = r.sorted["position"][:, :3].astype(np.float64)
    v = r.sorted["intermediate_velocity"][:, :3].astype(np.float64) + \
        r.forces["acceleration"][:, :3].astype(np.float64) * dt
    sp = np.linalg.norm(v, axis=1)
    vmax = float(st.params["max_velocity"])
    v = np.where(sp[:, None] > vmax, v / np.maximum(sp, 1e-30)[:, None] * vmax, v)
    free = x + v * dt
    return int(np.sum(np.linalg.norm(r.final["position"][:, :3] - free, axis=1) > 1e-5))


GEO_NAME = "frame_ref_300"


def make_geo_golden() -> None:
    """The reference's own .geo frame writer (oracle/_ref/ref_geo: the
    reference's houdini_file_saver.cpp and HoudiniFileDumpHelper.cpp compiled
    unchanged) on 300 particles whose densities cover every branch of its
    colour ramp (below 0, the 500 / 1000 / 1500 / 2000 boundaries, above
    2000) and whose coordinates span many magnitudes and signs (the stream's
    default 6-significant-digit formatting, exponents, -0). Writes
    tests/golden/geo/frame_ref_300.npz (inputs) and frame_ref_300.geo (output),
    outside the substep fixtures' folder."""
    import shutil
    import subprocess
    import tempfile

    from libclsph_gb300.layout import PARAMS, PARTICLE

    rng = np.random.default_rng(20)
    n = 300
    parts = np.zeros(n, dtype=PARTICLE)
    scale = 10.0 ** rng.integers(-7, 4, (n, 1))
    parts["position"][:, :3] = (rng.normal(0, 1, (n, 3)) * scale).astype(np.float32)
    parts["velocity"][:, :3] = (rng.normal(0, 1, (n, 3)) * scale[::-1]).astype(np.float32)
    parts["intermediate_velocity"][:, :3] = rng.normal(0, 1, (n, 3)).astype(np.float32)
    parts["position"][0, :3] = [-0.0, 0.0, 1.0]
    parts["velocity"][1, :3] = [123456.789, -0.000123456789, 1e-30]
    dens = rng.uniform(-100, 2600, n).astype(np.float32)
    edges = [-1.0, 0.0, 1e-3, 250.0, 499.99997, 500.0, 500.00003, 750.0, 999.99994, 1000.0,
             1000.0001, 1250.0, 1499.9999, 1500.0, 1500.0001, 1800.0, 1999.9999, 2000.0,
             2000.0002, 3000.0]
    dens[2:2 + len(edges)] = np.array(edges, dtype=np.float32)
    parts["density"] = dens
    parts["pressure"] = rng.normal(0, 1e4, n).astype(np.float32)
    parts["grid_index"] = rng.integers(0, 1 << 20, n).astype(np.uint32)
    params = np.zeros(1, dtype=PARAMS)
    params["particles_count"] = n
    params["particle_mass"] = np.float32(7.9717e-4)
    with tempfile.TemporaryDirectory() as tmp:
        t = Path(tmp)
        (t / "frames").mkdir()
        params.tofile(t / "params.bin")
        parts.tofile(t / "particles.bin")
        subprocess.run([str(ROOT / "oracle" / "_ref" / "ref_geo"), str(t / "params.bin"),
                        str(t / "particles.bin"), str(t) + "/"], check=True)
        (HERE / "geo").mkdir(exist_ok=True)
        shutil.copyfile(t / "frames" / "frame0000001.geo", HERE / "geo" / f"{GEO_NAME}.geo")
    np.savez_compressed(HERE / "geo" / f"{GEO_NAME}.npz", params=params, particles=parts)
    print(GEO_NAME, (HERE / "geo" / f"{GEO_NAME}.geo").stat().st_size, "bytes")


def main() -> None:
    """Writes every fixture, or only those named on the command line (the
    others keep their files and manifest entries)."""
    if build_ref() is None:
        raise SystemExit("reference sources not found; fixtures are generated in the dev container")
    only = set(sys.argv[1:])
    if not only or GEO_NAME in only:
        make_geo_golden()
    ref = RefBuild()
    mpath = HERE / "manifest.json"
    manifest = json.loads(mpath.read_text()) if only and mpath.exists() else {}
    for make in CASES:
        name, st, parts, mesh, steps = make()
        if only and name not in only:
            continue
        out = {"params": np.array(st.params).reshape(1), "terms": np.array(st.terms).reshape(1),
               "particles": parts, "vertices": mesh["vertices"], "indices": mesh["indices"],
               "face_normals": mesh["face_normals"], "steps": np.array([steps])}
        if steps == 1:
            r = ref.step(st.params, st.terms, parts, mesh)
            out.update(params_out=np.array(r.params).reshape(1), perm=r.perm, sorted=r.sorted,
                       final=r.final, capped=np.array([r.capped]))
            if name not in COMPACT:
                out.update(table=r.table, density=r.density, forces=r.forces)
        else:
            cur = parts
            for _ in range(steps):
                cur = ref.step(st.params, st.terms, cur, mesh).final
            out.update(final=cur)
        np.savez_compressed(HERE / f"{name}.npz", **out)
        manifest[name] = {"n": int(len(parts)), "steps": steps,
                          "faces": int(len(mesh["indices"]) // 3)}
        if steps == 1:
            manifest[name]["collided"] = collided(st, r)
        print(name, manifest[name])
    mpath.write_text(json.dumps(manifest, indent=1) + "\n")


if __name__ == "__main__":
    main()
