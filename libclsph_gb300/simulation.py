"""Python mirror of libclsph's sph_simulation and houdini_file_saver.

`Simulation` keeps the reference's surface (libclsph/sph_simulation.h:8-52):
`load_settings(fluid_file, parameters_file)`, `simulate(frame_count=0)`,
`parameters`, `precomputed_terms`, `pre_frame` / `post_frame` callbacks
`(particles, parameters, full_frame)`, `write_intermediate_frames`,
`serialize`, `initial_volume`, `current_scene`. Substeps run on the GPU
engine (gpu.GpuSolver); the particle AoS is copied to the host only when a
callback needs it (see `transfers`).

`HoudiniFileSaver` writes the reference's ASCII .geo frames
(libclsph/file_save_delegates/houdini_file_saver.cpp:25-92).
"""

from __future__ import annotations

import math
import os
from pathlib import Path
from typing import Callable, Optional

import numpy as np

from .layout import PARAMS, PARTICLE, TERMS
from .scene import Scene
from .settings import cbrtf, load_settings

f32 = np.float32

EVERY_SUBSTEP = "every_substep"
FRAMES_ONLY = "frames_only"
# fields of simulation_parameters that the engine recomputes every substep
GRID_FIELDS = ("min_point", "max_point", "grid_size_x", "grid_size_y", "grid_size_z", "grid_cell_count")


def init_lattice(n: int, initial_volume: float) -> np.ndarray:
    """sph_simulation.cpp:48-94 cube lattice (no last_frame.bin)."""
    side = int(math.ceil(float(cbrtf(n))))
    length = cbrtf(initial_volume)
    gap = f32(length / f32(side))
    i = np.arange(n, dtype=np.int64)
    out = np.zeros(n, dtype=PARTICLE)
    half = f32(length / f32(2.0))
    out["position"][:, 0] = ((i % side).astype(f32) * gap - half).astype(f32)
    out["position"][:, 1] = (((i // side) % side).astype(f32) * gap).astype(f32)
    out["position"][:, 2] = ((i // (side * side)).astype(f32) * gap - half).astype(f32)
    return out


class Simulation:
    def __init__(self):
        self.parameters = np.zeros(1, dtype=PARAMS)[0]
        self.precomputed_terms = np.zeros(1, dtype=TERMS)[0]
        self.pre_frame: Optional[Callable] = None
        self.post_frame: Optional[Callable] = None
        self.write_intermediate_frames = False
        self.serialize = False
        self.initial_volume = 0.0
        self.current_scene = Scene()
        self.transfers = EVERY_SUBSTEP
        self.collision_iteration_cap = 1024
        self.last_particles: Optional[np.ndarray] = None

    def load_settings(self, fluid_file, parameters_file) -> None:
        st = load_settings(fluid_file, parameters_file)
        self.parameters = st.params
        self.precomputed_terms = st.terms
        self.initial_volume = st.initial_volume
        self.write_intermediate_frames = st.write_intermediate_frames
        self.serialize = st.serialize

    def init_particles(self) -> np.ndarray:
        n = int(self.parameters["particles_count"])
        if os.path.exists("last_frame.bin"):
            raw = np.fromfile("last_frame.bin", dtype=np.uint8)
            if raw.size < n * PARTICLE.itemsize:
                raise RuntimeError("last_frame.bin is shorter than the particle count")
            return raw[: n * PARTICLE.itemsize].view(PARTICLE).copy()
        return init_lattice(n, self.initial_volume)

    def simulate(self, frame_count: int = 0) -> np.ndarray:
        from .gpu import GpuSolver

        p = self.parameters
        if frame_count == 0:
            frame_count = int(math.ceil(float(f32(p["simulation_time"]) * f32(p["target_fps"]))))
        n = int(p["particles_count"])
        particles = self.init_particles()
        # The reference hands current_scene to the kernels every substep
        # (sph_simulation.cpp:296-337), so a callback may edit the scene in
        # place; after a callback the scene is compared with the copy last
        # uploaded and uploaded again when it differs.
        # The same holds for `parameters` and `precomputed_terms`, which the
        # reference's kernels receive by value every substep: edits other than
        # to the grid fields (the engine's own) are handed to the device.
        state = {"device_newer": False, "host_dirty": False, "scene_check": False, "uploaded": None,
                 "inputs": None}

        def inputs_copy():
            prm = np.array(self.parameters, dtype=PARAMS).reshape(1).copy()
            for f in GRID_FIELDS:
                prm[f] = 0
            prm["constant_acceleration"][..., 3] = 0  # the padding lane of cl_float3
            return prm.tobytes() + np.array(self.precomputed_terms, dtype=TERMS).reshape(1).tobytes()

        def scene_copy():
            sc = self.current_scene
            return (int(sc.face_count), np.array(sc.face_normals, copy=True), np.array(sc.vertices, copy=True),
                    np.array(sc.indices, copy=True))

        def upload_scene(gpu):
            sc = self.current_scene
            gpu.set_mesh(sc.mesh() if sc.face_count else {"face_normals": np.zeros(0, np.float32),
                                                           "vertices": np.zeros(0, np.float32),
                                                           "indices": np.zeros(0, np.uint32)})
            state["uploaded"] = scene_copy()

        def refresh_scene(gpu):
            if not state["scene_check"]:
                return
            state["scene_check"] = False
            now, up = scene_copy(), state["uploaded"]
            if now[0] != up[0] or any(a.shape != b.shape or not np.array_equal(a, b)
                                      for a, b in zip(now[1:], up[1:])):
                upload_scene(gpu)
            inputs = inputs_copy()
            if inputs != state["inputs"]:
                if int(self.parameters["particles_count"]) != n:
                    raise RuntimeError("the particle count cannot change during simulate()")
                gpu.set_parameters(self.parameters, self.precomputed_terms)
                state["inputs"] = inputs

        with GpuSolver(p, self.precomputed_terms, n, None) as gpu:
            if self.current_scene.face_count:
                upload_scene(gpu)
            else:
                state["uploaded"] = scene_copy()
            state["inputs"] = inputs_copy()
            gpu.set_collision_cap(self.collision_iteration_cap)
            gpu.upload(particles)

            def refresh():
                if not state["device_newer"]:
                    return
                gpu.download(particles)
                grid = gpu.parameters()
                for f in GRID_FIELDS:
                    self.parameters[f] = grid[f]
                flags = gpu.sync()
                if flags & 1:
                    raise RuntimeError("particle grid reached 1024 cells on an axis")
                state["device_newer"] = False

            def call(cb, full):
                if cb is None:
                    return
                state["scene_check"] = True
                if full or self.transfers == EVERY_SUBSTEP:
                    refresh()
                    cb(particles, self.parameters, full)
                    state["host_dirty"] = True
                else:
                    cb(particles, self.parameters, full)

            for _ in range(frame_count):
                call(self.pre_frame, True)
                # the loop bound is read every substep, as the reference's is
                j = 0
                while f32(j) < f32(1.0) / f32(self.parameters["simulation_scale"]):
                    call(self.pre_frame, False)
                    if state["host_dirty"]:
                        gpu.upload(particles)
                        state["host_dirty"] = False
                    refresh_scene(gpu)
                    gpu.step(1)
                    state["device_newer"] = True
                    call(self.post_frame, False)
                    j += 1
                call(self.post_frame, True)
            refresh()
        self.last_particles = particles
        return particles


def _g(x) -> str:
    """A float printed like std::ostream's default formatting."""
    return f"{float(f32(x)):g}"


def density_color(d):
    d = f32(d)
    r = (d - f32(1000)) / f32(1000) if (d > 1000 and d <= 2000) else f32(0)
    g = f32(1) - d / f32(1000) if (d >= 0 and d < 1000) else f32(0)
    if 500 <= d <= 1000:
        b = (d - f32(500)) / f32(500)
    elif 1000 <= d <= 1500:
        b = f32(1) - (d - f32(1000)) / f32(500)
    else:
        b = f32(0)
    return f32(r), f32(g), f32(b)


def density_colors(d: np.ndarray) -> np.ndarray:
    """density_color over an array (float32 throughout): (n, 3) RGB."""
    d = np.asarray(d, dtype=np.float32)
    one, k500, k1000 = np.float32(1), np.float32(500), np.float32(1000)
    r = np.where((d > 1000) & (d <= 2000), (d - k1000) / k1000, np.float32(0))
    g = np.where((d >= 0) & (d < 1000), one - d / k1000, np.float32(0))
    b = np.where((d >= 500) & (d <= 1000), (d - k500) / k500,
                 np.where((d >= 1000) & (d <= 1500), one - (d - k1000) / k500, np.float32(0)))
    return np.stack([r, g, b], axis=1).astype(np.float32)


def bgeo_bytes(particles: np.ndarray, parameters) -> bytes:
    """One frame as classic binary Houdini geometry (version 5), the file the
    reference's USE_PARTIO build writes through Partio::write
    (libclsph/file_save_delegates/houdini_file_saver.cpp:76-88) with the
    attributes of makeData (util/partio/PartioFunctions.h:5-65): velocity,
    color (vectors), id (int), mass and pscale (floats) after the position.
    Big-endian throughout; 16-bit point indices up to 65,535 points, else
    32-bit. The full velocity is stored (makeData writes only component 0)."""
    n = int(parameters["particles_count"])
    be = np.dtype(">i4")

    def name(s: str) -> bytes:
        return np.array([len(s)], ">u2").tobytes() + s.encode()

    head = b"BgeoV" + np.array([5, n, 1, 0, 0, 5, 0, 1, 0], be).tobytes()
    for nm, size, typ in (("velocity", 3, 5), ("color", 3, 5), ("id", 1, 1), ("mass", 1, 0),
                          ("pscale", 1, 0)):
        head += name(nm) + np.array([size], ">u2").tobytes() + np.array([typ] + [0] * size, be).tobytes()
    rec = np.dtype([("p", ">f4", 4), ("v", ">f4", 3), ("c", ">f4", 3), ("id", ">i4"), ("m", ">f4"),
                    ("ps", ">f4")])
    pts = np.zeros(n, dtype=rec)
    pts["p"][:, :3] = particles["position"][:n, :3]
    pts["p"][:, 3] = 1.0
    pts["v"] = particles["velocity"][:n, :3]
    pts["c"] = density_colors(particles["density"][:n])
    pts["id"] = np.arange(n)
    pts["m"] = np.float32(parameters["particle_mass"])
    pts["ps"] = np.float32(parameters["h"])
    prim = (name("generator") + np.array([1], ">u2").tobytes() + np.array([4, 1], be).tobytes() +
            name("papi") + np.array([0x8000, n], be).tobytes())
    idx = np.arange(n, dtype=">u2" if n <= 65535 else ">i4").tobytes()
    return head + pts.tobytes() + prim + idx + np.array([0], be).tobytes() + b"\x00\xff"


class HoudiniFileSaver:
    """houdini_file_saver (libclsph/file_save_delegates/houdini_file_saver.h:8-20).

    `binary_bgeo` (default False) selects the binary .bgeo frame that the
    reference writes when built with USE_PARTIO."""

    def __init__(self, frames_folder_prefix: str, binary_bgeo: bool = False):
        self.frames_folder_prefix = frames_folder_prefix
        self.binary_bgeo = binary_bgeo
        self.frame_count = 0

    def writeFrameToFile(self, particles: np.ndarray, parameters) -> int:
        self.frame_count += 1
        stem = f"{self.frames_folder_prefix}frames/frame{str(self.frame_count).zfill(9)[-7:]}"
        if self.binary_bgeo:
            try:
                Path(stem + ".bgeo").write_bytes(bgeo_bytes(particles, parameters))
            except OSError:
                import sys

                sys.stderr.write(f"Error while writing to {stem}.bgeo\n")
            return 0
        name = stem + ".geo"
        n = int(parameters["particles_count"])
        mass = _g(parameters["particle_mass"])
        lines = ["PGEOMETRY V5", f"NPoints {n} NPrims 1", "NPointGroups 0 NPrimGroups 1",
                 "NPointAttrib 3 NVertexAttrib 0 NPrimAttrib 2 NAttrib 0", "PointAttrib",
                 "v 3 float 1 1 1", "color 3 float 1 1 1", "mass 1 float 1"]
        pos = particles["position"]
        vel = particles["velocity"]
        dens = particles["density"]
        for i in range(n):
            r, g, b = density_color(dens[i])
            lines.append(f"{_g(pos[i, 0])} {_g(pos[i, 1])} {_g(pos[i, 2])} 0 "
                         f"({_g(vel[i, 0])} {_g(vel[i, 1])} {_g(vel[i, 2])}\t"
                         f"{_g(r)} {_g(g)} {_g(b)}\t{mass})")
        lines += ["PrimitiveAttrib", "generator 1 index 1 location1",
                  "dopobject 1 index 1 /obj/AutoDopNetwork:1",
                  "Part " + str(n) + "".join(f" {i}" for i in range(n)) + " [0\t0]",
                  "box_object1 unordered", "1 1", "beginExtra", "endExtra"]
        try:
            Path(name).write_text("\n".join(lines) + "\n")
        except OSError:
            import sys

            sys.stderr.write(f"Error while writing to {name}\n")
        return 0


def save_last_frame(particles: np.ndarray, path: str = "last_frame.bin") -> None:
    """The example's serialize step (example/particles.cpp:40-44): raw AoS bytes."""
    np.ascontiguousarray(particles, dtype=PARTICLE).tofile(path)
