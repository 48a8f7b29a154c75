"""Seeded synthetic scenes of the benchmark shapes.

No public dataset is involved: every workload is generated here from a seed.

* `dam_break(32)`: 32,768 particles as a 32^3 lattice (spacing h/2, jitter
  +-1 % of the spacing) in a closed 1 x 1 x 1 m box (12 triangles); water
  constants of fluid_properties/water.json, gravity -9.81, m = 0.05 kg.
* `dam_break((128, 128, 64), box=(4, 2, 2))`: 1,048,576 particles as a
  128 x 128 x 64 lattice (1 m wide in x, 1 m tall, 0.5 m deep; a 128^3
  lattice would hold 2,097,152) in the left quarter (x in [0, 1] m) of a
  4 x 2 x 2 m box; the particle mass is chosen so that h = 1/64 m and the
  block fits at spacing h/2.
* `pour(...)`: a 64 x 64 x L column falling at 2 m/s (+-5 % per-particle
  noise) onto a 256 x 256-quad heightfield (131,072 triangles, seeded sum of
  four sinusoids, amplitude 0.2 m) inside a 4 x 4 x 2 m box.
"""

from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

from .layout import PARAMS, PARTICLE, particles_from_arrays
from .settings import WATER, DEFAULT_SIM, settings_from_dicts


@dataclass
class Scene:
    name: str
    params: np.void
    terms: np.void
    particles: np.ndarray
    mesh: dict
    steps: int
    info: dict = field(default_factory=dict)

    @property
    def n(self) -> int:
        return len(self.particles)


def face_normals(vertices: np.ndarray, indices: np.ndarray) -> np.ndarray:
    """Unit normals from the cross product (libclsph/scene.cpp:35-64), float32."""
    v = np.asarray(vertices, dtype=np.float32).reshape(-1, 3)
    t = v[np.asarray(indices, dtype=np.int64).reshape(-1, 3)]
    u = (t[:, 1] - t[:, 0]).astype(np.float32)
    w = (t[:, 2] - t[:, 0]).astype(np.float32)
    n = np.stack([u[:, 1] * w[:, 2] - u[:, 2] * w[:, 1],
                  u[:, 2] * w[:, 0] - u[:, 0] * w[:, 2],
                  u[:, 0] * w[:, 1] - u[:, 1] * w[:, 0]], axis=1).astype(np.float32)
    length = np.sqrt((n[:, 0] * n[:, 0] + n[:, 1] * n[:, 1]) + n[:, 2] * n[:, 2]).astype(np.float32)
    with np.errstate(invalid="ignore", divide="ignore"):  # degenerate faces give NaN, as in C
        return (n / length[:, None]).astype(np.float32).ravel()


def make_mesh(vertices, indices) -> dict:
    v = np.ascontiguousarray(np.asarray(vertices, dtype=np.float32).ravel())
    i = np.ascontiguousarray(np.asarray(indices, dtype=np.uint32).ravel())
    return {"vertices": v, "indices": i, "face_normals": face_normals(v, i)}


def box_mesh(lo, hi) -> dict:
    """Closed axis-aligned box, 12 triangles."""
    x0, y0, z0 = lo
    x1, y1, z1 = hi
    v = [(x0, y0, z0), (x1, y0, z0), (x1, y1, z0), (x0, y1, z0),
         (x0, y0, z1), (x1, y0, z1), (x1, y1, z1), (x0, y1, z1)]
    quads = [(0, 3, 2, 1), (4, 5, 6, 7), (0, 1, 5, 4), (3, 7, 6, 2), (0, 4, 7, 3), (1, 2, 6, 5)]
    tris = []
    for a, b, c, d in quads:
        tris += [a, b, c, a, c, d]
    return make_mesh(v, tris)


def merge_meshes(*meshes) -> dict:
    verts, idx, off = [], [], 0
    for m in meshes:
        v = m["vertices"].reshape(-1, 3)
        verts.append(v)
        idx.append(m["indices"].astype(np.int64) + off)
        off += len(v)
    return make_mesh(np.concatenate(verts), np.concatenate(idx))


def heightfield_mesh(lo_xz, hi_xz, quads, base_y, amplitude, seed) -> dict:
    """quads x quads grid, two triangles per quad, height = sum of 4 seeded sinusoids."""
    rng = np.random.default_rng(seed)
    kx = rng.uniform(0.5, 3.0, 4) * 2 * math.pi / (hi_xz[0] - lo_xz[0])
    kz = rng.uniform(0.5, 3.0, 4) * 2 * math.pi / (hi_xz[1] - lo_xz[1])
    ph = rng.uniform(0, 2 * math.pi, 4)
    amp = rng.uniform(0.5, 1.0, 4)
    amp *= amplitude / amp.sum()
    xs = np.linspace(lo_xz[0], hi_xz[0], quads + 1)
    zs = np.linspace(lo_xz[1], hi_xz[1], quads + 1)
    X, Z = np.meshgrid(xs, zs, indexing="ij")
    Y = base_y + sum(amp[k] * np.sin(kx[k] * X + kz[k] * Z + ph[k]) for k in range(4))
    verts = np.stack([X, Y, Z], -1).reshape(-1, 3)
    i, j = np.meshgrid(np.arange(quads), np.arange(quads), indexing="ij")
    a = (i * (quads + 1) + j).ravel()
    b = a + 1
    c = a + quads + 1
    d = c + 1
    tris = np.stack([a, c, b, b, c, d], -1).reshape(-1)
    return make_mesh(verts, tris)


def water_settings(n: int, mass: float = 0.05, gravity: float = -9.81, **fluid_overrides):
    fluid = dict(WATER, **fluid_overrides)
    sim = dict(DEFAULT_SIM, particles_count=n, particle_mass=mass,
               constant_acceleration={"x": 0.0, "y": gravity, "z": 0.0})
    return settings_from_dicts(fluid, sim)


def mass_for_h(h: float, rho0: float = WATER["fluid_density"], k: int = 20) -> float:
    """Particle mass that makes load_settings derive smoothing radius h."""
    return h ** 3 * 4.0 * math.pi * rho0 / (3.0 * k)


def lattice(shape, spacing, origin, jitter_frac, rng) -> np.ndarray:
    nx, ny, nz = shape
    g = np.stack(np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij"), -1)
    g = g.reshape(-1, 3).astype(np.float64)
    pos = np.asarray(origin, dtype=np.float64) + (g + 0.5) * spacing
    pos += rng.uniform(-jitter_frac * spacing, jitter_frac * spacing, pos.shape)
    return pos.astype(np.float32)


def dam_break(shape=(32, 32, 32), box=(1.0, 1.0, 1.0), seed: int = 1, mass: float | None = None,
              steps: int = 1000, jitter: float = 0.01) -> Scene:
    if isinstance(shape, int):
        shape = (shape, shape, shape)
    n = int(np.prod(shape))
    if mass is None:
        mass = 0.05 if box == (1.0, 1.0, 1.0) else mass_for_h(1.0 / 64.0)
    st = water_settings(n, mass=mass)
    h = float(st.params["h"])
    s = h / 2
    rng = np.random.default_rng(seed)
    ext = [k * s for k in shape]
    if box == (1.0, 1.0, 1.0):
        origin = tuple((1.0 - e) / 2 for e in ext)
    else:  # left quarter, on the floor, centred in z
        origin = (0.0, 0.0, (box[2] - ext[2]) / 2)
    pos = lattice(tuple(shape), s, origin, jitter, rng)
    parts = particles_from_arrays(pos)
    return Scene(f"dam_break_{n}", st.params, st.terms, parts, box_mesh((0, 0, 0), box), steps,
                 {"h": h, "spacing": s, "mass": mass, "box": list(box), "seed": seed,
                  "lattice": list(shape)})


def dam_break_32k(seed: int = 1) -> Scene:
    """32,768 particles, 32^3 lattice, 1 m box, 1000 substeps."""
    return dam_break((32, 32, 32), seed=seed, steps=1000)


def dam_break_1m(seed: int = 1) -> Scene:
    """1,048,576 particles, 128 x 128 x 64 lattice, 4 x 2 x 2 m box, 2000 substeps."""
    return dam_break((128, 128, 64), box=(4.0, 2.0, 2.0), seed=seed, steps=2000)


def batched_dam_breaks(count: int = 256, seed: int = 5, n_min: int = 2048, n_max: int = 65536,
                       steps: int = 1000) -> list:
    """`count` independent dam breaks: particle count log-uniform in
    [n_min, n_max], rest density uniform in [900, 1200] kg/m^3, viscosity
    uniform in [0.5, 4] x water's. Each is a water column released in a box
    scaled to it: lattice spacing h/2 with h = 1/64 m (through the particle
    mass) and seeded jitter, a column ny layers high (log-uniform in
    [16, 128], i.e. up to the 1 m of the large dam break, which sets the
    hydrostatic range the scenes cover) with an nx : nz = 2 : 1 footprint
    (the large dam break's), top layer ragged, in the left quarter of a box
    four columns long, twice its height and four columns deep (12 triangles)."""
    rng = np.random.default_rng(seed)
    h = 1.0 / 64.0
    s = h / 2
    out = []
    for k in range(count):
        n = int(round(math.exp(rng.uniform(math.log(n_min), math.log(n_max)))))
        rho0 = float(rng.uniform(900.0, 1200.0))
        mu = float(WATER["dynamic_viscosity"] * rng.uniform(0.5, 4.0))
        ny = int(round(math.exp(rng.uniform(math.log(16), math.log(128)))))
        nz = max(2, int(math.ceil(math.sqrt(n / (2.0 * ny)))))
        nx = 2 * nz
        ny = max(ny, int(math.ceil(n / (nx * nz))))
        st = water_settings(n, mass=mass_for_h(h, rho0), fluid_density=rho0, dynamic_viscosity=mu)
        dims = (nx, ny, nz)
        block = lattice(dims, s, (0.0, 0.0, 0.0), 0.01, rng)
        # fill the column layer by layer from the floor: sort by height, keep n
        block = block[np.argsort(block[:, 1], kind="stable")][:n]
        box = (4 * nx * s, 2 * ny * s, 4 * nz * s)
        out.append(Scene(f"batched_{k}", st.params, st.terms, particles_from_arrays(block),
                         box_mesh((0, 0, 0), box), steps,
                         {"h": float(st.params["h"]), "rho0": rho0, "mu": mu, "box": box,
                          "dims": dims, "seed": seed}))
    return out


def pour(cross: int = 64, length: int = 1024, quads: int = 256, seed: int = 3,
         steps: int = 3000) -> Scene:
    box = (4.0, 2.0, 4.0)  # x, y (up), z
    top = 1.9
    bottom_y = 0.5
    s = (top - bottom_y) / length
    h = 2 * s
    mass = mass_for_h(h)
    n = cross * cross * length
    st = water_settings(n, mass=mass)
    rng = np.random.default_rng(seed)
    origin = (box[0] / 2 - cross * s / 2, bottom_y, box[2] / 2 - cross * s / 2)
    pos = lattice((cross, length, cross), s, origin, 0.01, rng)
    vel = np.zeros_like(pos)
    vel[:, 1] = -2.0 * (1.0 + rng.uniform(-0.05, 0.05, n))
    parts = particles_from_arrays(pos, vel, vel)
    field_mesh = heightfield_mesh((0.0, 0.0), (box[0], box[2]), quads, 0.25, 0.2, seed)
    mesh = merge_meshes(field_mesh, box_mesh((0, 0, 0), box))
    return Scene(f"pour_{n}", st.params, st.terms, parts, mesh, steps,
                 {"h": float(st.params["h"]), "spacing": s, "mass": mass, "faces": len(mesh["indices"]) // 3,
                  "seed": seed})


def small_block(n_side: int = 8, seed: int = 0, box=(1.0, 1.0, 1.0), offset=(0.3, 0.05, 0.3),
                velocity_sigma: float = 0.0, spacing_frac: float = 0.5) -> Scene:
    """A small jittered block for parity tests (sizes the oracle finishes fast)."""
    n = n_side ** 3
    st = water_settings(n)
    h = float(st.params["h"])
    rng = np.random.default_rng(seed)
    pos = lattice((n_side,) * 3, h * spacing_frac, offset, 0.01, rng)
    vel = rng.normal(0.0, velocity_sigma, pos.shape).astype(np.float32) if velocity_sigma else None
    parts = particles_from_arrays(pos, vel, vel)
    return Scene(f"block_{n}", st.params, st.terms, parts, box_mesh((0, 0, 0), box), 10,
                 {"h": h, "seed": seed})


__all__ = ["Scene", "box_mesh", "heightfield_mesh", "merge_meshes", "make_mesh", "face_normals",
           "water_settings", "mass_for_h", "dam_break", "dam_break_32k", "dam_break_1m", "pour",
           "batched_dam_breaks", "small_block", "lattice",
           "PARAMS", "PARTICLE"]
