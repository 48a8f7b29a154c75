"""Byte layouts of the reference's shared host/device structs.

`PARTICLE` is `particle` (libclsph/common/structures.h:42-46) with the host's
16-byte `cl_float3`: 80 bytes, density at 64, grid_index at 72.
`PARAMS` is `simulation_parameters` (structures.h:16-40): 128 bytes.
`TERMS` is `precomputed_kernel_values` (structures.h:48-54): 20 bytes.

These are the byte formats of the drop-in boundary: the AoS that
`sph_simulation::simulate` hands to `pre_frame`/`post_frame`, the
`last_frame.bin` checkpoint (a raw dump of that AoS) and the parameter block
handed to the callbacks. The GPU path stores particles as SoA internally and
converts at the boundary.
"""

from __future__ import annotations

import numpy as np

F3 = ("<f4", (4,))  # cl_float3 is 16 bytes on the host (x, y, z, pad)

PARTICLE = np.dtype(
    {
        "names": [
            "position",
            "velocity",
            "intermediate_velocity",
            "acceleration",
            "density",
            "pressure",
            "grid_index",
        ],
        "formats": [F3, F3, F3, F3, "<f4", "<f4", "<u4"],
        "offsets": [0, 16, 32, 48, 64, 68, 72],
        "itemsize": 80,
    }
)

PARAMS = np.dtype(
    {
        "names": [
            "particles_count",
            "max_velocity",
            "fluid_density",
            "total_mass",
            "particle_mass",
            "dynamic_viscosity",
            "simulation_time",
            "target_fps",
            "h",
            "simulation_scale",
            "time_delta",
            "surface_tension_threshold",
            "surface_tension",
            "restitution",
            "K",
            "constant_acceleration",
            "grid_size_x",
            "grid_size_y",
            "grid_size_z",
            "grid_cell_count",
            "min_point",
            "max_point",
        ],
        "formats": ["<u4"] + ["<f4"] * 14 + [F3, "<i4", "<i4", "<i4", "<u4", F3, F3],
        "offsets": [4 * i for i in range(15)] + [64, 80, 84, 88, 92, 96, 112],
        "itemsize": 128,
    }
)

TERMS = np.dtype(
    [
        ("poly_6", "<f4"),
        ("poly_6_gradient", "<f4"),
        ("poly_6_laplacian", "<f4"),
        ("spiky", "<f4"),
        ("viscosity", "<f4"),
    ]
)

assert PARTICLE.itemsize == 80 and PARAMS.itemsize == 128 and TERMS.itemsize == 20


def empty_particles(n: int) -> np.ndarray:
    return np.zeros(n, dtype=PARTICLE)


def particles_from_arrays(pos, vel=None, ivel=None) -> np.ndarray:
    """AoS from (n, 3) arrays; missing velocities are zero."""
    pos = np.asarray(pos, dtype=np.float32)
    n = pos.shape[0]
    out = empty_particles(n)
    out["position"][:, :3] = pos
    if vel is not None:
        out["velocity"][:, :3] = np.asarray(vel, dtype=np.float32)
    if ivel is not None:
        out["intermediate_velocity"][:, :3] = np.asarray(ivel, dtype=np.float32)
    return out


def ptr(a: np.ndarray) -> int:
    """Address of a C-contiguous numpy buffer (for ctypes calls)."""
    if not a.flags["C_CONTIGUOUS"]:
        raise ValueError("buffer must be C-contiguous")
    return a.ctypes.data
