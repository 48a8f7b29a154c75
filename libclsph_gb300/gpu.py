"""ctypes binding of the C ABI in include/clsph_gpu.h.

`GpuSolver` owns one device handle: create -> set_mesh -> upload -> step ->
download. It is the thin layer the Python mirror of `sph_simulation`
(simulation.py), the tests and bench.py use; there is no CPU fallback: if the
CUDA library or a device is missing, construction raises.
"""

from __future__ import annotations

import ctypes
from pathlib import Path

import numpy as np

from .layout import PARAMS, PARTICLE, TERMS

_LIB = None

STAGE_GRID, STAGE_SORT, STAGE_DENSITY, STAGE_FORCES, STAGE_ADVECT = 1, 2, 3, 4, 5
# neighbour search modes of the density kernel (include/clsph_gpu.h)
SEARCH_WINDOW, SEARCH_CELL_WARPS, SEARCH_PARTICLE_WARPS = 0, 1, 2
SEARCH_MODES = (SEARCH_WINDOW, SEARCH_CELL_WARPS, SEARCH_PARTICLE_WARPS)
WARN_GRID_OVERFLOW, WARN_COLLISION_CAP, WARN_NONFINITE = 1, 2, 4
# bounds of the device waits (clsph_gpu_set_wait_limits)
DEFAULT_LOOKBACK_SPINS, DEFAULT_MLP_WAIT_POLLS, NO_TILE = 1 << 20, 1 << 24, 0xFFFFFFFF
DEFAULT_BARRIER_SPINS, NO_BLOCK = 1 << 22, 0xFFFFFFFF

_vp = ctypes.c_void_p
_u32 = ctypes.c_uint32

# (name, restype, argtypes) of every symbol include/clsph_gpu.h declares
SIGNATURES = [
    ("clsph_gpu_create", ctypes.c_int, [_vp, _vp, _u32, ctypes.POINTER(_vp)]),
    ("clsph_gpu_create_batched", ctypes.c_int, [_vp, _vp, _vp, _u32, ctypes.POINTER(_vp)]),
    ("clsph_gpu_set_scene_mesh", ctypes.c_int, [_vp, _u32, _vp, _vp, _u32, _vp, _u32]),
    ("clsph_gpu_set_graph", ctypes.c_int, [_vp, ctypes.c_int]),
    ("clsph_gpu_get_scene_parameters", ctypes.c_int, [_vp, _u32, _vp]),
    ("clsph_gpu_set_parameters", ctypes.c_int, [_vp, _vp, _vp]),
    ("clsph_gpu_set_scene_parameters", ctypes.c_int, [_vp, _u32, _vp, _vp]),
    ("clsph_gpu_read_cell_table_scene", ctypes.c_int, [_vp, _u32, _vp, ctypes.c_uint64]),
    ("clsph_gpu_destroy", ctypes.c_int, [_vp]),
    ("clsph_gpu_set_collision_cap", ctypes.c_int, [_vp, _u32]),
    ("clsph_gpu_set_stream", ctypes.c_int, [_vp, _vp]),
    ("clsph_gpu_set_mesh", ctypes.c_int, [_vp, _vp, _vp, _u32, _vp, _u32]),
    ("clsph_gpu_upload", ctypes.c_int, [_vp, _vp]),
    ("clsph_gpu_download", ctypes.c_int, [_vp, _vp]),
    ("clsph_gpu_step", ctypes.c_int, [_vp, _u32]),
    ("clsph_gpu_step_until", ctypes.c_int, [_vp, ctypes.c_int]),
    ("clsph_gpu_sync", ctypes.c_int, [_vp, ctypes.POINTER(_u32)]),
    ("clsph_gpu_get_parameters", ctypes.c_int, [_vp, _vp]),
    ("clsph_gpu_read_keys", ctypes.c_int, [_vp, _vp, _vp]),
    ("clsph_gpu_read_cell_table", ctypes.c_int, [_vp, _vp, ctypes.c_uint64]),
    ("clsph_gpu_read_fields", ctypes.c_int, [_vp, _vp, _vp, _vp]),
    ("clsph_gpu_read_ids", ctypes.c_int, [_vp, _vp]),
    ("clsph_gpu_set_profiling", ctypes.c_int, [_vp, ctypes.c_int]),
    ("clsph_gpu_kernel_times", ctypes.c_int,
     [_vp, ctypes.c_int, ctypes.c_char_p, ctypes.c_int, _vp, _vp, ctypes.POINTER(ctypes.c_int)]),
    ("clsph_gpu_counters", ctypes.c_int, [_vp, _vp]),
    ("clsph_gpu_sort_keys_noalloc", ctypes.c_int, [_vp, _vp, _vp, _u32, _vp]),
    ("clsph_gpu_autotune", ctypes.c_int, [_vp, _u32, ctypes.c_char_p, ctypes.c_int]),
    ("clsph_gpu_set_launch_shape", ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_int, _u32]),
    ("clsph_gpu_set_neighbour_search", ctypes.c_int, [_vp, ctypes.c_int]),
    ("clsph_gpu_set_wait_limits", ctypes.c_int, [_vp, _u32, _u32, _u32]),
    ("clsph_gpu_set_persistent", ctypes.c_int, [_vp, ctypes.c_int]),
    ("clsph_gpu_set_barrier_limits", ctypes.c_int, [_vp, _u32, _u32]),
    ("clsph_gpu_read_face_lists", ctypes.c_int,
     [_vp, _u32, _vp, _vp, ctypes.c_uint64, _vp, ctypes.c_uint64, _vp]),
    ("clsph_gpu_last_error", ctypes.c_char_p, []),
]


def lib_path() -> Path:
    return Path(__file__).resolve().parent / "_lib" / "libclsph_gpu.so"


def load_library(build: bool = False) -> ctypes.CDLL:
    """Loads libclsph_gpu.so (building it first if asked). Raises if absent."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = lib_path()
    if build or not path.exists():
        if not build:
            raise RuntimeError(
                f"{path} is missing: run `python -c 'import __graft_entry__ as g; g.build()'` "
                "(the CUDA engine has no CPU fallback)")
        from .build import build_gpu
        build_gpu()
    lib = ctypes.CDLL(str(path))
    for name, res, args in SIGNATURES:
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _LIB = lib
    return lib


class ClsphError(RuntimeError):
    def __init__(self, fn: str, code: int, msg: str):
        super().__init__(f"{fn} failed with status {code}: {msg}")
        self.code = code


def _check(fn: str, code: int) -> None:
    if code != 0:
        msg = (_LIB.clsph_gpu_last_error() or b"").decode(errors="replace")
        raise ClsphError(fn, code, msg)


def _a(x: np.ndarray) -> int:
    if not x.flags["C_CONTIGUOUS"]:
        raise ValueError("buffers passed to the C ABI must be C-contiguous")
    return x.ctypes.data


class GpuSolver:
    """SPH scenes on the current CUDA device (include/clsph_gpu.h).

    `GpuSolver(params, terms, n, mesh)` holds one scene;
    `GpuSolver.batched(params_list, terms_list, counts, meshes)` holds several
    independent scenes stepped by the same kernel launches (their particles
    are concatenated in scene order in upload/download)."""

    def __init__(self, params, terms, n: int | None = None, mesh=None, *, counts=None):
        self.lib = load_library()
        self.params = np.array(params, dtype=PARAMS).reshape(-1).copy()
        self.terms = np.array(terms, dtype=TERMS).reshape(-1).copy()
        handle = _vp()
        if counts is None:
            self.counts = [int(n if n is not None else self.params["particles_count"][0])]
            self.params["particles_count"] = self.counts[0]
            _check("clsph_gpu_create",
                   self.lib.clsph_gpu_create(_a(self.params), _a(self.terms), self.counts[0],
                                             ctypes.byref(handle)))
        else:
            self.counts = [int(c) for c in counts]
            cnt = np.array(self.counts, dtype=np.uint32)
            self.params["particles_count"] = cnt
            _check("clsph_gpu_create_batched",
                   self.lib.clsph_gpu_create_batched(_a(self.params), _a(self.terms), _a(cnt),
                                                     len(cnt), ctypes.byref(handle)))
        self.n = int(sum(self.counts))
        self.first = np.concatenate([[0], np.cumsum(self.counts)]).astype(np.int64)
        self.h = handle
        if mesh is not None:
            self.set_mesh(mesh)

    @classmethod
    def batched(cls, params_list, terms_list, counts, meshes=None):
        g = cls(np.array(list(params_list), dtype=PARAMS), np.array(list(terms_list), dtype=TERMS),
                counts=counts)
        for s, m in enumerate(meshes or []):
            if m is not None:
                g.set_mesh(m, scene=s)
        return g

    def close(self) -> None:
        if getattr(self, "h", None):
            self.lib.clsph_gpu_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # ------------------------------------------------------------ set-up
    def set_stream(self, stream_handle: int | None) -> None:
        _check("clsph_gpu_set_stream", self.lib.clsph_gpu_set_stream(self.h, stream_handle))

    def set_collision_cap(self, iterations: int) -> None:
        _check("clsph_gpu_set_collision_cap", self.lib.clsph_gpu_set_collision_cap(self.h, iterations))

    def set_mesh(self, mesh, scene: int = 0) -> None:
        normals = np.ascontiguousarray(mesh["face_normals"], dtype=np.float32)
        verts = np.ascontiguousarray(mesh["vertices"], dtype=np.float32)
        idx = np.ascontiguousarray(mesh["indices"], dtype=np.uint32)
        faces = len(idx) // 3
        if faces == 0:
            _check("clsph_gpu_set_scene_mesh",
                   self.lib.clsph_gpu_set_scene_mesh(self.h, scene, None, None, 0, None, 0))
            return
        _check("clsph_gpu_set_scene_mesh",
               self.lib.clsph_gpu_set_scene_mesh(self.h, scene, _a(normals), _a(verts),
                                                 len(verts) // 3, _a(idx), faces))

    def set_parameters(self, params, terms, scene: int = 0) -> None:
        """Replaces a scene's parameter block and kernel constants between
        substeps (include/clsph_gpu.h; the particle count cannot change)."""
        p = np.array(params, dtype=PARAMS).reshape(1).copy()
        t = np.array(terms, dtype=TERMS).reshape(1).copy()
        p["particles_count"] = self.counts[scene]
        _check("clsph_gpu_set_scene_parameters",
               self.lib.clsph_gpu_set_scene_parameters(self.h, scene, _a(p), _a(t)))
        self.params[scene] = p[0]
        self.terms[scene] = t[0]

    def set_graph(self, on: bool) -> None:
        _check("clsph_gpu_set_graph", self.lib.clsph_gpu_set_graph(self.h, 1 if on else 0))

    # ------------------------------------------------------------ transfers
    def upload(self, particles: np.ndarray) -> None:
        p = np.ascontiguousarray(particles, dtype=PARTICLE)
        if len(p) != self.n:
            raise ValueError(f"expected {self.n} particles, got {len(p)}")
        _check("clsph_gpu_upload", self.lib.clsph_gpu_upload(self.h, _a(p)))
        # the copy is asynchronous; keep the source alive until the next sync
        self._pinned_src = p

    def download(self, out: np.ndarray | None = None) -> np.ndarray:
        out = np.zeros(self.n, dtype=PARTICLE) if out is None else out
        _check("clsph_gpu_download", self.lib.clsph_gpu_download(self.h, _a(out)))
        return out

    # ------------------------------------------------------------ stepping
    def step(self, substeps: int = 1) -> None:
        _check("clsph_gpu_step", self.lib.clsph_gpu_step(self.h, substeps))

    def step_until(self, stage: int) -> None:
        _check("clsph_gpu_step_until", self.lib.clsph_gpu_step_until(self.h, stage))

    def sync(self) -> int:
        flags = _u32(0)
        _check("clsph_gpu_sync", self.lib.clsph_gpu_sync(self.h, ctypes.byref(flags)))
        return flags.value

    # ------------------------------------------------------------ inspection
    def parameters(self, scene: int = 0) -> np.void:
        out = np.zeros(1, dtype=PARAMS)
        _check("clsph_gpu_get_scene_parameters",
               self.lib.clsph_gpu_get_scene_parameters(self.h, scene, _a(out)))
        return out[0]

    def keys(self):
        keys = np.zeros(self.n, dtype=np.uint32)
        perm = np.zeros(self.n, dtype=np.uint32)
        _check("clsph_gpu_read_keys", self.lib.clsph_gpu_read_keys(self.h, _a(keys), _a(perm)))
        return keys, perm

    def cell_table(self, scene: int = 0) -> np.ndarray:
        cells = int(self.parameters(scene)["grid_cell_count"])
        table = np.zeros(max(cells, 1), dtype=np.uint32)
        _check("clsph_gpu_read_cell_table_scene",
               self.lib.clsph_gpu_read_cell_table_scene(self.h, scene, _a(table), cells))
        return table[:cells]

    def fields(self):
        rho = np.zeros(self.n, dtype=np.float32)
        prs = np.zeros(self.n, dtype=np.float32)
        acc = np.zeros((self.n, 4), dtype=np.float32)
        _check("clsph_gpu_read_fields",
               self.lib.clsph_gpu_read_fields(self.h, _a(rho), _a(prs), _a(acc)))
        return rho, prs, acc[:, :3]

    def ids(self) -> np.ndarray:
        out = np.zeros(self.n, dtype=np.uint32)
        _check("clsph_gpu_read_ids", self.lib.clsph_gpu_read_ids(self.h, _a(out)))
        return out

    def set_profiling(self, on: bool) -> None:
        _check("clsph_gpu_set_profiling", self.lib.clsph_gpu_set_profiling(self.h, 1 if on else 0))

    def kernel_times(self) -> dict:
        k = 32
        stride = 32
        names = ctypes.create_string_buffer(k * stride)
        ms = np.zeros(k, dtype=np.float32)
        counts = np.zeros(k, dtype=np.uint32)
        nk = ctypes.c_int(0)
        _check("clsph_gpu_kernel_times",
               self.lib.clsph_gpu_kernel_times(self.h, k, names, stride, _a(ms), _a(counts),
                                               ctypes.byref(nk)))
        out = {}
        for i in range(min(nk.value, k)):
            name = names.raw[i * stride:(i + 1) * stride].split(b"\0", 1)[0].decode()
            out[name] = (float(ms[i]), int(counts[i]))
        return out

    def autotune(self, substeps: int = 3) -> str:
        buf = ctypes.create_string_buffer(4096)
        _check("clsph_gpu_autotune", self.lib.clsph_gpu_autotune(self.h, substeps, buf, 4096))
        return buf.value.decode()

    def set_launch_shape(self, density_block: int, forces_block: int, advect_blocks_per_sm: int) -> None:
        _check("clsph_gpu_set_launch_shape",
               self.lib.clsph_gpu_set_launch_shape(self.h, density_block, forces_block,
                                                   advect_blocks_per_sm))

    def set_neighbour_search(self, mode: int) -> None:
        """SEARCH_WINDOW, SEARCH_CELL_WARPS or SEARCH_PARTICLE_WARPS (bit-identical results)."""
        _check("clsph_gpu_set_neighbour_search", self.lib.clsph_gpu_set_neighbour_search(self.h, mode))

    def set_wait_limits(self, radix_lookback_spins: int = DEFAULT_LOOKBACK_SPINS,
                        mlp_wait_polls: int = DEFAULT_MLP_WAIT_POLLS,
                        radix_withheld_tile: int = NO_TILE) -> None:
        """Bounds of the device-side waits; radix_withheld_tile is the test
        hook that makes one look-back wait run out (see clsph_gpu.h)."""
        _check("clsph_gpu_set_wait_limits",
               self.lib.clsph_gpu_set_wait_limits(self.h, radix_lookback_spins, mlp_wait_polls,
                                                  radix_withheld_tile))

    def set_persistent(self, on: bool) -> None:
        """Whole substeps as one persistent cooperative launch (see clsph_gpu.h)."""
        _check("clsph_gpu_set_persistent", self.lib.clsph_gpu_set_persistent(self.h, 1 if on else 0))

    def set_barrier_limits(self, barrier_spins: int = DEFAULT_BARRIER_SPINS,
                           withheld_block: int = NO_BLOCK) -> None:
        _check("clsph_gpu_set_barrier_limits",
               self.lib.clsph_gpu_set_barrier_limits(self.h, barrier_spins, withheld_block))

    def face_lists(self, scene: int = 0):
        """(plan dict, CSR starts, face lists) of the scene's per-cell
        triangle lists as built on the device; (None, None, None) without."""
        sizes = np.zeros(2, dtype=np.uint32)
        plan = np.zeros(10, dtype=np.float32)
        _check("clsph_gpu_read_face_lists",
               self.lib.clsph_gpu_read_face_lists(self.h, scene, _a(plan), None, 0, None, 0, _a(sizes)))
        if sizes[0] == 0:
            return None, None, None
        start = np.zeros(int(sizes[0]), dtype=np.uint32)
        faces = np.zeros(max(int(sizes[1]), 1), dtype=np.uint32)
        _check("clsph_gpu_read_face_lists",
               self.lib.clsph_gpu_read_face_lists(self.h, scene, None, _a(start), len(start), _a(faces),
                                                  len(faces), _a(sizes)))
        info = {"glo": plan[0:3].copy(), "cell": plan[3], "pad": plan[4], "tol": plan[5],
                "dims": plan[6:9].astype(np.int64), "reach": plan[9]}
        return info, start, faces[: int(sizes[1])]

    def counters(self) -> dict:
        c = np.zeros(3, dtype=np.uint64)
        _check("clsph_gpu_counters", self.lib.clsph_gpu_counters(self.h, _a(c)))
        return {"substeps": int(c[0]), "collision_capped": int(c[1]), "launches": int(c[2])}
