"""ctypes bindings of the CPU oracles — TEST INFRASTRUCTURE.

`Oracle` wraps oracle/liboracle.so (the restatement in clsph_oracle.cpp);
`RefBuild` wraps oracle/_ref/libclsph_ref.so (the reference's own kernel
sources compiled through oracle/ref_shim, development container only).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import
this package. The product never does.
"""

from __future__ import annotations

import ctypes
import os
import subprocess
from pathlib import Path

import numpy as np

from libclsph_gb300.layout import PARAMS, PARTICLE, TERMS

HERE = Path(__file__).resolve().parent
ORACLE_SO = HERE / "liboracle.so"
REF_SO = HERE / "_ref" / "libclsph_ref.so"

_u32p = ctypes.POINTER(ctypes.c_uint32)
_vp = ctypes.c_void_p


def build_oracle(force: bool = False) -> Path:
    if force or not ORACLE_SO.exists():
        subprocess.run(["make", "-s", "-C", str(HERE), "liboracle.so"], check=True)
    return ORACLE_SO


def _make_args(reference_root: str | None) -> list[str]:
    """REF=... for the Makefile: the argument, else CLSPH_REFERENCE_ROOT, else
    the Makefile's own default."""
    root = reference_root or os.environ.get("CLSPH_REFERENCE_ROOT")
    return [f"REF={root}"] if root else []


def reference_root() -> Path:
    """Where the reference checkout is looked for (CLSPH_REFERENCE_ROOT, else
    the Makefile's default); it may not exist on this machine."""
    out = subprocess.run(["make", "-s", "-C", str(HERE), "print-ref", *_make_args(None)],
                         capture_output=True, text=True)
    return Path(out.stdout.strip() or "/nonexistent")


def build_ref(reference_root: str | None = None) -> Path | None:
    """Builds oracle/_ref when the reference sources are present; else None."""
    args = _make_args(reference_root)
    if subprocess.run(["make", "-s", "-C", str(HERE), "has-ref", *args],
                      capture_output=True).returncode != 0:
        return None
    subprocess.run(["make", "-s", "-C", str(HERE), "ref", *args], check=True)
    return REF_SO


def _addr(a):
    return None if a is None else a.ctypes.data


class StepResult:
    """Outputs of one substep: params (grid filled), perm, cell table, AoS
    snapshots after sort / density / forces, the final AoS and the number of
    particles whose collision loop hit the cap."""

    def __init__(self, params, perm, table, sorted_, density, forces, final, capped):
        self.params = params
        self.perm = perm
        self.table = table
        self.sorted = sorted_
        self.density = density
        self.forces = forces
        self.final = final
        self.capped = capped


def _mesh_args(mesh):
    if mesh is None:
        return None, None, None, 0
    normals = np.ascontiguousarray(mesh["face_normals"], dtype=np.float32)
    verts = np.ascontiguousarray(mesh["vertices"], dtype=np.float32)
    idx = np.ascontiguousarray(mesh["indices"], dtype=np.uint32)
    return normals, verts, idx, len(idx) // 3


class _StepLib:
    _step_name = ""

    def _run_step(self, fn, params, terms, particles, mesh, max_iters, extra):
        n = len(particles)
        p_in = np.array(params, dtype=PARAMS).reshape(1)
        p_out = np.zeros(1, dtype=PARAMS)
        t_in = np.array(terms, dtype=TERMS).reshape(1)
        io = np.ascontiguousarray(particles, dtype=PARTICLE).copy()
        perm = np.zeros(n, dtype=np.uint32)
        snaps = [np.zeros(n, dtype=PARTICLE) for _ in range(3)]
        normals, verts, idx, faces = _mesh_args(mesh)
        # a first call learns the cell count, then the table is fetched
        capped = ctypes.c_uint32(0)
        rc = fn(
            _addr(p_in), _addr(p_out), _addr(t_in), _addr(normals), _addr(verts), _addr(idx),
            faces, _addr(io), n, _addr(perm), None, 0, _addr(snaps[0]), _addr(snaps[1]),
            _addr(snaps[2]), max_iters, ctypes.byref(capped), *extra,
        )
        if rc != 0:
            raise RuntimeError(f"{self._step_name} failed with status {rc}")
        cells = int(p_out["grid_cell_count"][0])
        table = np.zeros(max(cells, 1), dtype=np.uint32)
        io2 = np.ascontiguousarray(particles, dtype=PARTICLE).copy()
        rc = fn(
            _addr(p_in), None, _addr(t_in), _addr(normals), _addr(verts), _addr(idx), faces,
            _addr(io2), n, None, _addr(table), cells, None, None, None, max_iters, None, *extra,
        )
        if rc != 0:
            raise RuntimeError(f"{self._step_name} failed with status {rc}")
        return StepResult(p_out[0], perm, table[:cells], snaps[0], snaps[1], snaps[2], io,
                          capped.value)


class Oracle(_StepLib):
    _step_name = "clsph_oracle_step"

    def __init__(self, path: Path | None = None):
        self.lib = ctypes.CDLL(str(path or build_oracle()))
        L = self.lib
        L.clsph_oracle_step.restype = ctypes.c_int
        L.clsph_oracle_step.argtypes = [_vp, _vp, _vp, _vp, _vp, _vp, ctypes.c_uint32, _vp,
                                        ctypes.c_uint32, _vp, _vp, ctypes.c_uint64, _vp, _vp,
                                        _vp, ctypes.c_uint32, _vp, ctypes.c_int]
        L.clsph_oracle_run.restype = ctypes.c_int
        L.clsph_oracle_run.argtypes = [_vp, _vp, _vp, _vp, _vp, ctypes.c_uint32, _vp,
                                       ctypes.c_uint32, ctypes.c_uint32, ctypes.c_int]
        L.clsph_oracle_fields_f64.restype = ctypes.c_int
        L.clsph_oracle_fields_f64.argtypes = [_vp, _vp, ctypes.c_uint32, _vp, _vp, _vp, _vp,
                                              ctypes.c_int]
        L.clsph_oracle_derive.restype = None
        L.clsph_oracle_derive.argtypes = [_vp, _vp, ctypes.c_int, ctypes.POINTER(ctypes.c_float)]
        L.clsph_oracle_init_lattice.restype = None
        L.clsph_oracle_init_lattice.argtypes = [_vp, ctypes.c_uint32, ctypes.c_float]
        L.clsph_oracle_morton.restype = ctypes.c_uint32
        L.clsph_oracle_morton.argtypes = [ctypes.c_uint32] * 3
        L.clsph_oracle_cell_coords.restype = None
        L.clsph_oracle_cell_coords.argtypes = [ctypes.c_uint32, _u32p]

    def step(self, params, terms, particles, mesh=None, max_iters=0, threads=0) -> StepResult:
        return self._run_step(self.lib.clsph_oracle_step, params, terms, particles, mesh,
                              max_iters, (threads,))

    def run(self, params, terms, particles, steps, mesh=None, threads=0) -> np.ndarray:
        p_in = np.array(params, dtype=PARAMS).reshape(1)
        t_in = np.array(terms, dtype=TERMS).reshape(1)
        io = np.ascontiguousarray(particles, dtype=PARTICLE).copy()
        normals, verts, idx, faces = _mesh_args(mesh)
        rc = self.lib.clsph_oracle_run(_addr(p_in), _addr(t_in), _addr(normals), _addr(verts),
                                       _addr(idx), faces, _addr(io), len(io), steps, threads)
        if rc != 0:
            raise RuntimeError(f"clsph_oracle_run failed with status {rc}")
        return io

    def fields_f64(self, params, sorted_aos, table, threads=0):
        n = len(sorted_aos)
        p_in = np.array(params, dtype=PARAMS).reshape(1)
        aos = np.ascontiguousarray(sorted_aos, dtype=PARTICLE)
        tab = np.ascontiguousarray(table, dtype=np.uint32)
        rho = np.zeros(n)
        prs = np.zeros(n)
        acc = np.zeros((n, 3))
        rc = self.lib.clsph_oracle_fields_f64(_addr(p_in), _addr(aos), n, _addr(tab), _addr(rho),
                                              _addr(prs), _addr(acc), threads)
        if rc != 0:
            raise RuntimeError(f"clsph_oracle_fields_f64 failed with status {rc}")
        return rho, prs, acc

    def derive(self, params, influence_count):
        p = np.array(params, dtype=PARAMS).reshape(1).copy()
        t = np.zeros(1, dtype=TERMS)
        vol = ctypes.c_float(0)
        self.lib.clsph_oracle_derive(_addr(p), _addr(t), influence_count, ctypes.byref(vol))
        return p[0], t[0], vol.value

    def init_lattice(self, n, initial_volume):
        out = np.zeros(n, dtype=PARTICLE)
        self.lib.clsph_oracle_init_lattice(_addr(out), n, initial_volume)
        return out

    def morton(self, x, y, z):
        return self.lib.clsph_oracle_morton(x, y, z)

    def cell_coords(self, key):
        buf = (ctypes.c_uint32 * 3)()
        self.lib.clsph_oracle_cell_coords(key, buf)
        return tuple(buf)


class RefBuild(_StepLib):
    """The reference's kernel sources compiled as C++ (oracle/_ref)."""

    _step_name = "clsph_ref_step"

    def __init__(self, path: Path | None = None):
        path = path or REF_SO
        if not Path(path).exists():
            raise FileNotFoundError(f"{path} not built (make -C oracle ref)")
        self.lib = ctypes.CDLL(str(path))
        L = self.lib
        L.clsph_ref_step.restype = ctypes.c_int
        L.clsph_ref_step.argtypes = [_vp, _vp, _vp, _vp, _vp, _vp, ctypes.c_uint32, _vp,
                                     ctypes.c_uint32, _vp, _vp, ctypes.c_uint64, _vp, _vp, _vp,
                                     ctypes.c_uint32, _vp]
        L.clsph_ref_morton.restype = ctypes.c_uint32
        L.clsph_ref_morton.argtypes = [ctypes.c_uint32] * 3
        L.clsph_ref_cell_coords.restype = None
        L.clsph_ref_cell_coords.argtypes = [ctypes.c_uint32, _u32p]
        L.clsph_ref_smoothing.restype = None
        L.clsph_ref_smoothing.argtypes = [ctypes.c_float] * 4 + [_vp, _vp]

    def step(self, params, terms, particles, mesh=None, max_iters=0) -> StepResult:
        return self._run_step(self.lib.clsph_ref_step, params, terms, particles, mesh, max_iters,
                              ())

    def morton(self, x, y, z):
        return self.lib.clsph_ref_morton(x, y, z)

    def cell_coords(self, key):
        buf = (ctypes.c_uint32 * 3)()
        self.lib.clsph_ref_cell_coords(key, buf)
        return tuple(buf)

    def smoothing(self, r, h, terms):
        t = np.array(terms, dtype=TERMS).reshape(1)
        out = np.zeros(9, dtype=np.float32)
        self.lib.clsph_ref_smoothing(float(r[0]), float(r[1]), float(r[2]), float(h), _addr(t),
                                     _addr(out))
        return out


def have_ref() -> bool:
    if REF_SO.exists():
        return True
    return subprocess.run(["make", "-s", "-C", str(HERE), "has-ref", *_make_args(None)],
                          capture_output=True).returncode == 0


__all__ = ["Oracle", "RefBuild", "StepResult", "build_oracle", "build_ref", "have_ref", "reference_root",
           "ORACLE_SO", "REF_SO"]

os.environ.setdefault("OMP_WAIT_POLICY", "PASSIVE")
