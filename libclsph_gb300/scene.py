"""`scene` of the reference (libclsph/scene.h:7-15, scene.cpp:9-67) in Python.

`Scene.load(filename)` reads `scenes/<filename>` (relative to the working
directory, like the reference; `base` overrides the folder) with the same
geometry semantics as the vendored tinyobjloader 0.9.6 the reference uses
(util/tinyobj/tiny_obj_loader.cc:118-661):

* `v`/`vn`/`vt` records parsed with C `atof` (longest numeric prefix),
* `f` records of `i`, `i/j`, `i//k`, `i/j/k` with 1-based or negative
  (relative) indices, polygons split into a triangle fan (i0, i_{k-1}, i_k),
* vertices re-indexed per shape in first-use order, de-duplicated on the
  (position, normal, texcoord) index triple,
* a new shape at every `o` / `g` record that follows faces,
* `mtllib` must name a readable file next to the scene, else loading fails.

Then, as scene.cpp does per shape: `indices` and `vertices` are REPLACED by
the shape's arrays while one unit normal per face (cross product of the two
edges from the first vertex) is APPENDED to `face_normals`, so a multi-shape
file keeps the last shape's mesh but every shape's normals (the reference's
behaviour; `fix_multi_shape=True` concatenates the shapes instead).
"""

from __future__ import annotations

import re
import sys
from pathlib import Path

import numpy as np

_FLOAT_PREFIX = re.compile(r"[ \t\n\v\f\r]*([+-]?(?:(?:\d+\.?\d*|\.\d+)(?:[eE][+-]?\d+)?|inf(?:inity)?|nan))",
                           re.IGNORECASE)
_INT_PREFIX = re.compile(r"[ \t\n\v\f\r]*([+-]?\d+)")


def c_atof(s: str) -> float:
    m = _FLOAT_PREFIX.match(s)
    return float(m.group(1)) if m else 0.0


def c_atoi(s: str) -> int:
    m = _INT_PREFIX.match(s)
    if not m:
        return 0
    v = int(m.group(1))
    return ((v + 2**31) % 2**32) - 2**31


def _fix_index(idx: int, n: int) -> int:
    if idx > 0:
        return idx - 1
    if idx == 0:
        return 0
    return n + idx


def _span(s: str, i: int, chars: str) -> int:
    while i < len(s) and s[i] in chars:
        i += 1
    return i


def _cspan(s: str, i: int, chars: str) -> int:
    while i < len(s) and s[i] not in chars:
        i += 1
    return i


def _parse_triple(s: str, i: int, vsize: int, vnsize: int, vtsize: int):
    v = _fix_index(c_atoi(s[i:]), vsize)
    vt = vn = -1
    i = _cspan(s, i, "/ \t\r")
    if i < len(s) and s[i] == "/":
        i += 1
        if i < len(s) and s[i] == "/":
            i += 1
            vn = _fix_index(c_atoi(s[i:]), vnsize)
            i = _cspan(s, i, "/ \t\r")
        else:
            vt = _fix_index(c_atoi(s[i:]), vtsize)
            i = _cspan(s, i, "/ \t\r")
            if i < len(s) and s[i] == "/":
                i += 1
                vn = _fix_index(c_atoi(s[i:]), vnsize)
                i = _cspan(s, i, "/ \t\r")
    return (v, vn, vt), i


def _parse_floats(s: str, i: int, count: int):
    out = []
    for _ in range(count):
        i = _span(s, i, " \t")
        out.append(np.float32(c_atof(s[i:])))
        i = _cspan(s, i, " \t\r")
    return out, i


class ObjError(RuntimeError):
    pass


def load_obj_shapes(path: Path, mtl_base: Path):
    """Shapes of an OBJ file as (name, positions[float32], indices[uint32])."""
    try:
        raw = Path(path).read_bytes()
    except OSError:
        raise ObjError(f"Cannot open file [{path}]")
    text = raw.decode("latin-1")
    v: list = []
    vn: list = []
    vt: list = []
    group: list = []
    shapes = []
    name = ""

    def flush():
        if not group:
            return
        cache: dict = {}
        pos: list = []
        idx: list = []

        def vertex(key):
            if key in cache:
                return cache[key]
            vi = key[0]
            if vi < 0 or 3 * vi + 2 >= len(v):
                raise ObjError(f"{path}: vertex index out of range")
            pos.extend(v[3 * vi:3 * vi + 3])
            cache[key] = len(pos) // 3 - 1
            return cache[key]

        for face in group:
            for k in range(2, len(face)):
                a, b, c = face[0], face[k - 1], face[k]
                ia = vertex(a)
                ib = vertex(b)
                ic = vertex(c)
                idx += [ia, ib, ic]
        shapes.append((name, np.array(pos, dtype=np.float32), np.array(idx, dtype=np.uint32)))
        group.clear()

    for line in text.split("\n"):
        line = line[:8191]
        i = _span(line, 0, " \t")
        if i >= len(line) or line[i] == "#":
            continue
        rest = line[i:]
        if rest.startswith("v") and len(rest) > 1 and rest[1] in " \t":
            vals, _ = _parse_floats(rest, 2, 3)
            v.extend(vals)
        elif rest.startswith("vn") and len(rest) > 2 and rest[2] in " \t":
            vals, _ = _parse_floats(rest, 3, 3)
            vn.extend(vals)
        elif rest.startswith("vt") and len(rest) > 2 and rest[2] in " \t":
            vals, _ = _parse_floats(rest, 3, 2)
            vt.extend(vals)
        elif rest.startswith("f") and len(rest) > 1 and rest[1] in " \t":
            j = _span(rest, 2, " \t")
            face = []
            while j < len(rest) and rest[j] not in "\r\n\0":
                key, j = _parse_triple(rest, j, len(v) // 3, len(vn) // 3, len(vt) // 2)
                face.append(key)
                j = _span(rest, j, " \t\r")
            group.append(face)
        elif rest.startswith("mtllib") and len(rest) > 6 and rest[6] in " \t":
            fname = rest[7:].split()[0] if rest[7:].split() else ""
            if not (Path(mtl_base) / fname).is_file():
                raise ObjError(f"Cannot open file [{Path(mtl_base) / fname}]")
        elif rest.startswith("g") and len(rest) > 1 and rest[1] in " \t":
            flush()
            toks = rest.replace("\r", "").split()
            name = toks[1] if len(toks) > 1 else ""
        elif rest.startswith("o") and len(rest) > 1 and rest[1] in " \t":
            flush()
            toks = rest[2:].split()
            name = toks[0] if toks else ""
    flush()
    return shapes


def _normals(vertices: np.ndarray, indices: np.ndarray) -> np.ndarray:
    from .workloads import face_normals

    if len(indices) == 0:
        return np.zeros(0, dtype=np.float32)
    return face_normals(vertices, indices)


class Scene:
    """scene (libclsph/scene.h:7-15): face_count, face_normals, vertices, indices."""

    def __init__(self):
        self.face_count = 0
        self.face_normals = np.zeros(0, dtype=np.float32)
        self.vertices = np.zeros(0, dtype=np.float32)
        self.indices = np.zeros(0, dtype=np.uint32)

    def load(self, filename: str, base: str | Path = "scenes", fix_multi_shape: bool = False) -> bool:
        base = Path(base)
        try:
            shapes = load_obj_shapes(base / filename, base)
        except ObjError as e:
            sys.stderr.write(f"{e}\n")
            return False
        print(f"Scene Loading - number of shapes in file [{filename}]: {len(shapes)}")
        if fix_multi_shape and shapes:
            verts, idx, off = [], [], 0
            for _, pos, ind in shapes:
                verts.append(pos)
                idx.append(ind.astype(np.int64) + off)
                off += len(pos) // 3
            shapes = [("", np.concatenate(verts), np.concatenate(idx).astype(np.uint32))]
        normals = [self.face_normals]
        for _, pos, ind in shapes:
            if len(ind) % 3 != 0:
                sys.stderr.write("Meshes must be made of triangles only\n")
                return False
            self.indices = ind
            self.face_count = len(ind) // 3
            self.vertices = pos
            normals.append(_normals(pos, ind))
        self.face_normals = np.concatenate(normals).astype(np.float32)
        return True

    def mesh(self) -> dict:
        """Arrays as the engine wants them (the normals of the current mesh's faces)."""
        return {"vertices": self.vertices, "indices": self.indices,
                "face_normals": self.face_normals[: 3 * self.face_count]
                if len(self.face_normals) >= 3 * self.face_count else self.face_normals}
