"""Binary .bgeo frames: the delegate the reference selects with USE_PARTIO
(libclsph/file_save_delegates/houdini_file_saver.cpp:76-88, attributes of
util/partio/PartioFunctions.h:5-65).

Partio is not part of the reference tree, so these files cannot be compared
with Partio's own output here. The tests decode every byte with a reader of
their own (classic binary Houdini geometry, version 5, big-endian), check each
attribute value against the particle array, and require the Python and C++
writers to agree byte for byte."""

import struct
import subprocess
from pathlib import Path

import numpy as np
import pytest

from libclsph_gb300.layout import PARAMS, PARTICLE
from libclsph_gb300.simulation import HoudiniFileSaver

ROOT = Path(__file__).resolve().parents[1]


class Reader:
    def __init__(self, data: bytes):
        self.d, self.o = data, 0

    def take(self, fmt: str):
        v = struct.unpack_from(">" + fmt, self.d, self.o)
        self.o += struct.calcsize(">" + fmt)
        return v if len(v) > 1 else v[0]

    def name(self) -> str:
        n = self.take("H")
        s = self.d[self.o:self.o + n].decode()
        self.o += n
        return s


def decode(data: bytes):
    r = Reader(data)
    assert data[:5] == b"BgeoV"
    r.o = 5
    version, npts, nprims, npg, nprg, npa, nva, nra, nda = r.take("9i")
    assert (version, nprims, npg, nprg, nva, nda) == (5, 1, 0, 0, 0, 0)
    attrs = []
    for _ in range(npa):
        nm, size, typ = r.name(), r.take("H"), r.take("i")
        defaults = [r.take("i") for _ in range(size)]
        assert defaults == [0] * size
        attrs.append((nm, size, typ))
    points = []
    for _ in range(npts):
        pos = r.take("4f")
        vals = {}
        for nm, size, typ in attrs:
            code = "i" if typ == 1 else "f"
            vals[nm] = r.take(code * size) if size > 1 else (r.take(code),)
        points.append((pos, vals))
    prim_attrs = []
    for _ in range(nra):
        nm, size, typ = r.name(), r.take("H"), r.take("i")
        assert typ == 4  # index attribute: a string table
        strings = [r.name() for _ in range(r.take("i"))]
        prim_attrs.append((nm, size, strings))
    assert r.take("i") == 0x8000  # particle system primitive
    count = r.take("i")
    index = [r.take("H" if npts <= 65535 else "i") for _ in range(count)]
    prim_values = [r.take("i") for _ in range(nra)]
    assert data[r.o:] == b"\x00\xff"
    return dict(attrs=attrs, points=points, prim_attrs=prim_attrs, index=index,
                prim_values=prim_values)


def frame(n, seed):
    rng = np.random.default_rng(seed)
    parts = np.zeros(n, dtype=PARTICLE)
    parts["position"][:, :3] = rng.normal(0, 1, (n, 3))
    parts["velocity"][:, :3] = rng.normal(0, 1, (n, 3))
    parts["density"] = rng.uniform(-100, 2200, n)
    parts["density"][:min(n, 7)] = [0, 500, 1000, 1500, 2000, -1, 999.5][:min(n, 7)]
    params = np.zeros(1, dtype=PARAMS)
    params["particles_count"] = n
    params["particle_mass"] = 0.0425
    params["h"] = 0.0620705
    return parts, params


def ramp(d):
    """makeData's colour ramp (PartioFunctions.h:39-55), one float32 at a time."""
    f = np.float32
    d = f(d)
    r = (d - f(1000)) / f(1000) if 1000 < d <= 2000 else f(0)
    g = f(1) - d / f(1000) if 0 <= d < 1000 else f(0)
    if 500 <= d <= 1000:
        b = (d - f(500)) / f(500)
    elif 1000 <= d <= 1500:
        b = f(1) - (d - f(1000)) / f(500)
    else:
        b = f(0)
    return (float(r), float(g), float(b))


def test_bgeo_decodes_to_the_particle_array(tmp_path):
    parts, params = frame(300, 5)
    (tmp_path / "frames").mkdir()
    HoudiniFileSaver(str(tmp_path) + "/", binary_bgeo=True).writeFrameToFile(parts, params[0])
    g = decode((tmp_path / "frames" / "frame0000001.bgeo").read_bytes())
    assert g["attrs"] == [("velocity", 3, 5), ("color", 3, 5), ("id", 1, 1), ("mass", 1, 0),
                          ("pscale", 1, 0)]
    assert g["prim_attrs"] == [("generator", 1, ["papi"])]
    assert g["prim_values"] == [0]
    assert g["index"] == list(range(300))
    f32 = lambda x: float(np.float32(x))  # noqa: E731
    for i, (pos, vals) in enumerate(g["points"]):
        assert pos == tuple(f32(x) for x in parts["position"][i, :3]) + (1.0,)
        assert vals["velocity"] == tuple(f32(x) for x in parts["velocity"][i, :3])
        assert vals["color"] == ramp(parts["density"][i])
        assert vals["id"] == (i,)
        assert vals["mass"] == (f32(0.0425),)
        assert vals["pscale"] == (f32(0.0620705),)


@pytest.mark.parametrize("n", [0, 1, 65535, 65536, 70001])
def test_bgeo_point_index_width(tmp_path, n):
    """16-bit point indices up to 65,535 points, 32-bit above."""
    parts, params = frame(n, 6)
    (tmp_path / "frames").mkdir()
    HoudiniFileSaver(str(tmp_path) + "/", binary_bgeo=True).writeFrameToFile(parts, params[0])
    data = (tmp_path / "frames" / "frame0000001.bgeo").read_bytes()
    head = 5 + 9 * 4 + sum(2 + len(nm) + 2 + 4 + 4 * sz for nm, sz in
                           (("velocity", 3), ("color", 3), ("id", 1), ("mass", 1), ("pscale", 1)))
    prim = 2 + 9 + 2 + 4 + 4 + 2 + 4 + 4 + 4
    width = 2 if n <= 65535 else 4
    assert len(data) == head + 52 * n + prim + width * n + 4 + 2
    if n <= 2000:
        assert decode(data)["index"] == list(range(n))
    else:
        idx = np.frombuffer(data, dtype=">u2" if width == 2 else ">i4", count=n,
                            offset=head + 52 * n + prim)
        assert np.array_equal(idx, np.arange(n))


@pytest.mark.parametrize("n", [50, 70001])
def test_bgeo_python_and_cpp_agree(tmp_path, n):
    """The C++ saver (threaded for large frames) writes the same bytes."""
    import ctypes

    from libclsph_gb300.build import build_gpu, build_host

    build_gpu()
    build_host()
    lib = ctypes.CDLL(str(ROOT / "libclsph_gb300" / "_lib" / "libclsph.so"))
    lib.clsph_host_write_bgeo.argtypes = [ctypes.c_char_p, ctypes.c_void_p, ctypes.c_void_p]
    parts, params = frame(n, 7)
    for d in ("py", "cpp"):
        (tmp_path / d / "frames").mkdir(parents=True)
    HoudiniFileSaver(str(tmp_path / "py") + "/", binary_bgeo=True).writeFrameToFile(parts, params[0])
    assert lib.clsph_host_write_bgeo((str(tmp_path / "cpp") + "/").encode(), parts.ctypes.data,
                                     params.ctypes.data) == 0
    a = (tmp_path / "py" / "frames" / "frame0000001.bgeo").read_bytes()
    b = (tmp_path / "cpp" / "frames" / "frame0000001.bgeo").read_bytes()
    assert a == b


def test_use_partio_build_writes_bgeo(tmp_path):
    """Code compiled with -DUSE_PARTIO, as the reference's Partio build is,
    gets savers that write .bgeo frames; without it, .geo."""
    from test_abi import compile_against_dropin

    src = tmp_path / "saver.cpp"
    src.write_text(
        '#include "file_save_delegates/houdini_file_saver.h"\n'
        "int main(int, char** argv) {\n"
        "  particle p[2] = {};\n"
        "  simulation_parameters prm = {};\n"
        "  prm.particles_count = 2;\n"
        "  houdini_file_saver s(argv[1]);\n"
        "  return s.writeFrameToFile(p, prm);\n"
        "}\n")
    for define, ext in ((True, ".bgeo"), (False, ".geo")):
        out = tmp_path / ("with" if define else "without")
        (out / "frames").mkdir(parents=True)
        exe = tmp_path / f"saver_{ext[1:]}"
        if define:
            src2 = tmp_path / "saver_partio.cpp"
            src2.write_text("#define USE_PARTIO\n" + src.read_text())
            r = compile_against_dropin(src2, exe)
        else:
            r = compile_against_dropin(src, exe)
        assert r.returncode == 0, r.stderr
        run = subprocess.run([str(exe), str(out) + "/"], capture_output=True, text=True)
        assert run.returncode == 0, run.stderr
        assert [p.name for p in (out / "frames").iterdir()] == ["frame0000001" + ext]
