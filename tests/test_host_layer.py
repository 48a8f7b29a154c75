"""Host logic on CPU: property files and derived parameters, the OBJ scene
reader, the Houdini .geo writer, last_frame.bin, and the C++ host library
(libclsph.so) against the Python mirror and the oracle."""

import ctypes
import json
from pathlib import Path

import numpy as np
import pytest

from libclsph_gb300 import settings as S
from libclsph_gb300.layout import PARAMS, PARTICLE, TERMS
from libclsph_gb300.scene import Scene, load_obj_shapes
from libclsph_gb300.simulation import HoudiniFileSaver, init_lattice

ROOT = Path(__file__).resolve().parents[1]
HOST_SO = ROOT / "libclsph_gb300" / "_lib" / "libclsph.so"
def _reference_root():
    from oracle import reference_root

    return reference_root()


REF_ROOT = _reference_root()  # the reference checkout, where this machine has one
REF_SCENES = REF_ROOT / "scenes"


@pytest.fixture(scope="module")
def host():
    if not HOST_SO.exists():
        from libclsph_gb300.build import build_gpu, build_host

        build_gpu()
        build_host()
    lib = ctypes.CDLL(str(HOST_SO))
    vp = ctypes.c_void_p
    lib.clsph_host_load_settings.argtypes = [ctypes.c_char_p, ctypes.c_char_p, vp, vp,
                                             ctypes.POINTER(ctypes.c_float),
                                             ctypes.POINTER(ctypes.c_int),
                                             ctypes.POINTER(ctypes.c_int)]
    lib.clsph_host_last_error.restype = ctypes.c_char_p
    lib.clsph_host_scene_new.restype = vp
    lib.clsph_host_scene_load.argtypes = [vp, ctypes.c_char_p]
    lib.clsph_host_scene_sizes.argtypes = [vp, ctypes.POINTER(ctypes.c_uint32)] + \
        [ctypes.POINTER(ctypes.c_uint64)] * 3
    lib.clsph_host_scene_copy.argtypes = [vp, vp, vp, vp]
    lib.clsph_host_scene_free.argtypes = [vp]
    lib.clsph_host_scene_set_fix_multi_shape.argtypes = [vp, ctypes.c_int]
    lib.clsph_host_write_houdini.argtypes = [ctypes.c_char_p, vp, vp]
    return lib


def write_props(tmp, fluid, sim, trailer=";\n"):
    f = tmp / "fluid.json"
    s = tmp / "sim.json"
    f.write_text(json.dumps(fluid, indent=4) + trailer)
    s.write_text(json.dumps(sim, indent=4) + trailer)
    return f, s


def host_settings(host, f, s):
    p = np.zeros(1, dtype=PARAMS)
    t = np.zeros(1, dtype=TERMS)
    vol = ctypes.c_float()
    wa, se = ctypes.c_int(), ctypes.c_int()
    rc = host.clsph_host_load_settings(str(f).encode(), str(s).encode(), p.ctypes.data,
                                       t.ctypes.data, ctypes.byref(vol), ctypes.byref(wa),
                                       ctypes.byref(se))
    return rc, p[0], t[0], vol.value, bool(wa.value), bool(se.value)


@pytest.mark.parametrize("fluid", [S.WATER, {"fluid_density": 1000, "dynamic_viscosity": 36,
                                             "restitution": 0.5, "k": 5,
                                             "surface_tension_threshold": 5, "surface_tension": 6,
                                             "particles_inside_influence_radius": 40}])
@pytest.mark.parametrize("n", [32000, 32768, 1000, 1 << 20])
def test_derived_parameters_match_oracle_and_cpp(tmp_path, oracle, host, fluid, n):
    sim = dict(S.DEFAULT_SIM, particles_count=n)
    f, s = write_props(tmp_path, fluid, sim)
    st = S.load_settings(f, s)
    # oracle restatement of sph_simulation.cpp:490-505
    raw = np.zeros(1, dtype=PARAMS)[0]
    for k in PARAMS.names:
        raw[k] = st.params[k]
    op, ot, ovol = oracle.derive(raw, int(fluid["particles_inside_influence_radius"]))
    for k in ("h", "time_delta", "max_velocity", "total_mass"):
        assert np.float32(st.params[k]) == np.float32(op[k]), k
    assert np.array(st.terms).tobytes() == np.array(ot).tobytes()
    assert np.float32(st.initial_volume) == np.float32(ovol)
    # the C++ host library
    rc, hp, ht, hvol, wa, se = host_settings(host, f, s)
    assert rc == 0, host.clsph_host_last_error()
    assert np.array(hp).tobytes() == np.array(st.params).tobytes()
    assert np.array(ht).tobytes() == np.array(st.terms).tobytes()
    assert np.float32(hvol) == np.float32(st.initial_volume)
    assert (wa, se) == (st.write_intermediate_frames, st.serialize)


def test_water_default_h():
    st = S.settings_from_dicts(S.WATER, S.DEFAULT_SIM)
    assert abs(float(st.params["h"]) - 0.0620705) < 1e-6
    assert abs(float(st.params["max_velocity"]) - 2.97938) < 1e-4


def test_reference_property_files(host):
    base = REF_ROOT
    if not base.is_dir():
        pytest.skip("reference files not present")
    for fluid in ("water", "mucus"):
        f = base / "fluid_properties" / f"{fluid}.json"
        s = base / "simulation_properties" / "default.json"
        st = S.load_settings(f, s)
        rc, hp, ht, *_ = host_settings(host, f, s)
        assert rc == 0
        assert np.array(hp).tobytes() == np.array(st.params).tobytes()
        assert np.array(ht).tobytes() == np.array(st.terms).tobytes()


def test_bad_restitution_and_missing_keys(tmp_path, host):
    f, s = write_props(tmp_path, dict(S.WATER, restitution=1.5), S.DEFAULT_SIM)
    with pytest.raises(ValueError, match="Restitution"):
        S.load_settings(f, s)
    rc, *_ = host_settings(host, f, s)
    assert rc != 0 and b"Restitution" in host.clsph_host_last_error()
    bad = dict(S.WATER)
    del bad["k"]
    f, s = write_props(tmp_path, bad, S.DEFAULT_SIM)
    with pytest.raises(KeyError):
        S.load_settings(f, s)
    rc, *_ = host_settings(host, f, s)
    assert rc != 0 and b"'k'" in host.clsph_host_last_error()


# ------------------------------------------------------------------ OBJ scenes
OBJ_CASES = {
    "quad_fan.obj": "v 0 0 0\nv 1 0 0\nv 1 1 0\nv 0 1 0\nv 0.5 1.5 0\nf 1 2 3 4 5\n",
    "forms.obj": ("# all index forms\nv 0 0 0\nv 1 0 0\nv 0 1 0\nv 0 0 1\nvt 0 0\nvt 1 0\n"
                  "vn 0 0 1\nf 1/1 2/2 3/1\nf 1//1 3//1 4//1\nf 1/1/1 2/2/1 4/1/1\nf -4 -3 -1\n"),
    "crlf.obj": "v 0 0 0\r\nv 2.5e-1 0 0\r\nv 0 1 0\r\n\r\nf 1 2 3\r\n",
    "shapes.obj": ("v 0 0 0\nv 1 0 0\nv 0 1 0\nv 0 0 1\no first\nf 1 2 3\ng second\n"
                   "f 1 3 4\nf 2 3 4\n"),
    "missing_mtl.obj": "mtllib nothere.mtl\nv 0 0 0\nv 1 0 0\nv 0 1 0\nf 1 2 3\n",
}


def cpp_scene(host, name):
    s = host.clsph_host_scene_new()
    ok = host.clsph_host_scene_load(s, name.encode())
    fc = ctypes.c_uint32()
    nn, nv, ni = ctypes.c_uint64(), ctypes.c_uint64(), ctypes.c_uint64()
    host.clsph_host_scene_sizes(s, ctypes.byref(fc), ctypes.byref(nn), ctypes.byref(nv),
                                ctypes.byref(ni))
    normals = np.zeros(nn.value, np.float32)
    verts = np.zeros(nv.value, np.float32)
    idx = np.zeros(ni.value, np.uint32)
    host.clsph_host_scene_copy(s, normals.ctypes.data, verts.ctypes.data, idx.ctypes.data)
    host.clsph_host_scene_free(s)
    return bool(ok), fc.value, normals, verts, idx


@pytest.mark.parametrize("name", sorted(OBJ_CASES))
def test_obj_reader_python_and_cpp_agree(tmp_path, host, name, monkeypatch):
    scenes = tmp_path / "scenes"
    scenes.mkdir()
    (scenes / name).write_text(OBJ_CASES[name])
    monkeypatch.chdir(tmp_path)
    py = Scene()
    ok = py.load(name)
    ok2, fc, normals, verts, idx = cpp_scene(host, name)
    assert ok == ok2
    if not ok:
        assert name == "missing_mtl.obj"
        return
    assert fc == py.face_count
    assert np.array_equal(idx, py.indices)
    assert np.array_equal(verts, py.vertices)
    assert np.array_equal(normals.view(np.uint32), py.face_normals.view(np.uint32))


@pytest.mark.parametrize("name", ["shapes.obj", "quad_fan.obj"])
def test_fix_multi_shape_python_and_cpp_agree(tmp_path, host, name, monkeypatch):
    """With fix_multi_shape every shape's faces form one mesh (scene.cpp:23-33
    keeps only the last shape's); one-shape files are unchanged."""
    scenes = tmp_path / "scenes"
    scenes.mkdir()
    (scenes / name).write_text(OBJ_CASES[name])
    monkeypatch.chdir(tmp_path)
    py = Scene()
    assert py.load(name, fix_multi_shape=True)
    s = host.clsph_host_scene_new()
    host.clsph_host_scene_set_fix_multi_shape(s, 1)
    assert host.clsph_host_scene_load(s, name.encode()) == 1
    fc = ctypes.c_uint32()
    nn, nv, ni = ctypes.c_uint64(), ctypes.c_uint64(), ctypes.c_uint64()
    host.clsph_host_scene_sizes(s, ctypes.byref(fc), ctypes.byref(nn), ctypes.byref(nv),
                                ctypes.byref(ni))
    normals = np.zeros(nn.value, np.float32)
    verts = np.zeros(nv.value, np.float32)
    idx = np.zeros(ni.value, np.uint32)
    host.clsph_host_scene_copy(s, normals.ctypes.data, verts.ctypes.data, idx.ctypes.data)
    host.clsph_host_scene_free(s)
    faces = sum(1 for line in OBJ_CASES[name].splitlines() if line.startswith("f "))
    if name == "quad_fan.obj":
        faces = 3  # one pentagon, fanned
        plain = Scene()
        assert plain.load(name)
        assert np.array_equal(plain.indices, py.indices)
    assert fc.value == py.face_count == faces
    assert len(normals) == 3 * faces
    assert np.array_equal(idx, py.indices) and np.array_equal(verts, py.vertices)
    assert np.array_equal(normals.view(np.uint32), py.face_normals.view(np.uint32))


def test_obj_reader_semantics(tmp_path):
    (tmp_path / "a.obj").write_text(OBJ_CASES["quad_fan.obj"])
    shapes = load_obj_shapes(tmp_path / "a.obj", tmp_path)
    assert len(shapes) == 1
    assert shapes[0][2].tolist() == [0, 1, 2, 0, 2, 3, 0, 3, 4]  # fan (v0, v[k-1], v[k])
    (tmp_path / "b.obj").write_text(OBJ_CASES["forms.obj"])
    (_, pos, idx), = load_obj_shapes(tmp_path / "b.obj", tmp_path)
    # every distinct (v, vt, vn) triple is its own vertex: 3 per face here,
    # and the relative -4 -3 -1 means 1 2 4 without texcoord or normal
    assert len(pos) // 3 == 12
    assert idx.tolist()[-3:] == [9, 10, 11]
    (tmp_path / "c.obj").write_text(OBJ_CASES["shapes.obj"])
    sc = Scene()
    assert sc.load("c.obj", base=tmp_path)
    # the reference keeps the last shape's mesh but appends every shape's normals
    assert sc.face_count == 2 and len(sc.face_normals) == 9
    fixed = Scene()
    assert fixed.load("c.obj", base=tmp_path, fix_multi_shape=True)
    assert fixed.face_count == 3 and len(fixed.face_normals) == 9


@pytest.mark.parametrize("name", ["cube.obj", "box.obj", "plane.obj", "cone.obj", "monkey.obj",
                                  "shower.obj"])
def test_reference_scenes(host, name, monkeypatch):
    if not REF_SCENES.is_dir():
        pytest.skip("reference scenes not present")
    monkeypatch.chdir(REF_SCENES.parent)
    py = Scene()
    assert py.load(name)
    ok, fc, normals, verts, idx = cpp_scene(host, name)
    assert ok and fc == py.face_count
    assert np.array_equal(idx, py.indices) and np.array_equal(verts, py.vertices)
    assert np.array_equal(normals.view(np.uint32), py.face_normals.view(np.uint32))
    faces = sum(1 for line in (REF_SCENES / name).read_text().splitlines() if line.startswith("f "))
    assert py.face_count >= faces


# ------------------------------------------------------------ Houdini / files
def test_houdini_writer_python_and_cpp_agree(tmp_path, host):
    rng = np.random.default_rng(3)
    n = 50
    parts = np.zeros(n, dtype=PARTICLE)
    parts["position"][:, :3] = rng.normal(0, 1, (n, 3))
    parts["velocity"][:, :3] = rng.normal(0, 1, (n, 3))
    parts["density"] = rng.uniform(0, 2200, n)
    parts["density"][:6] = [0, 500, 1000, 1500, 2000, -1]
    params = np.zeros(1, dtype=PARAMS)
    params["particles_count"] = n
    params["particle_mass"] = 0.05
    (tmp_path / "py" / "frames").mkdir(parents=True)
    (tmp_path / "cpp" / "frames").mkdir(parents=True)
    HoudiniFileSaver(str(tmp_path / "py") + "/").writeFrameToFile(parts, params[0])
    assert host.clsph_host_write_houdini((str(tmp_path / "cpp") + "/").encode(), parts.ctypes.data,
                                         params.ctypes.data) == 0
    a = (tmp_path / "py" / "frames" / "frame0000001.geo").read_text()
    b = (tmp_path / "cpp" / "frames" / "frame0000001.geo").read_text()
    assert a == b
    assert a.startswith("PGEOMETRY V5\nNPoints 50 NPrims 1\n")
    assert a.rstrip().endswith("beginExtra\nendExtra")


def test_houdini_writers_match_reference_frame(tmp_path, host):
    """Both writers against tests/golden/geo/frame_ref_300.geo, written by the
    reference's own houdini_file_saver.cpp + HoudiniFileDumpHelper.cpp
    (oracle/_ref/ref_geo, tests/golden/make_golden.py): every density branch
    of the colour ramp, coordinates from 1e-7 to 1e3, -0 and exponents."""
    golden = Path(__file__).resolve().parent / "golden" / "geo"
    d = np.load(golden / "frame_ref_300.npz")
    parts, params = d["particles"], d["params"]
    want = (golden / "frame_ref_300.geo").read_bytes()
    (tmp_path / "py" / "frames").mkdir(parents=True)
    (tmp_path / "cpp" / "frames").mkdir(parents=True)
    HoudiniFileSaver(str(tmp_path / "py") + "/").writeFrameToFile(parts, params[0])
    assert host.clsph_host_write_houdini((str(tmp_path / "cpp") + "/").encode(), parts.ctypes.data,
                                         params.ctypes.data) == 0
    assert (tmp_path / "py" / "frames" / "frame0000001.geo").read_bytes() == want
    assert (tmp_path / "cpp" / "frames" / "frame0000001.geo").read_bytes() == want


def test_houdini_writer_parallel_formatting_is_byte_identical(tmp_path, host):
    """A frame large enough for the C++ writer's threaded formatting."""
    rng = np.random.default_rng(4)
    n = 20000
    parts = np.zeros(n, dtype=PARTICLE)
    parts["position"][:, :3] = rng.normal(0, 1, (n, 3))
    parts["velocity"][:, :3] = rng.normal(0, 1, (n, 3))
    parts["density"] = rng.uniform(0, 2200, n)
    params = np.zeros(1, dtype=PARAMS)
    params["particles_count"] = n
    params["particle_mass"] = 0.05
    (tmp_path / "py" / "frames").mkdir(parents=True)
    (tmp_path / "cpp" / "frames").mkdir(parents=True)
    HoudiniFileSaver(str(tmp_path / "py") + "/").writeFrameToFile(parts, params[0])
    assert host.clsph_host_write_houdini((str(tmp_path / "cpp") + "/").encode(), parts.ctypes.data,
                                         params.ctypes.data) == 0
    a = (tmp_path / "py" / "frames" / "frame0000001.geo").read_bytes()
    b = (tmp_path / "cpp" / "frames" / "frame0000001.geo").read_bytes()
    assert a == b


def test_frame_counter_naming(tmp_path):
    (tmp_path / "frames").mkdir()
    sv = HoudiniFileSaver(str(tmp_path) + "/")
    p = np.zeros(1, dtype=PARAMS)[0]
    for _ in range(3):
        sv.writeFrameToFile(np.zeros(0, dtype=PARTICLE), p)
    assert sorted(x.name for x in (tmp_path / "frames").iterdir()) == [
        "frame0000001.geo", "frame0000002.geo", "frame0000003.geo"]


def test_init_lattice_matches_oracle(oracle):
    st = S.settings_from_dicts(S.WATER, S.DEFAULT_SIM)
    a = init_lattice(32000, st.initial_volume)
    b = oracle.init_lattice(32000, np.float32(st.initial_volume))
    assert np.array_equal(a["position"][:, :3], b["position"][:, :3])


def test_last_frame_bin_is_raw_aos(tmp_path):
    from libclsph_gb300.simulation import save_last_frame

    parts = np.zeros(7, dtype=PARTICLE)
    parts["position"][:, 0] = np.arange(7)
    parts["grid_index"] = 5
    save_last_frame(parts, str(tmp_path / "last_frame.bin"))
    raw = (tmp_path / "last_frame.bin").read_bytes()
    assert len(raw) == 7 * 80
    back = np.frombuffer(raw, dtype=PARTICLE)
    assert np.array_equal(back["position"], parts["position"])
    assert np.frombuffer(raw[72:76], np.uint32)[0] == 5  # grid_index at byte 72
