"""Host code under AddressSanitizer + UndefinedBehaviorSanitizer.

compute-sanitizer is not available for the device code, so the host side is
checked here instead: the CPU oracle (several substeps with every optional
output, plus the FP64 fields) and the host layer's parsers and writers (JSON
settings including malformed files, OBJ scenes including every index form and
broken files, .geo and .bgeo frames). A sanitizer report makes the program exit
non-zero; the oracle's result must also equal the regular build's bit for bit.
"""

import json
import os
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

from libclsph_gb300 import settings as S
from libclsph_gb300 import workloads as W

ROOT = Path(__file__).resolve().parents[1]
LIB = ROOT / "libclsph_gb300" / "_lib"
SAN = ["-fsanitize=address,undefined", "-fno-sanitize-recover=all", "-fno-omit-frame-pointer",
       "-g", "-O1"]
ENV = dict(os.environ, ASAN_OPTIONS="detect_leaks=1:protect_shadow_gap=0:abort_on_error=0",
           UBSAN_OPTIONS="print_stacktrace=1", OMP_NUM_THREADS="2")


@pytest.fixture(scope="module")
def cxx(tmp_path_factory):
    gxx = shutil.which("g++")
    if not gxx:
        pytest.skip("no g++")
    probe = tmp_path_factory.mktemp("probe")
    (probe / "t.cpp").write_text("int main() { return 0; }\n")
    r = subprocess.run([gxx, *SAN, str(probe / "t.cpp"), "-o", str(probe / "t")],
                       capture_output=True, text=True)
    if r.returncode != 0:
        pytest.skip("sanitizer runtimes not installed")
    r = subprocess.run([str(probe / "t")], capture_output=True, text=True, env=ENV)
    if r.returncode != 0:
        pytest.skip("sanitized programs cannot run here: " + r.stderr[-200:])
    return gxx


def run_checked(cmd, **kw):
    r = subprocess.run(cmd, capture_output=True, text=True, env=ENV, timeout=600, **kw)
    report = "ERROR: AddressSanitizer" in r.stderr or "runtime error:" in r.stderr or \
        "ERROR: LeakSanitizer" in r.stderr
    assert r.returncode == 0 and not report, r.stdout[-2000:] + r.stderr[-4000:]
    return r


def test_oracle_under_sanitizers(cxx, tmp_path):
    exe = tmp_path / "oracle_san"
    r = subprocess.run([cxx, "-std=c++17", *SAN, "-ffp-contract=off", "-fno-fast-math", "-fopenmp",
                        f"-I{ROOT / 'oracle'}", str(ROOT / "oracle" / "clsph_oracle.cpp"),
                        str(ROOT / "tests" / "cpp" / "oracle_sanitize.cpp"), "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    # A block with random velocities that reaches the walls within a few substeps.
    sc = W.small_block(9, seed=31, velocity_sigma=2.0, offset=(0.02, 0.02, 0.6))
    d = tmp_path / "in"
    d.mkdir()
    np.array(sc.params).tofile(d / "params.bin")
    np.array(sc.terms).tofile(d / "terms.bin")
    sc.particles.tofile(d / "particles.bin")
    sc.mesh["face_normals"].tofile(d / "normals.bin")
    sc.mesh["vertices"].tofile(d / "vertices.bin")
    sc.mesh["indices"].tofile(d / "indices.bin")
    steps = 10
    run_checked([str(exe), str(d), str(steps)])
    got = (d / "out.bin").read_bytes()

    from oracle import Oracle

    want = Oracle().run(sc.params, sc.terms, sc.particles, steps, mesh=sc.mesh, threads=2)
    # every field of the 80-byte records; bytes 76-79 are the struct's tail
    # padding, which neither program defines
    a = np.frombuffer(got, np.uint8).reshape(-1, 80)[:, :76]
    b = want.view(np.uint8).reshape(-1, 80)[:, :76]
    assert np.array_equal(a, b)


def test_host_layer_under_sanitizers(cxx, tmp_path):
    from libclsph_gb300.build import build_gpu

    build_gpu()
    host = ROOT / "libclsph_gb300" / "host"
    srcs = [host / f for f in ("json_reader.cpp", "scene.cpp", "houdini_file_saver.cpp",
                               "sph_simulation.cpp")]
    exe = tmp_path / "host_san"
    r = subprocess.run([cxx, "-std=c++17", *SAN, "-pthread", f"-I{ROOT / 'include' / 'clsph'}",
                        f"-I{ROOT / 'include'}", f"-I{host}", *map(str, srcs),
                        str(ROOT / "tests" / "cpp" / "host_sanitize.cpp"), "-o", str(exe),
                        f"-L{LIB}", "-lclsph_gpu", f"-Wl,-rpath,{LIB}"],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr

    from test_host_layer import OBJ_CASES

    scenes = tmp_path / "scenes"
    scenes.mkdir()
    for name, text in OBJ_CASES.items():
        (scenes / name).write_text(text)
    (scenes / "truncated.obj").write_text("v 0 0\nv 1 0 0\nf 1 2\nf 1 2 9\n")
    (scenes / "empty.obj").write_text("")
    names = sorted(OBJ_CASES) + ["truncated.obj", "empty.obj", "absent.obj"]
    (tmp_path / "frames").mkdir()

    def props(fluid, sim, tag, trailer=";\n"):
        f = tmp_path / f"fluid_{tag}.json"
        s = tmp_path / f"sim_{tag}.json"
        f.write_text(json.dumps(fluid, indent=4) + trailer)
        s.write_text(json.dumps(sim, indent=4) + trailer)
        return str(f), str(s)

    cases = [props(S.WATER, S.DEFAULT_SIM, "ok"),
             props(dict(S.WATER, restitution=1.5), S.DEFAULT_SIM, "restitution"),
             props({k: v for k, v in S.WATER.items() if k != "k"}, S.DEFAULT_SIM, "missing")]
    broken = tmp_path / "broken.json"
    broken.write_text('{"fluid_density": 1000, "k": [1, 2,')
    cases.append((str(broken), cases[0][1]))
    for i, (f, s) in enumerate(cases):
        out = run_checked([str(exe), f, s, str(tmp_path) + "/", *(names if i == 0 else [])],
                          cwd=tmp_path)
        if i == 0:
            assert "settings h=" in out.stdout
            assert "scene quad_fan.obj ok=1" in out.stdout
            assert "scene absent.obj ok=0" in out.stdout
        else:
            assert "settings error" in out.stdout
    frames = sorted(p.name for p in (tmp_path / "frames").iterdir())
    assert frames == ["frame0000001.bgeo", "frame0000001.geo", "frame0000002.bgeo",
                      "frame0000002.geo"]
