"""The reference-compatible host layer on the GPU: the Python Simulation mirror
and the C++ sph_simulation (through a drop-in example program) run the same
frames/substeps/callbacks loop as libclsph/sph_simulation.cpp:346-403."""

import json
import os
import subprocess
from pathlib import Path

import numpy as np
import pytest

from libclsph_gb300 import settings as S
from libclsph_gb300.gpu import GpuSolver
from libclsph_gb300.layout import PARTICLE
from libclsph_gb300.simulation import FRAMES_ONLY, Simulation, init_lattice, save_last_frame

pytestmark = pytest.mark.gpu

ROOT = Path(__file__).resolve().parents[1]
CUBE = """o Cube
v -0.5 -1.5 0.5
v -0.5 -1.5 -0.5
v 0.5 -1.5 -0.5
v 0.5 -1.5 0.5
v -0.5 -0.5 0.5
v -0.5 -0.5 -0.5
v 0.5 -0.5 -0.5
v 0.5 -0.5 0.5
f 5 6 1
f 6 7 2
f 7 8 4
f 8 5 1
f 1 2 3
f 8 7 6
f 6 2 1
f 7 3 2
f 3 7 4
f 4 8 1
f 4 1 3
f 5 8 6
"""


@pytest.fixture
def workdir(tmp_path, monkeypatch):
    """A working directory laid out like the reference's run directory."""
    (tmp_path / "scenes").mkdir()
    (tmp_path / "scenes" / "cube.obj").write_text(CUBE)
    (tmp_path / "frames").mkdir()
    sim = dict(S.DEFAULT_SIM, particles_count=2744, constant_acceleration={"x": 0, "y": -9.8, "z": 0})
    (tmp_path / "water.json").write_text(json.dumps(S.WATER) + "\n};\n")
    (tmp_path / "sim.json").write_text(json.dumps(sim) + "\n};\n")
    monkeypatch.chdir(tmp_path)
    return tmp_path


def make_sim():
    s = Simulation()
    s.load_settings("water.json", "sim.json")
    assert s.current_scene.load("cube.obj")
    return s


def test_simulation_matches_engine(gpu_lib, workdir):
    sim = make_sim()
    calls = {"pre": [0, 0], "post": [0, 0]}
    sim.pre_frame = lambda p, prm, full: calls["pre"].__setitem__(int(full), calls["pre"][int(full)] + 1)
    sim.post_frame = lambda p, prm, full: calls["post"].__setitem__(int(full), calls["post"][int(full)] + 1)
    out = sim.simulate(2)
    # 2 frames x 10 substeps (simulation_scale 0.1), as the reference calls them
    assert calls == {"pre": [20, 2], "post": [20, 2]}
    # the same 20 substeps straight through the engine
    p0 = init_lattice(2744, sim.initial_volume)
    with GpuSolver(sim.parameters, sim.precomputed_terms, 2744, sim.current_scene.mesh()) as g:
        g.upload(p0)
        g.step(20)
        ref = g.download()
    assert np.array_equal(out.view(np.uint8), ref.view(np.uint8))
    # the callbacks saw the grid of the last substep
    assert sim.parameters["grid_cell_count"] > 0


def test_callback_changes_reach_the_next_substep(gpu_lib, workdir):
    sim = make_sim()
    state = {"n": 0}

    def stop_everything(p, prm, full):
        if not full:
            state["n"] += 1
            p["velocity"][:] = 0
            p["intermediate_velocity"][:] = 0

    sim.pre_frame = stop_everything
    out = sim.simulate(1)
    # each substep starts from rest, so it moves by at most |g| dt^2 (+ pressure)
    p0 = init_lattice(2744, sim.initial_volume)
    with GpuSolver(sim.parameters, sim.precomputed_terms, 2744, sim.current_scene.mesh()) as g:
        cur = p0
        for _ in range(10):
            cur = cur.copy()
            cur["velocity"][:] = 0
            cur["intermediate_velocity"][:] = 0
            g.upload(cur)
            g.step(1)
            cur = g.download()
    assert state["n"] == 10
    assert np.array_equal(out.view(np.uint8), cur.view(np.uint8))


RAISE = np.float32(0.4995)  # moves the cube's top face to just below the lattice's lowest layer


def raise_mesh(mesh):
    out = dict(mesh, vertices=np.array(mesh["vertices"], dtype=np.float32, copy=True))
    out["vertices"][1::3] += RAISE
    return out


def test_scene_edits_in_callbacks_reach_the_next_substep(gpu_lib, workdir):
    """The reference hands current_scene to its kernels every substep
    (sph_simulation.cpp:296-337), so a callback that moves the mesh in place
    changes the collisions from the next substep on."""
    sim = make_sim()
    calls = {"n": 0}

    def move_mesh(p, prm, full):
        if not full:
            calls["n"] += 1
            if calls["n"] == 4:
                sim.current_scene.vertices[1::3] += RAISE

    sim.pre_frame = move_mesh
    out = sim.simulate(1)
    assert calls["n"] == 10
    # the engine: 3 substeps with the loaded mesh, 7 with the moved one
    p0 = init_lattice(2744, sim.initial_volume)
    m0 = make_sim().current_scene.mesh()
    with GpuSolver(sim.parameters, sim.precomputed_terms, 2744, m0) as g:
        g.upload(p0)
        g.step(3)
        g.set_mesh(raise_mesh(m0))
        g.step(7)
        moved = g.download()
        g.upload(p0)
        g.set_mesh(m0)
        g.step(10)
        still = g.download()
    assert np.array_equal(out.view(np.uint8), moved.view(np.uint8))
    # the moved mesh is hit: the edit changes the outcome
    assert not np.array_equal(moved["position"], still["position"])


def flip_gravity_at(sim, substep, calls):
    def cb(p, prm, full):
        if not full:
            calls["n"] += 1
            if calls["n"] == substep:
                sim.parameters["constant_acceleration"][1] = -sim.parameters["constant_acceleration"][1]
    return cb


def test_parameter_edits_in_callbacks_reach_the_next_substep(gpu_lib, workdir):
    """The reference hands `parameters` to its kernels by value every substep
    (sph_simulation.cpp:282-337), so a callback that edits them (here the
    gravity) changes the next substeps."""
    sim = make_sim()
    calls = {"n": 0}
    sim.pre_frame = flip_gravity_at(sim, 4, calls)
    out = sim.simulate(1)
    assert calls["n"] == 10
    assert sim.parameters["constant_acceleration"][1] > 0
    # the engine: 3 substeps under the loaded gravity, 7 under the flipped one
    base = make_sim()
    p0 = init_lattice(2744, base.initial_volume)
    flipped = base.parameters.copy()
    flipped["constant_acceleration"][1] = -flipped["constant_acceleration"][1]
    with GpuSolver(base.parameters, base.precomputed_terms, 2744, base.current_scene.mesh()) as g:
        g.upload(p0)
        g.step(3)
        g.set_parameters(flipped, base.precomputed_terms)
        g.step(7)
        want = g.download()
    assert np.array_equal(out.view(np.uint8), want.view(np.uint8))
    assert not np.array_equal(out["position"], make_sim().simulate(1)["position"])


def test_particle_count_edit_is_refused(gpu_lib, workdir):
    sim = make_sim()

    def shrink(p, prm, full):
        sim.parameters["particles_count"] = 100

    sim.pre_frame = shrink
    with pytest.raises(RuntimeError, match="particle count"):
        sim.simulate(1)


def test_frames_only_policy_matches_when_callbacks_only_read(gpu_lib, workdir):
    a = make_sim()
    a.pre_frame = lambda p, prm, full: None
    ra = a.simulate(2)
    b = make_sim()
    b.transfers = FRAMES_ONLY
    b.pre_frame = lambda p, prm, full: None
    rb = b.simulate(2)
    assert np.array_equal(ra.view(np.uint8), rb.view(np.uint8))


def test_resume_from_last_frame(gpu_lib, workdir):
    sim = make_sim()
    first = sim.simulate(1)
    save_last_frame(first)
    resumed = make_sim().simulate(1)
    os.remove("last_frame.bin")
    straight = make_sim().simulate(2)
    assert np.array_equal(resumed.view(np.uint8), straight.view(np.uint8))


def test_cpp_dropin_example_matches_python(gpu_lib, workdir):
    exe = workdir / "dropin_example"
    lib_dir = ROOT / "libclsph_gb300" / "_lib"
    r = subprocess.run(["g++", "-std=c++17", "-O1", f"-I{ROOT / 'include' / 'clsph'}",
                        f"-I{ROOT / 'include'}", str(ROOT / "tests" / "cpp" / "dropin_example.cpp"),
                        "-o", str(exe), f"-L{lib_dir}", "-lclsph", "-lclsph_gpu",
                        f"-Wl,-rpath,{lib_dir}"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    run = subprocess.run([str(exe), "water.json", "sim.json", "cube.obj", "2", "./"],
                         capture_output=True, text=True, timeout=300)
    assert run.returncode == 0, run.stdout + run.stderr
    assert "calls pre=22 post=22" in run.stdout
    cpp = np.fromfile("final.bin", dtype=PARTICLE)
    py = make_sim().simulate(2)
    assert np.array_equal(cpp.view(np.uint8), py.view(np.uint8))
    # one Houdini frame per full frame, named like the reference's
    assert sorted(f.name for f in (workdir / "frames").iterdir()) == [
        "frame0000001.geo", "frame0000002.geo"]
    # a scene edited in place by a callback reaches the device, as in Python
    run = subprocess.run([str(exe), "water.json", "sim.json", "cube.obj", "1", "./", "raise_mesh"],
                         capture_output=True, text=True, timeout=300)
    assert run.returncode == 0, run.stdout + run.stderr
    cpp = np.fromfile("final.bin", dtype=PARTICLE)
    sim = make_sim()
    calls = {"n": 0}

    def move_mesh(p, prm, full):
        if not full:
            calls["n"] += 1
            if calls["n"] == 4:
                sim.current_scene.vertices[1::3] += RAISE

    sim.pre_frame = move_mesh
    py = sim.simulate(1)
    assert np.array_equal(cpp.view(np.uint8), py.view(np.uint8))
    # so do parameters edited by a callback
    run = subprocess.run([str(exe), "water.json", "sim.json", "cube.obj", "1", "./", "flip_gravity"],
                         capture_output=True, text=True, timeout=300)
    assert run.returncode == 0, run.stdout + run.stderr
    cpp = np.fromfile("final.bin", dtype=PARTICLE)
    sim = make_sim()
    sim.pre_frame = flip_gravity_at(sim, 4, {"n": 0})
    py = sim.simulate(1)
    assert np.array_equal(cpp.view(np.uint8), py.view(np.uint8))
