"""The C-ABI libraries load on CPU and export every declared symbol; the C++
drop-in headers compile code written against the reference."""

import ctypes
import re
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
GPU_SO = ROOT / "libclsph_gb300" / "_lib" / "libclsph_gpu.so"
HOST_SO = ROOT / "libclsph_gb300" / "_lib" / "libclsph.so"


@pytest.fixture(scope="module", autouse=True)
def built():
    from libclsph_gb300.build import build_gpu, build_host

    build_gpu()
    build_host()


def declared(header: Path, prefix: str):
    text = header.read_text()
    return sorted(set(re.findall(r"\b(" + prefix + r"\w+)\s*\(", text)))


def test_gpu_library_exports_header_symbols():
    names = declared(ROOT / "include" / "clsph_gpu.h", "clsph_gpu_")
    assert len(names) >= 20
    lib = ctypes.CDLL(str(GPU_SO))
    for n in names:
        assert hasattr(lib, n), n
    from libclsph_gb300.gpu import SIGNATURES

    assert sorted(s[0] for s in SIGNATURES) == names


def test_gpu_library_exports_learned_symbols():
    header = ROOT / "include" / "clsph_learned.h"
    names = sorted(set(declared(header, "clsph_mlp_") + declared(header, "clsph_collector_") +
                       declared(header, "clsph_gpu_")) - set(declared(ROOT / "include" / "clsph_gpu.h", "clsph_gpu_")))
    assert len(names) >= 15
    lib = ctypes.CDLL(str(GPU_SO))
    for n in names:
        assert hasattr(lib, n), n
    from libclsph_gb300.learned import BLOB, SIGNATURES

    assert sorted(s[0] for s in SIGNATURES) == names
    lib.clsph_mlp_blob_size.restype = ctypes.c_uint64
    assert lib.clsph_mlp_blob_size() == BLOB == 75268 + 72


def test_learned_flags_match_header():
    text = (ROOT / "include" / "clsph_learned.h").read_text()
    flags = dict((k, int(v)) for k, v in re.findall(r"(CLSPH_LEARNED_\w+)\s*=\s*(\d+)", text))
    from libclsph_gb300 import learned

    assert flags == {"CLSPH_LEARNED_CALIBRATE": learned.CALIBRATE,
                     "CLSPH_LEARNED_NO_CHECK": learned.NO_CHECK}


def test_host_library_exports():
    lib = ctypes.CDLL(str(HOST_SO))
    for n in ("clsph_host_load_settings", "clsph_host_scene_new", "clsph_host_scene_load",
              "clsph_host_scene_sizes", "clsph_host_scene_copy", "clsph_host_scene_free",
              "clsph_host_scene_set_fix_multi_shape",
              "clsph_host_write_houdini", "clsph_host_write_bgeo", "clsph_host_simulate", "clsph_host_last_error"):
        assert hasattr(lib, n), n


def test_create_without_device_fails_cleanly():
    """No GPU here: create reports CLSPH_ERR_NO_DEVICE instead of crashing."""
    import torch

    if torch.cuda.is_available():
        pytest.skip("a device is present")
    from libclsph_gb300.gpu import ClsphError, GpuSolver
    from libclsph_gb300 import workloads as W

    sc = W.small_block(4)
    with pytest.raises(ClsphError) as e:
        GpuSolver(sc.params, sc.terms, sc.n)
    assert e.value.code == 1024


def compile_against_dropin(src: Path, out: Path):
    cxx = shutil.which("g++")
    cmd = [cxx, "-std=c++17", "-O1", f"-I{ROOT / 'include' / 'clsph'}", f"-I{ROOT / 'include'}",
           str(src), "-o", str(out), f"-L{GPU_SO.parent}", "-lclsph", "-lclsph_gpu",
           f"-Wl,-rpath,{GPU_SO.parent}"]
    return subprocess.run(cmd, capture_output=True, text=True)


def test_project_example_compiles(tmp_path):
    r = compile_against_dropin(ROOT / "tests" / "cpp" / "dropin_example.cpp", tmp_path / "ex")
    assert r.returncode == 0, r.stderr


def test_reference_example_compiles_unchanged(tmp_path):
    from oracle import reference_root

    src = reference_root() / "example" / "particles.cpp"
    if not src.exists():
        pytest.skip("reference sources not present")
    r = compile_against_dropin(src, tmp_path / "particles")
    assert r.returncode == 0, r.stderr
