"""Build recipes for the native parts (no cmake; nvcc + g++ in-tree).

  libclsph_gb300/_lib/libclsph_gpu.so  CUDA substep engine + C ABI (sm_103a only)
  libclsph_gb300/_lib/libclsph.so      C++ host layer: sph_simulation, scene,
                                       houdini_file_saver, JSON settings
                                       (links libclsph_gpu.so)

Outputs are git-ignored and rebuilt on every machine (the GPU host is aarch64).
"""

from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
LIB_DIR = PKG / "_lib"
CSRC = PKG / "csrc"
HOST = PKG / "host"
INCLUDE = ROOT / "include"

GPU_SO = LIB_DIR / "libclsph_gpu.so"
HOST_SO = LIB_DIR / "libclsph.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(cand).exists():
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libclsph_gb300")
    return cand


def _run(cmd: list[str]) -> None:
    proc = subprocess.run(cmd, capture_output=True, text=True)
    if proc.returncode != 0:
        sys.stderr.write(proc.stdout + proc.stderr)
        raise RuntimeError(f"build step failed: {' '.join(cmd[:3])} ...")


GPU_SOURCES = ["clsph_gpu.cu", "clsph_sort_noalloc.cu", "clsph_learned.cu"]
OBJ_DIR = LIB_DIR / "obj"


def gpu_compile_cmd(src: str, extra: list[str] | None = None) -> list[str]:
    """nvcc command compiling one translation unit of the engine to an object."""
    return [
        _nvcc(), *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-c",
        f"-I{INCLUDE}", f"-I{CSRC}", *(extra or []), "-o", str(OBJ_DIR / (Path(src).stem + ".o")),
        str(CSRC / src),
    ]


def gpu_link_cmd() -> list[str]:
    return [_nvcc(), *ARCH, "-shared", "-o", str(GPU_SO),
            *[str(OBJ_DIR / (Path(src).stem + ".o")) for src in GPU_SOURCES]]


def host_cmd() -> list[str]:
    srcs = sorted(str(p) for p in HOST.glob("*.cpp"))
    cuda_lib = Path(_nvcc()).resolve().parent.parent / "lib64"
    return [
        os.environ.get("CXX", "g++"), "-std=c++17", "-O2", "-fPIC", "-shared", "-pthread",
        "-ffp-contract=off", f"-I{INCLUDE}", f"-I{INCLUDE / 'clsph'}", *srcs, "-o", str(HOST_SO),
        f"-L{LIB_DIR}", "-lclsph_gpu", "-Wl,-rpath,$ORIGIN", f"-L{cuda_lib}",
    ]


def _stale(out: Path, deps: list[Path]) -> bool:
    if not out.exists():
        return True
    t = out.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build_gpu(force: bool = False) -> Path:
    deps = list(CSRC.glob("*")) + list(INCLUDE.glob("*.h"))
    if force or _stale(GPU_SO, deps):
        OBJ_DIR.mkdir(parents=True, exist_ok=True)
        with ThreadPoolExecutor(max_workers=len(GPU_SOURCES)) as ex:
            for f in [ex.submit(_run, gpu_compile_cmd(src)) for src in GPU_SOURCES]:
                f.result()
        _run(gpu_link_cmd())
    return GPU_SO


def build_host(force: bool = False) -> Path | None:
    srcs = list(HOST.glob("*.cpp"))
    if not srcs:
        return None
    deps = srcs + list(HOST.glob("*.h")) + list(INCLUDE.rglob("*.h*")) + [GPU_SO]
    if force or _stale(HOST_SO, deps):
        LIB_DIR.mkdir(exist_ok=True)
        _run(host_cmd())
    return HOST_SO


def build_all(force: bool = False, with_oracle: bool = False) -> None:
    """Compiles every native part of the library; the GPU engine first (the
    host layer links it). with_oracle also builds the CPU checkers under
    oracle/ (test infrastructure, never part of the library)."""
    jobs = []
    with ThreadPoolExecutor(max_workers=3) as ex:
        gpu = ex.submit(build_gpu, force)
        if with_oracle:
            jobs.append(ex.submit(_build_oracles))
        gpu.result()
        host = ex.submit(build_host, force)
        host.result()
        for j in jobs:
            j.result()


def _build_oracles() -> None:
    """oracle/liboracle.so, and oracle/_ref where the reference sources are
    present (the Makefile decides; CLSPH_REFERENCE_ROOT points elsewhere)."""
    oracle_dir = ROOT / "oracle"
    if not (oracle_dir / "Makefile").exists():
        return
    _run(["make", "-s", "-C", str(oracle_dir), "liboracle.so"])
    _run(["make", "-s", "-C", str(oracle_dir), "ref-if-present"])


if __name__ == "__main__":
    build_all(force="--force" in sys.argv)
    print("built:", GPU_SO, HOST_SO)
