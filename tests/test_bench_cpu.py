"""bench.py on a machine without a GPU: the reference arm (the oracle on the
host cores) prints its one JSON line with the keys of the bench contract, and
the GPU arm stops with an error instead of falling back to the CPU."""

import json
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def run_bench(*args):
    return subprocess.run([sys.executable, str(ROOT / "bench.py"), *args], capture_output=True,
                          text=True, cwd=ROOT, timeout=900)


def test_reference_arm_line():
    r = run_bench("--impl", "reference", "--steps", "1", "--warmup", "0", "--workload",
                  "dam_break_32k")
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference"
    assert d["metric"] == d["unit"] == "particle-steps/s"
    assert d["value"] > 0 and d["higher_is_better"] is True
    assert d["steps"] == 1 and d["warmup"] >= 3  # at least 3 warm-up steps, whatever is asked
    assert d["config"]["workload"] == "dam_break_32768"
    # the full workload, with the GPU arm's config object
    assert d["config"]["n_particles"] == 32768
    sys.path.insert(0, str(ROOT))
    import argparse

    import bench
    from libclsph_gb300 import workloads as W

    assert d["config"] == bench.workload_config(W.dam_break_32k(), argparse.Namespace(no_flush=False))
    assert "full workload" in d["cpu_baseline"]["sample"]
    cb = d["cpu_baseline"]
    assert cb["kind"] == "port" and cb["value"] == d["value"] and cb["cores"] >= 1
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}


def test_gpu_arm_fails_without_a_device():
    import torch

    if torch.cuda.is_available():
        pytest.skip("a device is present")
    r = run_bench("--steps", "1", "--warmup", "3", "--workload", "dam_break_32k")
    assert r.returncode != 0
    assert not [ln for ln in r.stdout.splitlines() if ln.startswith("{")]


def test_reference_arm_under_torchrun_prints_one_line():
    """Two ranks as the scaling run launches them: rank 0 times the oracle and
    prints the line, rank 1 exits 0 without work (gloo: no device needed)."""
    import socket

    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    r = subprocess.run([sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
                        "--master-addr", "127.0.0.1", "--master-port", str(port), str(ROOT / "bench.py"),
                        "--impl", "reference", "--gpus", "2", "--steps", "1", "--warmup", "0",
                        "--workload", "dam_break_32k"],
                       capture_output=True, text=True, cwd=ROOT, timeout=900)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["value"] > 0
