"""GPU substep against the golden fixtures: the outputs of the reference's own
kernel sources (compiled as C++ by oracle/_ref and stored under tests/golden/),
for the reference's initial lattice in scenes/cube.obj, a floor contact in
scenes/box.obj, mucus in a corner, coincident particles, a 5-substep drop,
paths that cross mesh edges and corners exactly (ties between faces), and
paths aimed through the faces, edges and vertices of the reference's dense
scenes monkey.obj (968 faces), shower.obj (1,248), labyrinth.obj (606) and
river.obj (332), where the GPU's per-cell face lists must find the same hit
as the reference's scan over every face.

Bar: bit for bit: cell keys, sorted order, cell table and grid parameters,
the state after the substep and the grid index of every particle (the
fixtures come from the reference's sources built with IEEE operations and
no contraction into FMAs, which the engine reproduces).
"""

from pathlib import Path

import numpy as np
import pytest

from libclsph_gb300.gpu import GpuSolver

pytestmark = pytest.mark.gpu

GOLDEN = Path(__file__).resolve().parent / "golden"
CASES = sorted(GOLDEN.glob("*.npz"))


def golden_table(d):
    """The fixture's dense cell table (compact fixtures: from the sorted keys)."""
    if "table" in d:
        return d["table"]
    cells = int(d["params_out"][0]["grid_cell_count"])
    return np.searchsorted(d["sorted"]["grid_index"], np.arange(cells, dtype=np.uint64),
                           side="left").astype(np.uint32)


def rel_err(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    scale = np.abs(b).max() if b.size else 0.0
    return float(np.abs(a - b).max() / scale) if scale > 0 else float(np.abs(a - b).max())


def same_state(out, want):
    """Bit for bit; a mismatch reports the largest relative difference."""
    for f in ("position", "velocity", "intermediate_velocity"):
        a, b = out[f][:, :3], want[f][:, :3]
        assert np.array_equal(a, b), f"{f}: max rel diff {rel_err(a, b):.3g}"
    for f in ("density", "pressure"):
        assert np.array_equal(out[f], want[f]), f"{f}: max rel diff {rel_err(out[f], want[f]):.3g}"
    assert np.array_equal(out["grid_index"], want["grid_index"])


@pytest.mark.parametrize("path", CASES, ids=lambda p: p.stem)
def test_substep_matches_reference_outputs(gpu_lib, path):
    d = np.load(path)
    params, terms, parts = d["params"][0], d["terms"][0], d["particles"]
    mesh = {"vertices": d["vertices"], "indices": d["indices"], "face_normals": d["face_normals"]}
    steps = int(d["steps"][0])
    with GpuSolver(params, terms, len(parts), mesh) as g:
        g.upload(parts)
        g.step(steps)
        assert g.sync() == 0
        if steps == 1:
            keys, perm = g.keys()
            table = g.cell_table()
            prm = g.parameters()
        out = g.download()
    if steps == 1:
        assert np.array_equal(keys, d["sorted"]["grid_index"])
        assert np.array_equal(perm, d["perm"])
        assert np.array_equal(table, golden_table(d))
        want_p = d["params_out"][0]
        for f in ("grid_size_x", "grid_size_y", "grid_size_z", "grid_cell_count"):
            assert prm[f] == want_p[f], f
        assert np.array_equal(prm["min_point"][:3], want_p["min_point"][:3])
        assert np.array_equal(prm["max_point"][:3], want_p["max_point"][:3])
    same_state(out, d["final"])
