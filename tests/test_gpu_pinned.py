"""GPU tests of the two host-transfer paths of clsph_gpu_upload/download:
pageable records go through the device staging copy, pinned records are read
and written in place by the unpacking and packing kernels. Both must give the
same bytes (sph_simulation.cpp:195-197 and 339-341 move the whole 80-byte
records either way).
"""

import numpy as np
import pytest

from libclsph_gb300 import workloads as W
from libclsph_gb300.gpu import GpuSolver
from libclsph_gb300.layout import PARTICLE

pytestmark = pytest.mark.gpu


def pinned(n: int, offset: int = 0) -> np.ndarray:
    """n particle records in page-locked memory, `offset` bytes into the
    allocation (the array keeps the allocation alive through its base)."""
    import torch

    buf = torch.empty(n * PARTICLE.itemsize + offset, dtype=torch.uint8, pin_memory=True)
    return np.frombuffer(buf.numpy(), dtype=PARTICLE, count=n, offset=offset)


def solver(sc):
    return GpuSolver(sc.params, sc.terms, sc.n, sc.mesh)


@pytest.mark.parametrize("steps", [0, 1, 5])
def test_pinned_and_pageable_transfers_agree(gpu_lib, steps):
    sc = W.dam_break_32k(seed=4)
    with solver(sc) as a, solver(sc) as b:
        a.upload(sc.particles)
        if steps:
            a.step(steps)
        ref = a.download()

        src = pinned(sc.n)
        src[:] = sc.particles
        b.upload(src)
        if steps:
            b.step(steps)
        out = pinned(sc.n)
        out.view(np.uint8)[:] = 0xA5  # every byte must be written
        b.download(out)
        assert out.tobytes() == ref.tobytes()
        assert b.download().tobytes() == ref.tobytes()  # pageable, same handle


def test_pinned_host_loop_matches_pageable_host_loop(gpu_lib):
    """upload -> substep -> download every substep through one buffer, as the
    reference's simulate_single_frame does."""
    sc = W.small_block(12, seed=61, velocity_sigma=0.2)
    with solver(sc) as a, solver(sc) as b:
        pageable = sc.particles.copy()
        host = pinned(sc.n)
        host[:] = sc.particles
        for _ in range(6):
            a.upload(pageable)
            a.step(1)
            a.download(pageable)
            b.upload(host)
            b.step(1)
            b.download(host)
        assert host.tobytes() == pageable.tobytes()


def test_unaligned_pinned_records_take_the_copy_path(gpu_lib):
    sc = W.small_block(8, seed=62, velocity_sigma=0.1)
    with solver(sc) as a, solver(sc) as b:
        a.upload(sc.particles)
        a.step(3)
        ref = a.download()
        src = pinned(sc.n, offset=8)  # 8-byte aligned only: no in-place float4 access
        src[:] = sc.particles
        b.upload(src)
        b.step(3)
        out = pinned(sc.n, offset=4)
        b.download(out)
        assert out.tobytes() == ref.tobytes()
