"""clsph_gpu_sort_keys_noalloc: the stable sort without any device allocation.

It serves callers that may not call cudaMalloc themselves (an application or
framework that owns every device allocation, or a real-time loop that must
not allocate after start-up). The caller supplies the input keys and both
outputs in device memory; the scratch space is a fixed file-scope device
array of the library (1,048,576 keys at most).

Checked here against the substep's own sort as the regular entry points
expose it (clsph_gpu_step_until(CLSPH_STAGE_SORT) + clsph_gpu_read_keys), on
two calls in a row with different inputs. Integer outputs: bit-exact.
This file sorts last in collection order (test_zz_*) and also passes alone.
"""

import ctypes

import numpy as np
import pytest

from libclsph_gb300 import workloads as W
from libclsph_gb300.gpu import STAGE_SORT, GpuSolver

pytestmark = pytest.mark.gpu

MAX_KEYS = 1 << 20


def substep_sort(scene):
    """Unsorted keys of the scene's first substep and the engine's own
    (sorted keys, permutation) for them."""
    with GpuSolver(scene.params, scene.terms, scene.n, scene.mesh) as g:
        g.upload(scene.particles)
        g.step_until(STAGE_SORT)
        keys, perm = g.keys()
    unsorted = np.empty_like(keys)
    unsorted[perm] = keys
    return unsorted, keys, perm


def noalloc_sort(lib, keys_host):
    import torch

    n = len(keys_host)
    dev_in = torch.from_numpy(keys_host.view(np.int32)).cuda()
    dev_keys = torch.full((max(n, 1),), -1, dtype=torch.int32, device="cuda")
    dev_perm = torch.full((max(n, 1),), -1, dtype=torch.int32, device="cuda")
    stream = torch.cuda.current_stream()
    rc = lib.clsph_gpu_sort_keys_noalloc(dev_in.data_ptr(), dev_keys.data_ptr(),
                                         dev_perm.data_ptr(), n, stream.cuda_stream)
    assert rc == 0, lib.clsph_gpu_last_error()
    stream.synchronize()
    return (dev_keys.cpu().numpy().view(np.uint32)[:n].copy(),
            dev_perm.cpu().numpy().view(np.uint32)[:n].copy())


def test_noalloc_sort_matches_substep_sort_twice(gpu_lib):
    first = W.small_block(16, seed=21, velocity_sigma=0.1)  # 4,096 keys: one tile, 2 radix passes
    second = W.dam_break_1m(seed=22)                         # 1,048,576 keys (the maximum): 3 passes
    for scene in (first, second):
        unsorted, keys, perm = substep_sort(scene)
        got_keys, got_perm = noalloc_sort(gpu_lib, unsorted)
        assert np.array_equal(got_keys, keys)
        assert np.array_equal(got_perm, perm)


def test_noalloc_sort_at_its_maximum(gpu_lib):
    rng = np.random.default_rng(23)
    keys = rng.integers(0, 1 << 30, MAX_KEYS, dtype=np.uint32)
    keys[::7] = keys[3]  # many equal keys: stability matters
    got_keys, got_perm = noalloc_sort(gpu_lib, keys)
    want = np.argsort(keys, kind="stable").astype(np.uint32)
    assert np.array_equal(got_perm, want)
    assert np.array_equal(got_keys, keys[want])


def test_noalloc_sort_allocates_no_device_memory(gpu_lib):
    """Free device memory is the same before and after two calls (the first
    call, which loads the library's device code and its static array, comes
    before the measurement; every buffer is allocated up front)."""
    import torch

    rng = np.random.default_rng(24)
    n = MAX_KEYS
    keys = rng.integers(0, 1 << 24, n, dtype=np.uint32)
    dev_in = torch.from_numpy(keys.view(np.int32)).cuda()
    dev_keys = torch.empty(n, dtype=torch.int32, device="cuda")
    dev_perm = torch.empty(n, dtype=torch.int32, device="cuda")
    stream = torch.cuda.current_stream()

    def call():
        rc = gpu_lib.clsph_gpu_sort_keys_noalloc(dev_in.data_ptr(), dev_keys.data_ptr(),
                                                 dev_perm.data_ptr(), n, stream.cuda_stream)
        assert rc == 0, gpu_lib.clsph_gpu_last_error()

    call()
    torch.cuda.synchronize()
    free_before, _ = torch.cuda.mem_get_info()
    call()
    call()
    torch.cuda.synchronize()
    free_after, _ = torch.cuda.mem_get_info()
    assert free_after == free_before
    want = np.argsort(keys, kind="stable").astype(np.uint32)
    assert np.array_equal(dev_perm.cpu().numpy().view(np.uint32), want)


def test_noalloc_sort_rejects_oversize(gpu_lib):
    rc = gpu_lib.clsph_gpu_sort_keys_noalloc(ctypes.c_void_p(16), ctypes.c_void_p(16),
                                             ctypes.c_void_p(16), MAX_KEYS + 1, None)
    assert rc == 4096  # CLSPH_ERR_TOO_LARGE, before any GPU work
    assert b"exceeds the maximum" in gpu_lib.clsph_gpu_last_error()
