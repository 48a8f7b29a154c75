"""GPU tests of the engine's bounded device waits: failure detection without a
GPU fault.

Each test makes one wait run out on purpose through clsph_gpu_set_wait_limits
and checks that the failure reaches the host as an error status while the
context stays usable:

* the radix sort's decoupled look-back: tile 0 of every pass withholds its
  digit counts (a word that nothing sets) and the look-back of the tile after
  it gives up after 64 spins; clsph_gpu_sync must report CLSPH_ERR_CUDA, and
  with the default bounds restored the same handle then runs a substep equal
  to the oracle bit for bit;
* the mbarrier waits of the learned stepper's tcgen05 MLP: a bound of 0 polls
  makes the first wait of the tile loop give up at once; clsph_gpu_step_learned
  must fail with CLSPH_ERR_CUDA in the checked and the unchecked mode (the
  kernel's teardown still waits, with the full bound, for the MMAs it has in
  flight before it frees tensor memory), and with the default bound restored
  the same handle steps exactly like a fresh one.

What keeps every access in bounds after a stall is stated beside the kernels:
destinations past the end are skipped, unwritten sort slots keep earlier
in-range values, the gather clamps its source slot, and the learned advection
reads correction rows that start zeroed and are clamped to the network's
output range.
"""

import numpy as np
import pytest

from libclsph_gb300 import learned as Lm
from libclsph_gb300 import workloads as W
from libclsph_gb300.gpu import ClsphError, GpuSolver

pytestmark = pytest.mark.gpu

CLSPH_ERR_CUDA = 512


def test_radix_lookback_wait_runs_out_and_reports(gpu_lib, oracle):
    sc = W.small_block(24, seed=61, velocity_sigma=0.05)  # 13,824 keys: 7 radix tiles per pass
    ref = oracle.step(sc.params, sc.terms, sc.particles, sc.mesh)
    with GpuSolver(sc.params, sc.terms, sc.n, sc.mesh) as g:
        g.set_wait_limits(radix_lookback_spins=64, radix_withheld_tile=0)
        g.upload(sc.particles)
        g.step(1)
        with pytest.raises(ClsphError) as err:
            g.sync()
        assert err.value.code == CLSPH_ERR_CUDA
        assert "look-back wait ran out" in str(err.value)
        assert g.sync() == 0  # the status word was cleared with the report
        g.set_wait_limits()
        g.upload(sc.particles)
        g.step(1)
        assert g.sync() == 0
        keys, perm = g.keys()
        out = g.download()
    assert np.array_equal(perm, ref.perm)
    assert np.array_equal(keys, ref.sorted["grid_index"])
    for field in ("position", "velocity", "intermediate_velocity"):
        assert np.array_equal(out[field][:, :3], ref.final[field][:, :3]), field


def _small_net():
    rng = np.random.default_rng(63)
    blob = np.zeros(Lm.BLOB, dtype=np.float32)
    blob[Lm.OFF_W1:Lm.OFF_B1] = rng.normal(0, 0.02, 32 * 256)
    blob[Lm.OFF_W2:Lm.OFF_B2] = rng.normal(0, 0.02, 256 * 256)
    blob[Lm.OFF_W3:Lm.OFF_B3] = rng.normal(0, 0.02, 256 * 4)
    blob[Lm.OFF_XSIGMA:Lm.OFF_YMU] = 1
    blob[Lm.OFF_YSIGMA:] = 0.01
    return Lm.Mlp(blob=blob)


def test_mlp_wait_runs_out_and_reports(gpu_lib):
    sc = W.small_block(16, seed=62, velocity_sigma=0.05)
    net = _small_net()
    try:
        with GpuSolver(sc.params, sc.terms, sc.n, sc.mesh) as g:
            g.upload(sc.particles)
            g.set_wait_limits(mlp_wait_polls=0)
            for check in (True, False):
                with pytest.raises(ClsphError) as err:
                    Lm.step_learned(g, net, 1, dt_mult=4, threshold=1e30, check=check)
                assert err.value.code == CLSPH_ERR_CUDA
                assert "tensor-core wait" in str(err.value) and "timed out" in str(err.value)
                g.upload(sc.particles)
            g.set_wait_limits()
            Lm.step_learned(g, net, 2, dt_mult=4, threshold=1e30, check=False)
            assert g.sync() == 0
            after_failure = g.download()
        with GpuSolver(sc.params, sc.terms, sc.n, sc.mesh) as fresh:
            fresh.upload(sc.particles)
            Lm.step_learned(fresh, net, 2, dt_mult=4, threshold=1e30, check=False)
            assert fresh.sync() == 0
            want = fresh.download()
    finally:
        net.close()
    for field in ("position", "velocity", "intermediate_velocity"):
        assert np.array_equal(after_failure[field][:, :3], want[field][:, :3]), field
