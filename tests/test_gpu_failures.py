"""Failure paths on the GPU, made without faulting, trapping or hanging it.

* A bounded in-kernel wait made to run out: a test hook
  (include/cfcull_testing.h) makes one CTA withhold a part — the one-launch
  kernel's CTA 0 its hit total, the brute-force kernel's CTA 0 producer its
  first light tile — with the wait limit shortened to 2 ms.  The other
  threads give up, the launch reports CF_ERROR_DEVICE_TIMEOUT through the
  context's device error word, the word clears when read, and the next call
  on the same context is bit-exact against the oracle.
* Device allocations made to fail on the host: each constructor reports
  CF_ERROR_OUT_OF_MEMORY, leaves nothing half-built, and works once the
  injection is off.

The reference's counterpart is VK_CHECK, which logs and carries on
(HelloVulkan/Header/Vulkan/VulkanCheck.h:17-19).
"""
import ctypes as C

import numpy as np
import pytest

from gpu_helpers import assert_matches_oracle, run_pipeline
from hellovulkan_gb300 import scenes

pytestmark = pytest.mark.gpu

LIMIT_NS = 2_000_000          # 2 ms instead of 2 s
STALL_ONE_LAUNCH = 1          # CF_TESTING_STALL_ONE_LAUNCH
STALL_BRUTE_FORCE = 2         # CF_TESTING_STALL_BRUTE_FORCE
ERR_FULL_WAIT, ERR_LOOKBACK = 1, 4  # device error bits: a consumer's tile wait, a one-launch CTA's wait
CF_ERROR_OUT_OF_MEMORY, CF_ERROR_DEVICE_TIMEOUT = 2, 6


@pytest.fixture
def hooks(cflib):
    yield cflib
    cflib.cf_testing_inject_stall(0)
    cflib.cf_testing_set_wait_limit_ns(0)
    cflib.cf_testing_fail_allocation_after(-1)


def cull_with_stall(gpu, lib, view, tuning, mode):
    """One culling call through the pipelines with `mode` injected; returns
    (status of cf_context_check_device_error, the device error word)."""
    from hellovulkan_gb300._lib import check
    from hellovulkan_gb300.pipelines import (PipelineAABBGenerator, PipelineLightCulling, ResourcesClusterForward,
                                             ResourcesLight)
    rl = ResourcesLight(gpu)
    rl.add_lights(view.lights)
    rc = ResourcesClusterForward(gpu)
    rc.create_buffers(*view.grid, view.cap)
    gen = PipelineAABBGenerator(gpu, rc)
    gen.set_cluster_forward_ubo(view.ubo)
    gen.fill_command_buffer()
    cu = PipelineLightCulling(gpu, rl, rc)
    if tuning:
        cu.set_tuning(*tuning)
    cu.set_cluster_forward_ubo(view.ubo)
    check(lib.cf_testing_set_wait_limit_ns(LIMIT_NS))
    check(lib.cf_testing_inject_stall(mode))
    try:
        cu.fill_command_buffer()
        word = C.c_uint32()
        status = lib.cf_context_check_device_error(gpu.handle, C.byref(word))
    finally:
        lib.cf_testing_inject_stall(0)
        lib.cf_testing_set_wait_limit_ns(0)
        for o in (cu, gen, rc, rl):
            o.close()
    return status, int(word.value)


def test_one_launch_wait_runs_out_and_the_context_recovers(gpu, hooks, oracle):
    v = scenes.plain_small(1)  # culled by the one-launch kernel
    status, word = cull_with_stall(gpu, hooks, v, None, STALL_ONE_LAUNCH)
    assert status == CF_ERROR_DEVICE_TIMEOUT and word & ERR_LOOKBACK, (status, word)
    assert gpu.check_device_error() == 0  # the word was cleared when read
    assert_matches_oracle(oracle, v, *run_pipeline(gpu, v))


@pytest.mark.parametrize("n_lights", [1000, 4000])  # 2 light tiles (all in flight at once), 8 tiles (4 stages)
def test_brute_force_tile_wait_runs_out_and_the_context_recovers(gpu, hooks, oracle, n_lights):
    rng = np.random.default_rng(n_lights)
    v = scenes.custom_view((16, 9, 24), 1920, 1080, 0.1, 300.0,
                           lights=scenes.uniform_box_lights(rng, n_lights, [-20, -10, -60], [20, 10, -1], 1.0, 6.0))
    tuning = (1, 8, 512, 4, 0)  # the brute-force kernel: a producer warp streams tiles to 8 consumer warps
    status, word = cull_with_stall(gpu, hooks, v, tuning, STALL_BRUTE_FORCE)
    assert status == CF_ERROR_DEVICE_TIMEOUT and word & ERR_FULL_WAIT, (status, word)
    assert gpu.check_device_error() == 0
    assert_matches_oracle(oracle, v, *run_pipeline(gpu, v, tuning))


def test_injections_are_validated(hooks):
    assert hooks.cf_testing_inject_stall(0x80) == 1  # CF_ERROR_INVALID_ARGUMENT


def test_failed_allocations_are_reported_and_leave_nothing_half_built(gpu, hooks, oracle):
    from hellovulkan_gb300._lib import CfError
    from hellovulkan_gb300.batch import Batch
    from hellovulkan_gb300.pipelines import Context, ResourcesClusterForward
    from hellovulkan_gb300.server import Server
    v = scenes.plain_small(2)
    for n in range(4):  # each of the four buffers of ResourcesClusterForward::CreateBuffers in turn
        rc = ResourcesClusterForward(gpu)
        hooks.cf_testing_fail_allocation_after(n)
        with pytest.raises(CfError) as e:
            rc.create_buffers(*v.grid, v.cap)
        assert e.value.status == CF_ERROR_OUT_OF_MEMORY
        hooks.cf_testing_fail_allocation_after(-1)
        rc.create_buffers(*v.grid, v.cap)  # the same object works once allocations succeed
        rc.close()
    for make in (lambda: Context(0), lambda: Batch(gpu), lambda: Server(gpu, budget_bytes=64 << 20, streams=1)):
        hooks.cf_testing_fail_allocation_after(0)
        with pytest.raises(CfError) as e:
            make()
        assert e.value.status == CF_ERROR_OUT_OF_MEMORY
        hooks.cf_testing_fail_allocation_after(-1)
        make().close()
    hooks.cf_testing_fail_allocation_after(0)  # a whole culling run: its first allocation fails
    with pytest.raises(CfError):
        run_pipeline(gpu, v)
    hooks.cf_testing_fail_allocation_after(-1)
    assert_matches_oracle(oracle, v, *run_pipeline(gpu, v))
