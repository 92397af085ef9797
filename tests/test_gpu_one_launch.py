"""GPU parity of the one-launch culling kernel (cf_fused.cu): light
transform, every sphere-box test, the capped ordered lists, the cluster-order
offsets and the packed output in a single launch.  Every result is compared
bit for bit with the oracle: light counts at each chunk and shape boundary,
every compiled shape with one to 32 clusters per CTA, non-finite lights, the
golden cases, and repeated launches on one workspace (the per-launch epoch
that tags each CTA's published total)."""
import ctypes as C

import numpy as np
import pytest

from gpu_helpers import assert_matches_oracle, run_pipeline
from hellovulkan_gb300 import scenes
from hellovulkan_gb300.camera import ubo_from_bytes

pytestmark = pytest.mark.gpu

ONE_LAUNCH = 2  # CullConfig mode: everything in one launch
SHAPES = [(32, 1024), (16, 2048), (16, 1024)]  # (warps per CTA, most lights)


def one_launch_tuning(clusters, n_lights, per_cta=None, shape=None):
    warps, max_lights = shape or ((32, 1024) if n_lights <= 1024 else (16, 2048))
    if per_cta is None:
        per_cta = max(1, -(-clusters // 152))
    return (per_cta, warps, max_lights, 1, ONE_LAUNCH)


def view_with(n_lights, seed=3, grid=(16, 9, 24), far=1000.0):
    rng = np.random.default_rng(seed)
    lights = scenes.uniform_box_lights(rng, n_lights, [-20, 0, -40], [20, 15, 10], 1.0, 5.0)
    return scenes.custom_view(grid, 1920, 1080, 0.1, far, lights=lights)


def test_small_views_default_to_one_launch(gpu):
    from hellovulkan_gb300.pipelines import PipelineLightCulling, ResourcesClusterForward, ResourcesLight
    for v, want in ((scenes.plain_small(1), ONE_LAUNCH), (view_with(2048), ONE_LAUNCH), (view_with(2049), 0),
                    (scenes.plain_large(2), 1)):
        rl = ResourcesLight(gpu)
        rl.add_lights(v.lights)
        rc = ResourcesClusterForward(gpu)
        rc.create_buffers(*v.grid, v.cap)
        cu = PipelineLightCulling(gpu, rl, rc)
        cu.set_cluster_forward_ubo(v.ubo)
        assert cu.tuning()[4] == want, (v.name, cu.tuning())
        for o in (cu, rc, rl):
            o.close()


@pytest.mark.parametrize("n_lights", [0, 1, 31, 32, 33, 63, 64, 65, 511, 1023, 1024, 1025, 1500, 2047, 2048])
def test_light_counts_at_chunk_and_shape_boundaries(gpu, oracle, n_lights):
    v = view_with(n_lights, seed=n_lights)
    assert_matches_oracle(oracle, v, *run_pipeline(gpu, v))


@pytest.mark.parametrize("shape", SHAPES)
@pytest.mark.parametrize("per_cta", [None, 32])
def test_every_shape_and_cluster_split(gpu, oracle, golden, shape, per_cta):
    """Golden views (dense capping, every cluster capped, non-finite lights,
    an odd grid, one cluster) and a 1920x1080 view, per compiled shape, with
    the fewest clusters per CTA the CTA limit allows and with 32."""
    names = ("cap_dense", "all_capped", "nonfinite_lights", "odd_grid_odd_lights", "grid_1x1x1", "behind_and_rotated")
    views = [scenes.View(ubo_from_bytes(golden[n + "/ubo"]), golden[n + "/lights"], int(golden[n + "/cap"][0]), n)
             for n in names] + [scenes.plain_small(4)]
    for v in views:
        if v.light_count > shape[1]:
            continue
        m = per_cta or max(1, -(-v.clusters // 256))
        assert_matches_oracle(oracle, v, *run_pipeline(gpu, v, one_launch_tuning(v.clusters, v.light_count, m, shape)))


def test_one_cluster_per_cta(gpu, oracle):
    v = view_with(700, seed=5, grid=(8, 8, 4))  # 256 clusters: 256 CTAs of one cluster
    assert_matches_oracle(oracle, v, *run_pipeline(gpu, v, one_launch_tuning(v.clusters, v.light_count, 1)))


def test_too_many_lights_for_the_shape_is_an_error(gpu):
    from hellovulkan_gb300._lib import CfError
    v = view_with(1025)
    with pytest.raises(CfError):
        run_pipeline(gpu, v, one_launch_tuning(v.clusters, v.light_count, 23, (32, 1024)))


def test_repeated_launches_on_one_workspace(gpu, oracle):
    """Frames of changing light sets culled through one pipeline, each read
    back and checked: a CTA that read a total published by an earlier launch
    would shift every offset after it."""
    from hellovulkan_gb300.pipelines import (PipelineAABBGenerator, PipelineLightCulling, ResourcesClusterForward,
                                             ResourcesLight)
    base = scenes.plain_small(6)
    rl = ResourcesLight(gpu)
    rc = ResourcesClusterForward(gpu)
    rc.create_buffers(*base.grid, base.cap)
    gen = PipelineAABBGenerator(gpu, rc)
    gen.set_cluster_forward_ubo(base.ubo)
    gen.fill_command_buffer()
    cu = PipelineLightCulling(gpu, rl, rc)
    cu.set_cluster_forward_ubo(base.ubo)
    aabbs = oracle.generate_aabbs(base.ubo)
    rng = np.random.default_rng(8)
    for frame in range(12):
        n = int(rng.integers(0, 2049))
        lights = scenes.uniform_box_lights(rng, n, [-20, 0, -40], [20, 15, 10], 0.5, 6.0 + frame)
        rl.add_lights(lights)
        for _ in range(1 + frame % 3):  # some frames launch more than once before the read-back
            cu.fill_command_buffer()
        assert cu.tuning()[4] == ONE_LAUNCH
        cells, idx = rc.read_outputs()
        oc, oi, _ = oracle.cull(base.ubo, aabbs, lights, base.cap)
        assert np.array_equal(cells, oc) and np.array_equal(idx, oi), frame
    assert gpu.check_device_error() == 0
    for o in (cu, gen, rc, rl):
        o.close()


def test_one_workspace_across_views_of_different_cta_counts(gpu, oracle):
    """The stateless entry point on one zero-filled workspace, alternating
    views of 151, 105, 152 and 64 CTAs, three rounds."""
    import torch
    from hellovulkan_gb300._lib import check, lib
    L = lib()
    views = [scenes.plain_small(7), view_with(300, seed=9, grid=(7, 5, 3)), view_with(1800, seed=10, grid=(16, 16, 16)),
             view_with(2000, seed=11, grid=(4, 4, 4))]
    sizes = []
    for v in views:
        n = C.c_uint64()
        check(L.cf_cull_workspace_size(C.byref(v.ubo), v.light_count, v.cap, C.byref(n)))
        sizes.append(n.value)
    ws = torch.zeros(max(sizes), dtype=torch.uint8, device="cuda")
    s = torch.cuda.current_stream().cuda_stream
    for rep in range(3):
        for v in views:
            Cn = v.clusters
            aabbs = torch.empty(Cn * 8, dtype=torch.float32, device="cuda")
            d_lights = torch.from_numpy(np.ascontiguousarray(v.lights)).cuda()
            cells = torch.empty(Cn * 2, dtype=torch.int32, device="cuda")
            idx = torch.empty(Cn * v.cap, dtype=torch.int32, device="cuda")
            total = torch.zeros(1, dtype=torch.int32, device="cuda")
            check(L.cf_generate_aabbs(C.byref(v.ubo), aabbs.data_ptr(), s))
            check(L.cf_cull_lights(C.byref(v.ubo), aabbs.data_ptr(), d_lights.data_ptr() if v.light_count else None,
                                   v.light_count, v.cap, cells.data_ptr(), idx.data_ptr(), Cn * v.cap,
                                   total.data_ptr(), ws.data_ptr(), ws.numel(), s))
            torch.cuda.synchronize()
            t_ = int(total.item())
            assert_matches_oracle(oracle, v, aabbs.cpu().numpy().reshape(Cn, 8),
                                  cells.cpu().numpy().view(np.uint32).reshape(Cn, 2),
                                  idx[:t_].cpu().numpy().view(np.uint32).copy())
    err = C.c_uint32()
    check(L.cf_cull_workspace_device_error(ws.data_ptr(), C.byref(err)))
    assert err.value == 0
