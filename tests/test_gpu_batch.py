"""GPU parity of the batched path: every view of a batch against the oracle,
bit for bit, through CUDA-graph replays, in-place light updates, new view
matrices and autotuned configurations."""
import numpy as np
import pytest

from gpu_helpers import assert_matches_oracle, bits
from hellovulkan_gb300 import scenes
from hellovulkan_gb300.camera import look_at_rh, ubo_from_bytes

pytestmark = pytest.mark.gpu


def mixed_views():
    rng = np.random.default_rng(21)
    vs = []
    for _ in range(10):  # the benchmark mix with the light sets cut to keep the oracle quick
        v = scenes.batch_view(rng)
        vs.append(scenes.View(v.ubo, v.lights[: min(v.light_count, 6000)], v.cap, v.name))
    vs.append(scenes.plain_small(1))
    vs.append(scenes.custom_view((16, 9, 24), 1920, 1080, 0.1, 1000.0))  # no lights
    vs.append(scenes.custom_view((1, 1, 1), 640, 480, 0.5, 50.0,
                                 lights=scenes.uniform_box_lights(rng, 37, [-10, -10, -60], [10, 10, 5])))
    L = scenes.uniform_box_lights(rng, 300, [-20, -10, -60], [20, 10, 0], 1.0, 8.0)
    L[5, 0] = np.nan
    L[17, 1] = np.inf
    L[90, 8] = np.inf
    vs.append(scenes.custom_view((16, 9, 24), 1920, 1080, 0.1, 100.0, lights=L))
    vs.append(scenes.custom_view((8, 8, 16), 1024, 1024, 0.1, 200.0,
                                 lights=scenes.uniform_box_lights(rng, 1000, [-15, -15, -40], [15, 15, -1], 3.0, 12.0)))
    return vs


def check_all(oracle, bufs):
    for i, v in enumerate(bufs.views):
        assert_matches_oracle(oracle, v, *bufs.read(i))


def test_batch_matches_oracle_with_graph_replays(gpu, oracle):
    import torch
    from hellovulkan_gb300.batch import Batch, BatchBuffers
    views = mixed_views()
    bufs = BatchBuffers(views)
    b = Batch(gpu)
    b.set_views(bufs.batch_views())
    s = torch.cuda.Stream()
    b.generate_aabbs(s)
    b.cull(s)  # captures the graph
    check_all(oracle, bufs)
    # move every light of three views in place and replay the same graph
    rng = np.random.default_rng(5)
    for i in (0, 3, 10):
        L = views[i].lights.copy()
        L[:, :3] += rng.normal(0, 0.5, size=(L.shape[0], 3)).astype(np.float32)
        views[i].lights = L
        bufs.set_lights(i, L)
    torch.cuda.synchronize()
    b.cull(s)
    b.cull(s)
    check_all(oracle, bufs)
    assert gpu.check_device_error() == 0
    info = b.info()
    assert info["views"] == len(views) and info["buckets"] >= 2


def test_batch_persistent_grid_counts_large_shared_memory_configs(gpu):
    """A configuration above 48 KB of shared memory must size its persistent
    grid from the real occupancy before its first launch, not from one CTA per SM."""
    import torch
    from hellovulkan_gb300.batch import Batch, BatchBuffers
    views = scenes.batch_mix(3, 64)  # enough work items that no bucket is capped by its item count
    bufs = BatchBuffers(views)
    b = Batch(gpu)
    keys = sorted({v.grid[0] * v.grid[1] for v in views})
    for xy in keys:
        b.set_tuning(xy, 4, 8, 1024, 2)  # 8 warps, 1024-light stages x2: > 48 KB
    b.set_views(bufs.batch_views())
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    buckets = b.info()["bucket_configs"]
    assert all(bc["config"] == [4, 8, 1024, 2] for bc in buckets)
    assert max(bc["ctas"] for bc in buckets) >= 2 * sms, buckets
    b.close()
    del bufs


def test_batch_without_graph_and_new_view_matrices(gpu, oracle):
    import torch
    from hellovulkan_gb300.batch import Batch, BatchBuffers
    views = mixed_views()[:6]
    bufs = BatchBuffers(views)
    b = Batch(gpu)
    b.set_graph(False)
    b.set_views(bufs.batch_views())
    b.generate_aabbs()
    b.cull()
    check_all(oracle, bufs)
    # new cameraView matrices, same projections: AABBs stay valid
    rng = np.random.default_rng(8)
    ubos = []
    for v in views:
        u = ubo_from_bytes(bytes(v.ubo))
        vm = look_at_rh(rng.uniform(-30, 30, 3), rng.uniform(-5, 5, 3))
        u.cameraView[:] = np.ascontiguousarray(vm.T).reshape(16).tolist()
        v.ubo = u
        ubos.append(u)
    b.update_view_matrices(ubos)
    b.cull()
    torch.cuda.synchronize()
    check_all(oracle, bufs)


def test_batch_autotune_and_every_configuration_stay_exact(gpu, oracle):
    import torch
    from hellovulkan_gb300.batch import Batch, BatchBuffers
    views = mixed_views()[8:]
    bufs = BatchBuffers(views)
    b = Batch(gpu)
    b.set_views(bufs.batch_views())
    s = torch.cuda.Stream()
    b.generate_aabbs(s)
    keys = sorted({v.grid[0] * v.grid[1] for v in views})
    for cfg in [(1, 4, 256, 4), (4, 8, 256, 4), (2, 4, 512, 2), (4, 8, 1024, 2)]:
        for k in keys:
            b.set_tuning(k, *cfg)
        b.cull(s)
        check_all(oracle, bufs)
    b.autotune(2, s)
    b.cull(s)
    check_all(oracle, bufs)
    assert all(bc["config"][0] in (1, 2, 4) for bc in b.info()["bucket_configs"])


def test_batch_rejects_bad_views(gpu):
    from hellovulkan_gb300 import CfError
    from hellovulkan_gb300.batch import Batch, BatchBuffers
    v = scenes.plain_small(1)
    bufs = BatchBuffers([v])
    bvs = bufs.batch_views()
    bvs[0].index_capacity = 10
    b = Batch(gpu)
    with pytest.raises(CfError) as e:
        b.set_views(bvs)
    assert e.value.status == 4
    bvs = bufs.batch_views()
    bvs[0].d_cells = None
    with pytest.raises(CfError) as e:
        b.set_views(bvs)
    assert e.value.status == 1
