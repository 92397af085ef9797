"""GPU parity: the CUDA path through the C ABI against the oracle and the
golden fixtures made from the reference's own shaders.  The bar is bit-exact:
AABB float bits, LightCells and the index list."""
import numpy as np
import pytest

from gpu_helpers import assert_matches_oracle, bits, run_pipeline, run_stateless, sha
from hellovulkan_gb300 import scenes
from hellovulkan_gb300.camera import look_at_rh, ubo_from_bytes

pytestmark = pytest.mark.gpu

TUNINGS = ([(k, w, 512, 4, 0) for k in (1, 2, 4) for w in (4, 8)] + [(k, w, 256, 4, 1) for k in (1, 2, 4) for w in (4, 8)]
           + [(k, w, 512, 2, 1) for k in (2, 4) for w in (4, 8)] + [(k, 8, 1024, 2, 1) for k in (2, 4)])


def golden_views(golden):
    for name in [str(n) for n in golden["names"]]:
        v = scenes.View(ubo_from_bytes(golden[name + "/ubo"]), golden[name + "/lights"],
                        int(golden[name + "/cap"][0]), name)
        yield name, v


def test_golden_cases_through_the_pipelines(gpu, golden):
    for name, v in golden_views(golden):
        aabbs, cells, idx = run_pipeline(gpu, v)
        if name + "/aabbs" in golden.files:
            assert np.array_equal(bits(aabbs), golden[name + "/aabbs"]), name
            assert np.array_equal(cells, golden[name + "/cells"]), name
            assert np.array_equal(idx, golden[name + "/indices"]), name
        else:
            assert sha(bits(aabbs)) == str(golden[name + "/sha_aabbs"]), name
            assert sha(cells) == str(golden[name + "/sha_cells"]), name
            assert sha(idx) == str(golden[name + "/sha_indices"]), name


def test_golden_cases_through_the_stateless_entry_points(gpu, golden):
    for name, v in golden_views(golden):
        aabbs, cells, idx = run_stateless(v)
        if name + "/aabbs" in golden.files:
            assert np.array_equal(bits(aabbs), golden[name + "/aabbs"]), name
            assert np.array_equal(cells, golden[name + "/cells"]), name
            assert np.array_equal(idx, golden[name + "/indices"]), name


def test_plain_small_full_size(gpu, oracle):
    v = scenes.plain_small(1)
    assert_matches_oracle(oracle, v, *run_pipeline(gpu, v))


def test_plain_large_full_size(gpu, oracle):
    v = scenes.plain_large(2)
    assert_matches_oracle(oracle, v, *run_pipeline(gpu, v))


@pytest.mark.parametrize("tuning", TUNINGS)
def test_every_kernel_configuration(gpu, oracle, golden, tuning):
    views = dict(golden_views(golden))
    for name in ("cap_dense", "all_capped", "nonfinite_lights", "odd_grid_odd_lights", "grid_1x1x1"):
        assert_matches_oracle(oracle, views[name], *run_pipeline(gpu, views[name], tuning))
    v = scenes.plain_large(9, n_lights=3000)
    assert_matches_oracle(oracle, v, *run_pipeline(gpu, v, tuning))


@pytest.mark.parametrize("tuning", [(2, 8, 1024, 2, 1), (4, 8, 1024, 2, 1), (4, 4, 512, 2, 1), (2, 8, 256, 4, 1)])
def test_dense_slices_with_a_short_last_group(gpu, oracle, tuning):
    """Slices with thousands of candidates (several tiles per cluster group)
    on a 15-wide grid, whose last group per slice is short."""
    rng = np.random.default_rng(17)
    lights = scenes.uniform_box_lights(rng, 8000, [-30, -15, -60], [30, 15, -5], 2.0, 6.0)
    v = scenes.custom_view((15, 9, 24), 1920, 1080, 0.1, 300.0, lights=lights)
    assert_matches_oracle(oracle, v, *run_pipeline(gpu, v, tuning))


@pytest.mark.parametrize("tuning", TUNINGS + [None])
def test_nan_lights_where_a_warp_holds_a_cluster_past_the_end(gpu, oracle, tuning):
    """A warp's cluster past the end of its item (a slice's short last group,
    or the view's last group for the brute-force kernel) holds a +inf box,
    which a light with a NaN coordinate still reaches: the shader's test
    counts a NaN axis as 0.  15x9 clusters per slice and 945 in all put such a
    cluster in the same warp as real ones for every K > 1; nothing may be
    written for it (it would land in the next slice's lists, or past the
    staging rows)."""
    rng = np.random.default_rng(29)
    lights = scenes.uniform_box_lights(rng, 600, [-20, -10, -60], [20, 10, -1], 1.0, 6.0)
    lights[[3, 100, 301, 450], 0] = np.nan
    lights[7, 1] = np.nan
    lights[222, 2] = np.nan
    v = scenes.custom_view((15, 9, 7), 1920, 1080, 0.1, 300.0, lights=lights)
    assert_matches_oracle(oracle, v, *run_pipeline(gpu, v, tuning))


@pytest.mark.parametrize("n_lights", [1, 31, 33, 64, 65, 4097, 8193])
def test_list_segments_around_the_split(gpu, oracle, n_lights):
    """A binned single view bins each slice with two CTAs, one per half of
    the padded lights, into two segments of the slice's list: light counts
    around the split point, an empty second segment, tiles that take lights
    from both segments, and a non-finite light that only the second segment
    lists (its slices take the exact test)."""
    rng = np.random.default_rng(31 + n_lights)
    lights = scenes.uniform_box_lights(rng, n_lights, [-30, -15, -60], [30, 15, -5], 2.0, 6.0)
    if n_lights >= 33:
        lights[n_lights - 1, 1] = np.inf
    v = scenes.custom_view((15, 9, 24), 1920, 1080, 0.1, 300.0, lights=lights)
    assert_matches_oracle(oracle, v, *run_pipeline(gpu, v, (2, 8, 1024, 2, 1)))


@pytest.mark.parametrize("tuning", [(1, 4, 512, 4, 0), (1, 4, 256, 4, 1), (2, 8, 1024, 2, 1)])
def test_offsets_with_and_without_a_scan_launch(gpu, oracle, tuning):
    """Views of more than 8192 cluster groups scan the group totals in a launch
    of their own; smaller ones let each copy block sum the earlier groups."""
    rng = np.random.default_rng(23)
    v = scenes.custom_view((64, 36, 24), 3840, 2160, 0.1, 500.0,
                           lights=scenes.uniform_box_lights(rng, 600, [-40, -20, -150], [40, 20, -1], 1.0, 6.0))
    assert_matches_oracle(oracle, v, *run_pipeline(gpu, v, tuning))


@pytest.mark.parametrize("tuning", [None, (1, 8, 512, 4, 0)])
def test_single_view_step_replayed_from_a_cuda_graph(gpu, oracle, tuning):
    """A caller may capture a step (launched with programmatic dependent
    launch) into a CUDA graph and replay it over new light positions."""
    import torch
    from hellovulkan_gb300.pipelines import (PipelineAABBGenerator, PipelineLightCulling, ResourcesClusterForward,
                                             ResourcesLight)
    v = scenes.plain_large(5, n_lights=6000)
    rl = ResourcesLight(gpu)
    rl.add_lights(v.lights)
    rc = ResourcesClusterForward(gpu)
    rc.create_buffers(*v.grid, v.cap)
    gen = PipelineAABBGenerator(gpu, rc)
    gen.set_cluster_forward_ubo(v.ubo)
    gen.fill_command_buffer()
    cull = PipelineLightCulling(gpu, rl, rc)
    if tuning:
        cull.set_tuning(*tuning)
    cull.set_cluster_forward_ubo(v.ubo)
    cull.fill_command_buffer()  # outside the capture: workspace and kernel attributes
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g):
        cull.fill_command_buffer(torch.cuda.current_stream())
    aabbs = oracle.generate_aabbs(v.ubo)
    rng = np.random.default_rng(31)
    for _ in range(2):
        moved = v.lights.copy()
        moved[:, :3] += rng.normal(0.0, 2.0, size=(moved.shape[0], 3)).astype(np.float32)
        host = torch.from_numpy(moved).pin_memory()
        rl.upload_async(host, moved.shape[0], torch.cuda.current_stream())
        g.replay()
        torch.cuda.synchronize()
        cells, idx = rc.read_outputs()
        oc, oi, _ = oracle.cull(v.ubo, aabbs, moved, v.cap)
        assert np.array_equal(cells, oc) and np.array_equal(idx, oi)
    assert gpu.check_device_error() == 0
    for o in (cull, gen, rc, rl):
        o.close()


def test_read_outputs_into_pinned_memory(gpu, oracle):
    """The one-launch read-back into pinned host buffers gives what the
    two-copy path gives: the full lists, and a prefix for a short index buffer."""
    import torch
    from hellovulkan_gb300.pipelines import (PipelineAABBGenerator, PipelineLightCulling, ResourcesClusterForward,
                                             ResourcesLight)
    v = scenes.plain_large(4, n_lights=8000)
    rl = ResourcesLight(gpu)
    rl.add_lights(v.lights)
    rc = ResourcesClusterForward(gpu)
    rc.create_buffers(*v.grid, v.cap)
    gen = PipelineAABBGenerator(gpu, rc)
    gen.set_cluster_forward_ubo(v.ubo)
    gen.fill_command_buffer()
    cull = PipelineLightCulling(gpu, rl, rc)
    cull.set_cluster_forward_ubo(v.ubo)
    cull.fill_command_buffer()
    cells_p, idx_p = rc.read_outputs()  # pageable numpy buffers: two copies
    oc, oi, _ = oracle.cull(v.ubo, oracle.generate_aabbs(v.ubo), v.lights, v.cap)
    assert np.array_equal(cells_p, oc) and np.array_equal(idx_p, oi)
    b = rc.buffers()
    pinned = [torch.zeros((b.cluster_count, 2), dtype=torch.int32).pin_memory(),
              torch.zeros(b.index_capacity, dtype=torch.int32).pin_memory(),
              torch.zeros(1001, dtype=torch.int32).pin_memory()]
    h_cells, h_idx, h_short = (t.numpy().view(np.uint32) for t in pinned)
    s = torch.cuda.Stream()
    cells, idx = rc.read_outputs(s, h_cells, h_idx)
    assert np.array_equal(cells, oc) and np.array_equal(idx, oi)
    # a short host index buffer (offset by one word: no 16-byte accesses) gets a prefix
    short = h_short[1:]
    _, part = rc.read_outputs(s, h_cells, short)
    assert part.size == min(oi.size, short.size) and np.array_equal(part, oi[:part.size])
    assert gpu.check_device_error() == 0
    for o in (cull, gen, rc, rl):
        o.close()


def test_batch_mix_views(gpu, oracle):
    views = scenes.batch_mix(3, n_views=12)
    views.sort(key=lambda v: -v.light_count)
    for v in views[:3] + views[-3:]:  # the largest (up to 65536 lights) and the smallest
        assert_matches_oracle(oracle, v, *run_pipeline(gpu, v))


def test_aabbs_over_varied_projections(gpu, oracle):
    """Exercises the pinned pow and the mat4 order on the device."""
    rng = np.random.default_rng(11)
    for _ in range(12):
        grid = (int(rng.integers(1, 40)), int(rng.integers(1, 30)), int(rng.integers(1, 64)))
        near = float(rng.uniform(0.01, 2.0))
        far = float(near * 10 ** rng.uniform(0.5, 5))
        fovy = float(np.radians(rng.uniform(20, 110)))
        v = scenes.custom_view(grid, int(rng.integers(64, 4096)), int(rng.integers(64, 4096)), near, far,
                               view=look_at_rh(rng.uniform(-5, 5, 3), rng.uniform(-5, 5, 3) + [0, 0, -10]),
                               lights=scenes.uniform_box_lights(rng, 100, [-50, -50, -200], [50, 50, 10]), fovy=fovy)
        assert_matches_oracle(oracle, v, *run_stateless(v))


def test_known_answer_cap_order(gpu, oracle):
    v = scenes.custom_view((1, 1, 1), 100, 100, 1.0, 10.0)
    a = oracle.generate_aabbs(v.ubo)
    centre = (a[0, 0:3] + a[0, 4:7]) / 2
    pos = np.array([[0.0, 0.0, 1e4] if i % 3 == 0 else centre for i in range(400)], np.float32)
    v.lights = scenes.make_lights(pos, np.ones(400, np.float32))
    aabbs, cells, idx = run_pipeline(gpu, v)
    assert list(idx) == [i for i in range(400) if i % 3 != 0][:150]


def test_deterministic_across_runs_and_streams(gpu):
    import torch
    v = scenes.plain_large(4, n_lights=8000)
    a1 = run_pipeline(gpu, v)
    s = torch.cuda.Stream()
    a2 = run_pipeline(gpu, v, stream=s)
    for x, y in zip(a1, a2):
        assert np.array_equal(np.asarray(x).view(np.uint32), np.asarray(y).view(np.uint32))


def test_pipeline_semantics(gpu, oracle):
    """aabbDirty_ handling, UpdateLightPosition and ResetGlobalIndex."""
    from hellovulkan_gb300.pipelines import (PipelineAABBGenerator, PipelineLightCulling, ResourcesClusterForward,
                                             ResourcesLight)
    v = scenes.plain_small(2)
    rl = ResourcesLight(gpu)
    rl.add_lights(v.lights)
    assert rl.light_count == v.light_count and rl.device_buffer != 0
    rc = ResourcesClusterForward(gpu)
    rc.create_buffers(16, 9, 24, 150)
    gen = PipelineAABBGenerator(gpu, rc)
    cull = PipelineLightCulling(gpu, rl, rc)
    assert rc.aabb_dirty
    gen.set_cluster_forward_ubo(v.ubo)
    gen.fill_command_buffer()
    assert not rc.aabb_dirty
    gen.set_cluster_forward_ubo(v.ubo)  # same projection: stays clean
    assert not rc.aabb_dirty
    gen.on_window_resized()
    assert rc.aabb_dirty
    gen.fill_command_buffer()
    zoomed = scenes.custom_view((16, 9, 24), 1920, 1080, 0.1, 1000.0, fovy=np.radians(30.0)).ubo
    gen.set_cluster_forward_ubo(zoomed)  # a zoom changes the projection: dirty again
    assert rc.aabb_dirty
    gen.set_cluster_forward_ubo(v.ubo)
    gen.fill_command_buffer()
    # move one light, as ResourcesLight::UpdateLightPosition
    moved = v.lights.copy()
    moved[7, :4] = [1.0, 2.0, -30.0, 1.0]
    rl.update_light_position(7, (1.0, 2.0, -30.0))
    rl.update_light_position(10 ** 6, (0.0, 0.0, 0.0))  # out of range: ignored
    cull.reset_global_index()
    cull.set_cluster_forward_ubo(v.ubo)
    cull.fill_command_buffer()
    cells, idx = rc.read_outputs()
    a = oracle.generate_aabbs(v.ubo)
    oc, oi, _ = oracle.cull(v.ubo, a, moved)
    assert np.array_equal(cells, oc) and np.array_equal(idx, oi)
    # running twice without re-uploading gives the same result (no counter to reset)
    cull.fill_command_buffer()
    cells2, idx2 = rc.read_outputs()
    assert np.array_equal(cells, cells2) and np.array_equal(idx, idx2)


def test_pipeline_error_paths(gpu):
    from hellovulkan_gb300 import CfError
    from hellovulkan_gb300.pipelines import (PipelineAABBGenerator, PipelineLightCulling, ResourcesClusterForward,
                                             ResourcesLight)
    rl, rc = ResourcesLight(gpu), ResourcesClusterForward(gpu)
    gen, cull = PipelineAABBGenerator(gpu, rc), PipelineLightCulling(gpu, rl, rc)
    with pytest.raises(CfError) as e:
        gen.fill_command_buffer()
    assert e.value.status == 5  # no UBO yet
    with pytest.raises(CfError) as e:
        rc.create_buffers(0, 9, 24)
    assert e.value.status == 1
    rc.create_buffers(16, 9, 24)
    v = scenes.plain_small(1)
    cull.set_cluster_forward_ubo(v.ubo)
    with pytest.raises(CfError) as e:
        cull.fill_command_buffer()  # the AABB generator never ran
    assert e.value.status == 5
    wrong = scenes.custom_view((8, 8, 8), 100, 100, 0.1, 10.0).ubo
    gen.set_cluster_forward_ubo(wrong)
    with pytest.raises(CfError) as e:
        gen.fill_command_buffer()
    assert e.value.status == 1
