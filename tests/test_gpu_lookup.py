"""GPU tests of Scene.frag's cluster lookup over the culled lists
(cf_lookup_clusters): every per-pixel field bit for bit against the oracle,
the cluster, cell and LinearDepth against the reference fragment code's own
outputs (golden_consumers.npz), and the drop-in property at full resolution (a light that contains a
fragment is in its cluster's list unless the fragment lies outside the
cluster's box or the list is capped)."""
import numpy as np
import pytest

from hellovulkan_gb300 import scenes
from hellovulkan_gb300._lib import FRAGMENT_BAD_CELL, FRAGMENT_CAPPED, FRAGMENT_OUTSIDE_AABB, FRAGMENT_OUTSIDE_GRID

pytestmark = pytest.mark.gpu


def culled(gpu, view):
    """(pipeline objects, aabbs, cells, indices) for a view culled on the GPU."""
    from gpu_helpers import run_pipeline
    return run_pipeline(gpu, view)


def device_lookup(view, depth, cells, idx, aabbs, check_all=True):
    import torch
    from hellovulkan_gb300.consumer import lookup_clusters, samples_to_numpy
    d_depth = torch.from_numpy(depth).cuda()
    d_cells = torch.from_numpy(cells.view(np.int32)).cuda()
    d_idx = torch.from_numpy(idx.view(np.int32).copy() if idx.size else np.zeros(1, np.int32)).cuda()
    d_lights = torch.from_numpy(np.ascontiguousarray(view.lights)).cuda()
    d_aabbs = torch.from_numpy(np.ascontiguousarray(aabbs, np.float32)).cuda()
    out = lookup_clusters(view.ubo, d_depth, d_cells, d_idx, d_lights, idx.size, view.light_count, view.cap,
                          d_aabbs, check_all)
    torch.cuda.synchronize()
    return samples_to_numpy(out, *depth.shape)


def same(a, b):
    return all(np.array_equal(a[k].view(np.uint32), b[k].view(np.uint32)) for k in a.dtype.names)


@pytest.mark.parametrize("res", [(480, 270), (640, 400)])
def test_lookup_matches_the_oracle(gpu, oracle, res):
    rng = np.random.default_rng(res[0])
    w, h = res
    grid = (16, 9, 24) if w * 9 == h * 16 else (32, 20, 32)
    v = scenes.custom_view(grid, w, h, 0.1, 1000.0, scenes.random_camera(rng),
                           scenes.blob_lights(rng, 3000))
    aabbs, cells, idx = culled(gpu, v)
    depth = scenes.depth_log_uniform(rng, w, h, 0.1, 1000.0, far_plane_fraction=0.02)
    got = device_lookup(v, depth, cells, idx, aabbs)
    want = oracle.lookup_clusters(v.ubo, depth, cells, idx, v.lights, v.cap, aabbs, True)
    assert same(got, want)
    assert np.all((got["flags"] & FRAGMENT_OUTSIDE_GRID > 0) == (depth == 1.0))
    assert got["covering"].sum() > 0


def test_lookup_drop_in_property_at_full_resolution(gpu):
    v = scenes.plain_small(1)  # 1920x1080, 16x9x24, 1024 lights
    aabbs, cells, idx = culled(gpu, v)
    depth = scenes.depth_log_uniform(np.random.default_rng(7), 1920, 1080, 0.1, 1000.0)
    s = device_lookup(v, depth, cells, idx, aabbs)
    f = s["flags"]
    assert not np.any(f & (FRAGMENT_BAD_CELL | FRAGMENT_OUTSIDE_GRID))
    explained = (f & (FRAGMENT_OUTSIDE_AABB | FRAGMENT_CAPPED)) > 0
    assert not np.any((s["missing"] > 0) & ~explained)
    assert explained.mean() < 1e-3  # boundary rounding only
    assert np.all(s["covering"] <= s["count"])


def test_lookup_matches_the_reference_golden(gpu, golden_consumers):
    """cluster, count, offset and LinearDepth bits as Scene.frag:54-78 computes
    them (a fragment past the last slice reads a zero cell there, and is
    flagged OUTSIDE_GRID with count 0 here)."""
    from hellovulkan_gb300.camera import ubo_from_bytes
    g = golden_consumers
    ubo = ubo_from_bytes(g["frag/ubo"])
    cells, idx = g["frag/cells"], g["frag/indices"]
    v = scenes.View(ubo, g["frag/lights"], 150, "golden")
    aabbs = np.zeros((cells.shape[0], 8), np.float32)
    s = device_lookup(v, g["frag/depth"], cells, idx, aabbs, check_all=False)
    inside = g["frag/lookup_cluster"] < cells.shape[0]
    assert np.array_equal((s["flags"] & FRAGMENT_OUTSIDE_GRID) == 0, inside)
    assert np.array_equal(s["cluster"][inside], g["frag/lookup_cluster"][inside])
    assert np.array_equal(s["count"], g["frag/lookup_count"])
    assert np.array_equal(s["offset"], g["frag/lookup_offset"])
    assert np.array_equal(s["linear_depth"].view(np.uint32), g["frag/lookup_linear_depth"])
