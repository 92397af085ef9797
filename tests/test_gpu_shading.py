"""GPU tests of Scene.frag's direct clustered lighting over the culled lists
(cf_shade_clusters): every texel bit for bit against the oracle's
restatement of Radiance.glsl, at a reduced and at the full 1920x1080 size,
and against the reference fragment code's own outputs (golden_consumers.npz),
including a signed-zero case."""
import numpy as np
import pytest

from hellovulkan_gb300 import scenes
from hellovulkan_gb300._lib import CfPBRPushConstant

pytestmark = pytest.mark.gpu

PC = CfPBRPushConstant(1.75, 0.01, 0.0, 0.1, 0.1)  # the reference UI's defaults (Header/UIData.h:23-29)


def shade_both(gpu, oracle, view, seed):
    import torch
    from gpu_helpers import run_pipeline
    from hellovulkan_gb300.consumer import shade_clusters
    aabbs, cells, idx = run_pipeline(gpu, view)
    g = scenes.gbuffer(np.random.default_rng(seed), view.ubo, far_plane_fraction=0.01)
    cam = scenes.camera_position(view.ubo)
    d_idx = torch.from_numpy(idx.view(np.int32).copy() if idx.size else np.zeros(1, np.int32)).cuda()
    out = shade_clusters(view.ubo, cam, PC, torch.from_numpy(g).cuda(), torch.from_numpy(cells.view(np.int32)).cuda(),
                         d_idx, idx.size, torch.from_numpy(np.ascontiguousarray(view.lights)).cuda(),
                         view.light_count)
    got = out.cpu().numpy()
    want = oracle.shade_clusters(view.ubo, cam, PC, g, cells, idx, view.lights)
    return got, want, g


def test_shading_matches_the_oracle(gpu, oracle):
    rng = np.random.default_rng(21)
    v = scenes.custom_view((16, 9, 24), 480, 270, 0.1, 1000.0, np.eye(4, dtype=np.float32),
                           scenes.uniform_box_lights(rng, 2000, [-20, -5, -60], [20, 15, -1], 1.0, 8.0))
    got, want, g = shade_both(gpu, oracle, v, 22)
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))
    assert np.all((got[..., 3] == 0) == (g[..., 3] == 1.0))  # far-plane texels leave the grid
    lit = got[..., :3] > (g[..., 8:11] * PC.albedoMultipler)
    assert lit.any()


def test_shading_at_full_resolution(gpu, oracle):
    v = scenes.plain_small(1)  # 1920x1080, 16x9x24, 1024 lights
    got, want, _ = shade_both(gpu, oracle, v, 23)
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))
    assert np.isfinite(got).all() and (got[..., 3] == 1.0).mean() > 0.98


def _shade_golden(g, prefix, ubo, cam):
    import torch
    from hellovulkan_gb300.consumer import shade_clusters
    cells, idx, lights = g[prefix + "/cells"], g[prefix + "/indices"], g[prefix + "/lights"]
    pc = CfPBRPushConstant(*g[prefix + "/pc"].tolist())
    out = shade_clusters(ubo, cam, pc, torch.from_numpy(g[prefix + "/gbuffer"]).cuda(),
                         torch.from_numpy(cells.view(np.int32)).cuda(),
                         torch.from_numpy(idx.view(np.int32).copy()).cuda(), idx.size,
                         torch.from_numpy(np.ascontiguousarray(lights)).cuda(), lights.shape[0])
    return out.cpu().numpy()


def test_shading_matches_the_reference_golden(gpu, golden_consumers):
    """Lo bits as Scene.frag's loop over Radiance.glsl computes them, and alpha
    1 exactly where the lookup lands in the grid."""
    from hellovulkan_gb300.camera import ubo_from_bytes
    g = golden_consumers
    got = _shade_golden(g, "frag", ubo_from_bytes(g["frag/ubo"]), g["frag/camera"])
    assert np.array_equal(got[..., :3].view(np.uint32), g["frag/shade_rgb"])
    assert np.array_equal(got[..., 3] == 1.0, g["frag/shade_cluster"] < g["frag/cells"].shape[0])


def test_shading_signed_zero_matches_the_reference_golden(gpu, golden_consumers):
    """albedoMultipler -0.0 and a light whose term is -0: Radiance's own Lo
    starts at +0, so the texel's Lo is +0 in every channel, as in the shader."""
    from hellovulkan_gb300.camera import ubo_from_bytes
    g = golden_consumers
    got = _shade_golden(g, "negzero", ubo_from_bytes(g["negzero/ubo"]), np.zeros(3))
    assert np.array_equal(got[..., :3].view(np.uint32), g["negzero/shade_rgb"])
    assert not np.signbit(got[..., :3]).any()
