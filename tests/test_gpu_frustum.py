"""GPU tests of FrustumCulling.comp (cf_frustum_cull): every box's
instanceCount bit for bit against the oracle and against the reference
shader's own outputs (golden_consumers.npz), the commands' other fields
untouched, and the optional visible count."""
import math

import numpy as np
import pytest

from hellovulkan_gb300 import scenes
from hellovulkan_gb300.camera import frustum_ubo

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n,seed", [(10000, 1), (1_000_003, 2)])
def test_frustum_culling_matches_the_oracle(gpu, oracle, n, seed):
    import torch
    from hellovulkan_gb300.consumer import frustum_cull
    rng = np.random.default_rng(seed)
    boxes = scenes.random_boxes(rng, n)
    # boxes the fast plane test must treat like the shader: inverted (min >
    # max on an axis), degenerate, far beyond the safe magnitude, non-finite
    k = n // 10
    boxes[:k, [0, 4]] = boxes[:k, [4, 0]]
    boxes[k:2 * k, 4:7] = boxes[k:2 * k, 0:3]
    boxes[2 * k:2 * k + 50, 0] = -3e20
    boxes[2 * k + 50:2 * k + 100, 5] = np.inf
    boxes[2 * k + 100:2 * k + 150, 2] = np.nan
    cmds = np.zeros((n, 4), np.uint32)
    cmds[:, 0] = 36  # vertexCount, firstVertex, firstInstance must stay as they are
    cmds[:, 1] = 7
    cmds[:, 2] = np.arange(n, dtype=np.uint32)
    cmds[:, 3] = 3
    for _ in range(3):
        f = frustum_ubo(math.radians(rng.uniform(30, 90)), rng.uniform(1.0, 2.5), 0.1, float(rng.uniform(100, 1000)),
                        scenes.random_camera(rng))
        d_boxes = torch.from_numpy(boxes).cuda()
        d_cmds = torch.from_numpy(cmds.view(np.int32)).cuda()
        visible = torch.zeros(1, dtype=torch.int32, device="cuda")
        frustum_cull(f, d_boxes, d_cmds, visible)
        got = d_cmds.cpu().numpy().view(np.uint32)
        want = oracle.frustum_cull(f, boxes)
        assert np.array_equal(got[:, 1], want)
        assert np.array_equal(got[:, [0, 2, 3]], cmds[:, [0, 2, 3]])
        assert int(visible.item()) == int(want.sum()) and 0 < want.sum() < n


def test_frustum_culling_matches_the_reference_golden(gpu, golden_consumers):
    """The fixture's boxes (random, inverted, degenerate, huge, infinite, NaN,
    signed-zero) under three frusta: the kernel's single-corner plane test
    gives FrustumCulling.comp's eight-corner answers."""
    import torch
    from hellovulkan_gb300._lib import CfFrustum
    from hellovulkan_gb300.consumer import frustum_cull
    boxes = golden_consumers["frustum/boxes"]
    d_boxes = torch.from_numpy(boxes).cuda()
    for k in range(3):
        f = CfFrustum.from_buffer_copy(golden_consumers["frustum/f%d" % k].tobytes())
        d_cmds = torch.zeros((boxes.shape[0], 4), dtype=torch.int32, device="cuda")
        frustum_cull(f, d_boxes, d_cmds)
        got = d_cmds.cpu().numpy().view(np.uint32)[:, 1]
        assert np.array_equal(got, golden_consumers["frustum/instance%d" % k].astype(np.uint32)), k
