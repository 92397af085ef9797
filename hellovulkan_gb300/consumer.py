"""The consumer side of the culled lists (include/cfcull.h, cf_lookup_clusters,
cf_shade_clusters).

    samples = lookup_clusters(ubo, depth, cells, indices, lights, index_count, light_count)
    rgba = shade_clusters(ubo, camera_position, pc, gbuffer, cells, indices, index_count, lights, light_count)

Scene.frag's per-fragment cluster lookup (HelloVulkan/Shaders/ClusteredForward/
Scene.frag:54-78) run on the GPU over a depth buffer: which cluster each pixel
reads, its (offset, count), how many of its listed lights contain the
fragment, and (check mode) how many lights the list lacks.
"""
from __future__ import annotations

import numpy as np

from ._lib import FRAGMENT_DTYPE, check, lib, stream_handle


def lookup_clusters(ubo, depth, cells, indices, lights, index_count: int, light_count: int, cap: int = 150,
                    aabbs=None, check_all: bool = True, stream=None):
    """depth, cells, indices, lights, aabbs: device tensors (or addresses);
    returns a torch uint8 tensor holding height x width CfFragmentSample
    records (view it with .cpu().numpy().view(FRAGMENT_DTYPE))."""
    import ctypes as C

    import torch
    h, w = int(depth.shape[0]), int(depth.shape[1])
    out = torch.empty(h * w * FRAGMENT_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
    addr = lambda t: None if t is None else (t if isinstance(t, int) else t.data_ptr())  # noqa: E731
    check(lib().cf_lookup_clusters(C.byref(ubo), addr(depth), w, h, addr(cells), addr(indices), index_count,
                                   addr(lights), light_count, cap, addr(aabbs), int(check_all), out.data_ptr(),
                                   stream_handle(stream)))
    return out


def samples_to_numpy(out, height: int, width: int) -> np.ndarray:
    return out.cpu().numpy().view(FRAGMENT_DTYPE).reshape(height, width)


def shade_clusters(ubo, camera_position, pc, gbuffer, cells, indices, index_count: int, lights, light_count: int,
                   stream=None):
    """gbuffer: (h, w, 12) float32 device tensor of CfGBufferTexel records;
    returns an (h, w, 4) float32 device tensor (Lo, alpha) — Scene.frag's
    direct clustered lighting over the culled lists."""
    import ctypes as C

    import torch
    h, w = int(gbuffer.shape[0]), int(gbuffer.shape[1])
    out = torch.empty((h, w, 4), dtype=torch.float32, device="cuda")
    addr = lambda t: None if t is None else (t if isinstance(t, int) else t.data_ptr())  # noqa: E731
    cam = (C.c_float * 3)(*[float(v) for v in camera_position[:3]])
    check(lib().cf_shade_clusters(C.byref(ubo), cam, C.byref(pc), addr(gbuffer), w, h, addr(cells), addr(indices),
                                  index_count, addr(lights), light_count, out.data_ptr(), stream_handle(stream)))
    return out


def frustum_cull(frustum, boxes, commands, visible=None, stream=None) -> None:
    """FrustumCulling.comp over device tensors: boxes (n, 8) float32 AABBs,
    commands (n, 4) uint32/int32 VkDrawIndirectCommand records whose
    instanceCount is set to 0 or 1; visible: optional one-element counter."""
    import ctypes as C
    check(lib().cf_frustum_cull(C.byref(frustum), boxes.data_ptr(), int(boxes.shape[0]), commands.data_ptr(),
                                None if visible is None else visible.data_ptr(), stream_handle(stream)))
