"""The consumer side of the culled lists (include/cfcull.h, cf_lookup_clusters).

    samples = lookup_clusters(ubo, depth, cells, indices, lights, index_count)

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
