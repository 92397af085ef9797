"""Batched culling of many views (include/cfcull.h, cf_batch_*).

    bufs = BatchBuffers(views)          # device buffers for a list of scenes.View
    b = Batch(ctx); b.set_views(bufs.batch_views())
    b.generate_aabbs(stream); b.cull(stream)        # CUDA-graph replay after the first call
    aabbs, cells, indices = bufs.read(i)
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from ._lib import CfBatchInfo, CfBatchView, check, lib, stream_handle


class Batch:
    def __init__(self, ctx):
        self.ctx = ctx
        h = C.c_void_p()
        check(lib().cf_batch_create(ctx.handle, C.byref(h)))
        self.handle = h
        self._views = None

    def set_views(self, views) -> None:
        arr = (CfBatchView * len(views))(*views)
        self._views = arr
        check(lib().cf_batch_set_views(self.handle, arr, len(views)))

    def update_view_matrices(self, ubos, stream=None) -> None:
        from ._lib import CfClusterForwardUBO
        arr = (CfClusterForwardUBO * len(ubos))(*ubos)
        check(lib().cf_batch_update_view_matrices(self.handle, arr, len(ubos), stream_handle(stream)))

    def generate_aabbs(self, stream=None) -> None:
        check(lib().cf_batch_generate_aabbs(self.handle, stream_handle(stream)))

    def cull(self, stream=None) -> None:
        check(lib().cf_batch_cull(self.handle, stream_handle(stream)))

    def set_graph(self, enable: bool) -> None:
        check(lib().cf_batch_set_graph(self.handle, int(enable)))

    def set_tuning(self, slice_clusters: int, clusters_per_warp=0, warps=0, tile=0, stages=0) -> None:
        check(lib().cf_batch_set_tuning(self.handle, slice_clusters, clusters_per_warp, warps, tile, stages))

    def autotune(self, repeats: int = 3, stream=None) -> None:
        check(lib().cf_batch_autotune(self.handle, repeats, stream_handle(stream)))

    def info(self) -> dict:
        i = CfBatchInfo()
        check(lib().cf_batch_get_info(self.handle, C.byref(i)))
        return {"views": i.views, "items": i.items, "buckets": i.buckets, "workspace_bytes": i.workspace_bytes,
                "bucket_configs": [{"slice_clusters": i.bucket_slice_clusters[q],
                                    "config": list(i.bucket_config[q]), "ctas": i.bucket_ctas[q]}
                                   for q in range(min(i.buckets, 8))]}

    def close(self):
        if self.handle:
            lib().cf_batch_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class BatchBuffers:
    """Device buffers (torch tensors) of a list of scenes.View for a batch."""

    def __init__(self, views):
        import torch
        self.views = list(views)
        self.lights, self.aabbs, self.cells, self.indices, self.totals = [], [], [], [], []
        for v in self.views:
            n, cap = v.clusters, v.cap
            self.lights.append(torch.from_numpy(np.ascontiguousarray(v.lights, np.float32)).cuda())
            self.aabbs.append(torch.empty(n * 8, dtype=torch.float32, device="cuda"))
            self.cells.append(torch.empty(n * 2, dtype=torch.int32, device="cuda"))
            self.indices.append(torch.empty(n * cap, dtype=torch.int32, device="cuda"))
            self.totals.append(torch.zeros(1, dtype=torch.int32, device="cuda"))

    def batch_views(self):
        out = []
        for i, v in enumerate(self.views):
            bv = CfBatchView()
            bv.ubo = v.ubo
            bv.d_lights = self.lights[i].data_ptr() if v.light_count else None
            bv.d_aabbs = self.aabbs[i].data_ptr()
            bv.d_cells = self.cells[i].data_ptr()
            bv.d_indices = self.indices[i].data_ptr()
            bv.d_total = self.totals[i].data_ptr()
            bv.index_capacity = v.clusters * v.cap
            bv.light_count = v.light_count
            bv.max_lights_per_cluster = v.cap
            out.append(bv)
        return out

    def set_lights(self, i: int, lights: np.ndarray) -> None:
        """Overwrites view i's light records in place (same count)."""
        import torch
        self.lights[i].copy_(torch.from_numpy(np.ascontiguousarray(lights, np.float32)))

    def read(self, i: int):
        """(aabbs (C,8) float32, cells (C,2) uint32, indices (total,) uint32) of view i."""
        import torch
        torch.cuda.synchronize()
        v = self.views[i]
        t = int(self.totals[i].item())
        return (self.aabbs[i].cpu().numpy().reshape(v.clusters, 8),
                self.cells[i].cpu().numpy().view(np.uint32).reshape(v.clusters, 2),
                self.indices[i][:t].cpu().numpy().view(np.uint32).copy())

    @property
    def device_bytes(self) -> int:
        return sum(t.numel() * t.element_size() for ts in (self.lights, self.aabbs, self.cells, self.indices,
                                                              self.totals) for t in ts)
