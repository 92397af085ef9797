"""Python mirror of the reference's clustered-forward plugin classes over the C ABI.

    Context                  VulkanContext (one CUDA device)
    ResourcesLight           Header/Resources/ResourcesLight.h:42-81
    ResourcesClusterForward  Header/Resources/ResourcesClusterForward.h:11-31
    PipelineAABBGenerator    Header/Pipelines/PipelineAABBGenerator.h:17-39
    PipelineLightCulling     Header/Pipelines/PipelineLightCulling.h:18-30

Every method calls libcfcull.so and raises CfError on a non-zero status; the
per-frame sequence of AppPBRClusterForward::UpdateUBOs + FillCommandBuffer
(Source/Apps/AppPBRClusterForward.cpp:120-136, Source/Apps/AppBase.cpp:204-229)
becomes set_cluster_forward_ubo + fill_command_buffer(stream).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from ._lib import CfClusterForwardBuffers, CfClusterForwardUBO, check, lib, ptr, stream_handle


class Context:
    def __init__(self, device: int = 0):
        h = C.c_void_p()
        check(lib().cf_context_create(device, C.byref(h)))
        self.handle = h
        self.device = device

    def check_device_error(self) -> int:
        v = C.c_uint32(0)
        st = lib().cf_context_check_device_error(self.handle, C.byref(v))
        if st not in (0, 6):
            check(st)
        return int(v.value)

    def close(self):
        if self.handle:
            lib().cf_context_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class ResourcesLight:
    def __init__(self, ctx: Context):
        self.ctx = ctx
        h = C.c_void_p()
        check(lib().cf_resources_light_create(ctx.handle, C.byref(h)))
        self.handle = h

    def add_lights(self, lights: np.ndarray) -> None:
        """ResourcesLight::AddLights: lights is (n, 12) float32 (48-byte records)."""
        a = np.ascontiguousarray(lights, np.float32).reshape(-1, 12)
        check(lib().cf_resources_light_add_lights(self.handle, a.ctypes.data if a.size else None, a.shape[0]))

    def upload_async(self, lights, count: int, stream=None) -> None:
        """Copies `count` records from host memory (pinned torch tensor or numpy array)."""
        check(lib().cf_resources_light_upload_async(self.handle, ptr(lights), count, stream_handle(stream)))

    def update_light_position(self, index: int, position) -> None:
        p = (C.c_float * 3)(*[float(v) for v in position[:3]])
        check(lib().cf_resources_light_update_light_position(self.handle, index, p))

    @property
    def light_count(self) -> int:
        v = C.c_uint32()
        check(lib().cf_resources_light_get_light_count(self.handle, C.byref(v)))
        return int(v.value)

    @property
    def device_buffer(self) -> int:
        v = C.c_void_p()
        check(lib().cf_resources_light_get_device_buffer(self.handle, C.byref(v)))
        return int(v.value or 0)

    def close(self):
        if self.handle:
            lib().cf_resources_light_destroy(self.handle)
            self.handle = None


class ResourcesClusterForward:
    def __init__(self, ctx: Context):
        self.ctx = ctx
        h = C.c_void_p()
        check(lib().cf_resources_cluster_forward_create(ctx.handle, C.byref(h)))
        self.handle = h

    def create_buffers(self, x: int, y: int, z: int, max_lights_per_cluster: int = 150) -> None:
        check(lib().cf_resources_cluster_forward_create_buffers(self.handle, x, y, z, max_lights_per_cluster))

    def buffers(self) -> CfClusterForwardBuffers:
        b = CfClusterForwardBuffers()
        check(lib().cf_resources_cluster_forward_get_buffers(self.handle, C.byref(b)))
        return b

    @property
    def aabb_dirty(self) -> bool:
        v = C.c_int()
        check(lib().cf_resources_cluster_forward_is_aabb_dirty(self.handle, C.byref(v)))
        return bool(v.value)

    def read_outputs(self, stream=None, host_cells: np.ndarray | None = None, host_indices: np.ndarray | None = None):
        """Returns (cells (C, 2) uint32, indices (total,) uint32) copied to host."""
        b = self.buffers()
        cells = host_cells if host_cells is not None else np.empty((b.cluster_count, 2), np.uint32)
        idx = host_indices if host_indices is not None else np.empty(b.index_capacity, np.uint32)
        total = C.c_uint32()
        check(lib().cf_resources_cluster_forward_read_outputs(self.handle, ptr(cells), ptr(idx), idx.size,
                                                              C.byref(total), stream_handle(stream)))
        return cells, idx[: total.value]

    def read_aabbs(self) -> np.ndarray:
        """AABBs (C, 8) float32 copied to host (synchronises the device)."""
        b = self.buffers()
        return device_view(b.aabbs, (b.cluster_count, 8), "<f4").cpu().numpy()

    def close(self):
        if self.handle:
            lib().cf_resources_cluster_forward_destroy(self.handle)
            self.handle = None


class PipelineAABBGenerator:
    def __init__(self, ctx: Context, res_cf: ResourcesClusterForward):
        self.ctx, self.res = ctx, res_cf
        h = C.c_void_p()
        check(lib().cf_pipeline_aabb_generator_create(ctx.handle, res_cf.handle, C.byref(h)))
        self.handle = h

    def set_cluster_forward_ubo(self, ubo: CfClusterForwardUBO) -> None:
        check(lib().cf_pipeline_aabb_generator_set_cluster_forward_ubo(self.handle, C.byref(ubo)))

    def on_window_resized(self) -> None:
        check(lib().cf_pipeline_aabb_generator_on_window_resized(self.handle))

    def fill_command_buffer(self, stream=None) -> None:
        check(lib().cf_pipeline_aabb_generator_fill_command_buffer(self.handle, stream_handle(stream)))

    def close(self):
        if self.handle:
            lib().cf_pipeline_aabb_generator_destroy(self.handle)
            self.handle = None


class PipelineLightCulling:
    def __init__(self, ctx: Context, res_light: ResourcesLight, res_cf: ResourcesClusterForward):
        self.ctx, self.lights, self.res = ctx, res_light, res_cf
        h = C.c_void_p()
        check(lib().cf_pipeline_light_culling_create(ctx.handle, res_light.handle, res_cf.handle, C.byref(h)))
        self.handle = h

    def reset_global_index(self) -> None:
        check(lib().cf_pipeline_light_culling_reset_global_index(self.handle))

    def set_cluster_forward_ubo(self, ubo: CfClusterForwardUBO) -> None:
        check(lib().cf_pipeline_light_culling_set_cluster_forward_ubo(self.handle, C.byref(ubo)))

    def set_tuning(self, clusters_per_warp: int = 0, warps: int = 0, tile: int = 0, stages: int = 0,
                   binned: int = 0) -> None:
        """Selects a culling kernel configuration (clusters_per_warp 0 = automatic)."""
        check(lib().cf_pipeline_light_culling_set_tuning(self.handle, clusters_per_warp, warps, tile, stages, binned))

    def fill_command_buffer(self, stream=None) -> None:
        check(lib().cf_pipeline_light_culling_fill_command_buffer(self.handle, stream_handle(stream)))

    def tuning(self):
        """(clusters_per_warp, warps, tile, stages, binned) the next fill uses."""
        out = (C.c_int * 5)()
        check(lib().cf_pipeline_light_culling_get_tuning(self.handle, out))
        return tuple(out)

    def enable_stage_timing(self, enable: bool = True) -> None:
        check(lib().cf_pipeline_light_culling_enable_stage_timing(self.handle, int(enable)))

    def enable_work_counters(self, enable: bool = True) -> None:
        check(lib().cf_pipeline_light_culling_enable_work_counters(self.handle, int(enable)))

    def read_work_counters(self):
        """(slab/union-box tests, cluster-box tests) executed since the last read."""
        out = (C.c_uint64 * 2)()
        check(lib().cf_pipeline_light_culling_read_work_counters(self.handle, out))
        return int(out[0]), int(out[1])

    def stage_times_ms(self):
        """(light transform, culling, offset scan) of the last call, in ms."""
        ms = (C.c_float * 3)()
        check(lib().cf_pipeline_light_culling_get_stage_times(self.handle, ms))
        return tuple(float(x) for x in ms)

    def close(self):
        if self.handle:
            lib().cf_pipeline_light_culling_destroy(self.handle)
            self.handle = None


class _DeviceArray:
    """A __cuda_array_interface__ view of library-owned device memory."""

    def __init__(self, address: int, shape, typestr: str):
        self.__cuda_array_interface__ = {"shape": tuple(shape), "typestr": typestr, "data": (int(address), False),
                                         "version": 3, "strides": None}


def device_view(address: int, shape, typestr: str):
    """A torch tensor aliasing device memory at `address` (no copy, no ownership)."""
    import torch
    torch.cuda.synchronize()
    if int(np.prod(shape)) == 0:
        return torch.empty(shape, dtype={"<f4": torch.float32, "<u4": torch.int32}.get(typestr, torch.uint8), device="cuda")
    return torch.as_tensor(_DeviceArray(address, shape, typestr), device="cuda")
