"""ctypes binding of libcfcull.so (include/cfcull.h).

The library is the product: when it is missing this module raises instead of
falling back to anything else.
"""
from __future__ import annotations

import ctypes as C
import re
from pathlib import Path

import numpy as np

PKG = Path(__file__).resolve().parent
REPO = PKG.parent
LIB_PATH = PKG / "libcfcull.so"
HEADERS = [REPO / "include" / "cfcull.h"]


class CfLightData(C.Structure):
    _fields_ = [("position", C.c_float * 4), ("color", C.c_float * 4), ("radius", C.c_float), ("_pad", C.c_float * 3)]


class CfAABB(C.Structure):
    _fields_ = [("minPoint", C.c_float * 4), ("maxPoint", C.c_float * 4)]


class CfLightCell(C.Structure):
    _fields_ = [("offset", C.c_uint32), ("count", C.c_uint32)]


class CfLightOrbit(C.Structure):
    _fields_ = [("offset", C.c_float * 2), ("rot", C.c_float * 2), ("center", C.c_float * 4)]


class CfFragmentSample(C.Structure):
    _fields_ = [(n, C.c_uint32) for n in ("cluster", "offset", "count", "covering", "missing", "flags")] + [
        ("view_z", C.c_float), ("linear_depth", C.c_float)]


FRAGMENT_DTYPE = np.dtype([("cluster", "<u4"), ("offset", "<u4"), ("count", "<u4"), ("covering", "<u4"),
                           ("missing", "<u4"), ("flags", "<u4"), ("view_z", "<f4"), ("linear_depth", "<f4")])
FRAGMENT_OUTSIDE_GRID, FRAGMENT_OUTSIDE_AABB, FRAGMENT_CAPPED, FRAGMENT_BAD_CELL = 1, 2, 4, 8


class CfPBRPushConstant(C.Structure):
    _fields_ = [(n, C.c_float) for n in ("lightIntensity", "baseReflectivity", "maxReflectionLod", "lightFalloff",
                                         "albedoMultipler")]


class CfFrustum(C.Structure):
    _fields_ = [("planes", (C.c_float * 4) * 6), ("corners", (C.c_float * 4) * 8)]


class CfClusterForwardUBO(C.Structure):
    _fields_ = [
        ("cameraInverseProjection", C.c_float * 16),
        ("cameraView", C.c_float * 16),
        ("screenSize", C.c_float * 2),
        ("sliceScaling", C.c_float),
        ("sliceBias", C.c_float),
        ("cameraNear", C.c_float),
        ("cameraFar", C.c_float),
        ("sliceCountX", C.c_uint32),
        ("sliceCountY", C.c_uint32),
        ("sliceCountZ", C.c_uint32),
        ("_pad", C.c_uint32 * 3),
    ]


class CfClusterForwardBuffers(C.Structure):
    _fields_ = [
        ("aabbs", C.c_void_p),
        ("light_cells", C.c_void_p),
        ("light_indices", C.c_void_p),
        ("total_indices", C.c_void_p),
        ("cluster_count", C.c_uint32),
        ("max_lights_per_cluster", C.c_uint32),
        ("index_capacity", C.c_uint64),
    ]


class CfBatchView(C.Structure):
    _fields_ = [
        ("ubo", CfClusterForwardUBO),
        ("d_lights", C.c_void_p),
        ("d_aabbs", C.c_void_p),
        ("d_cells", C.c_void_p),
        ("d_indices", C.c_void_p),
        ("d_total", C.c_void_p),
        ("index_capacity", C.c_uint64),
        ("light_count", C.c_uint32),
        ("max_lights_per_cluster", C.c_uint32),
        ("_pad", C.c_uint32 * 2),
    ]


class CfBatchInfo(C.Structure):
    _fields_ = [
        ("views", C.c_uint32), ("items", C.c_uint32), ("buckets", C.c_uint32), ("_pad", C.c_uint32),
        ("workspace_bytes", C.c_uint64),
        ("bucket_slice_clusters", C.c_uint32 * 8),
        ("bucket_config", (C.c_int32 * 4) * 8),
        ("bucket_ctas", C.c_int32 * 8),
    ]


class CfServerConfig(C.Structure):
    _fields_ = [("hbm_budget_bytes", C.c_uint64), ("max_batch_views", C.c_uint32), ("streams", C.c_uint32),
                ("max_pending", C.c_uint32), ("max_groups_per_view", C.c_uint32)]


class CfServerRequest(C.Structure):
    _fields_ = [("ubo", CfClusterForwardUBO), ("light_set", C.c_uint64), ("user_tag", C.c_uint64),
                ("max_lights_per_cluster", C.c_uint32), ("_pad", C.c_uint32 * 3)]


class CfServerCompletion(C.Structure):
    _fields_ = [("request_id", C.c_uint64), ("user_tag", C.c_uint64), ("status", C.c_int32),
                ("clusters", C.c_uint32), ("t_submit", C.c_double), ("t_launch", C.c_double),
                ("t_complete", C.c_double), ("d_cells", C.c_void_p), ("d_indices", C.c_void_p),
                ("d_total", C.c_void_p)]


class CfServerStats(C.Structure):
    _fields_ = [(n, C.c_uint64) for n in ("submitted", "completed", "batches", "views_launched", "max_pending",
                                          "evictions", "arena_bytes", "arena_used_bytes", "arena_peak_bytes",
                                          "pending", "resident_light_sets", "resident_projections")] + [
        ("max_batch_views", C.c_uint32), ("max_held_outputs", C.c_uint32)]


class CfServeLoad(C.Structure):
    _fields_ = [("rate_per_s", C.c_double), ("duration_s", C.c_double), ("p_reuse", C.c_double),
                ("seed", C.c_uint64), ("jitter_sigma", C.c_float), ("recent_sets", C.c_uint32),
                ("submit_threads", C.c_uint32), ("max_lights_per_cluster", C.c_uint32),
                ("n_projections", C.c_uint32), ("n_base_sets", C.c_uint32),
                ("projections", C.c_void_p), ("base_sets", C.c_void_p), ("base_counts", C.c_void_p),
                ("eye_lo", C.c_float * 3), ("eye_hi", C.c_float * 3), ("target_lo", C.c_float * 3),
                ("target_hi", C.c_float * 3)]


class CfServeReport(C.Structure):
    _fields_ = [(n, C.c_uint64) for n in ("scheduled", "submitted", "completed", "failed", "new_sets",
                                          "reused_sets", "tests_brute_force")] + [
        (n, C.c_double) for n in ("wall_s", "offered_rate", "achieved_rate", "latency_p50_ms", "latency_p90_ms",
                                  "latency_p99_ms", "latency_p999_ms", "latency_max_ms", "queue_p50_ms",
                                  "queue_p99_ms", "submit_lag_p99_ms", "exec_p50_ms", "exec_p99_ms",
                                  "register_call_p50_us", "register_call_p99_us", "jitter_call_p50_us",
                                  "jitter_call_p99_us", "submit_call_p50_us", "submit_call_p99_us",
                                  "register_call_max_us", "jitter_call_max_us", "submit_call_max_us",
                                  "worst_lag_arrival_s")]


assert C.sizeof(CfServerConfig) == 24 and C.sizeof(CfServerRequest) == 208
assert C.sizeof(CfServerCompletion) == 72 and C.sizeof(CfServerStats) == 104
assert C.sizeof(CfServeLoad) == 128 and C.sizeof(CfServeReport) == 240
assert CfServeLoad.projections.offset == 56 and CfServeLoad.eye_lo.offset == 80
assert C.sizeof(CfBatchView) == 240 and C.sizeof(CfBatchInfo) == 216
assert C.sizeof(CfLightData) == 48 and C.sizeof(CfAABB) == 32 and C.sizeof(CfLightCell) == 8
assert C.sizeof(CfPBRPushConstant) == 20 and C.sizeof(CfFrustum) == 224
assert C.sizeof(CfLightOrbit) == 32 and C.sizeof(CfFragmentSample) == 32 == FRAGMENT_DTYPE.itemsize
assert C.sizeof(CfClusterForwardUBO) == 176

STATUS = {
    0: "CF_SUCCESS", 1: "CF_ERROR_INVALID_ARGUMENT", 2: "CF_ERROR_OUT_OF_MEMORY", 3: "CF_ERROR_CUDA",
    4: "CF_ERROR_CAPACITY", 5: "CF_ERROR_NOT_READY", 6: "CF_ERROR_DEVICE_TIMEOUT", 7: "CF_ERROR_BUDGET",
    8: "CF_ERROR_UNSUPPORTED",
}


class CfError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__("%s (%d): %s" % (STATUS.get(status, "?"), status, message))
        self.status = status


_P = C.c_void_p
_U32 = C.c_uint32
_U64 = C.c_uint64
_PU32 = C.POINTER(C.c_uint32)
_PU64 = C.POINTER(C.c_uint64)
_I = C.c_int

# name -> argtypes; every function returns int (CfStatus) unless listed in _RESTYPE
_SIGS = {
    "cf_status_string": [_I],
    "cf_last_error_message": [],
    "cf_version": [],
    "cf_context_create": [_I, C.POINTER(_P)],
    "cf_context_destroy": [_P],
    "cf_context_check_device_error": [_P, _PU32],
    "cf_resources_light_create": [_P, C.POINTER(_P)],
    "cf_resources_light_destroy": [_P],
    "cf_resources_light_add_lights": [_P, _P, _U32],
    "cf_resources_light_upload_async": [_P, _P, _U32, _P],
    "cf_resources_light_update_light_position": [_P, _U32, C.POINTER(C.c_float)],
    "cf_resources_light_get_light_count": [_P, _PU32],
    "cf_resources_light_get_device_buffer": [_P, C.POINTER(_P)],
    "cf_resources_cluster_forward_create": [_P, C.POINTER(_P)],
    "cf_resources_cluster_forward_destroy": [_P],
    "cf_resources_cluster_forward_create_buffers": [_P, _U32, _U32, _U32, _U32],
    "cf_resources_cluster_forward_get_buffers": [_P, C.POINTER(CfClusterForwardBuffers)],
    "cf_resources_cluster_forward_is_aabb_dirty": [_P, C.POINTER(_I)],
    "cf_resources_cluster_forward_read_outputs": [_P, _P, _P, _U64, _PU32, _P],
    "cf_pipeline_aabb_generator_create": [_P, _P, C.POINTER(_P)],
    "cf_pipeline_aabb_generator_destroy": [_P],
    "cf_pipeline_aabb_generator_set_cluster_forward_ubo": [_P, C.POINTER(CfClusterForwardUBO)],
    "cf_pipeline_aabb_generator_on_window_resized": [_P],
    "cf_pipeline_aabb_generator_fill_command_buffer": [_P, _P],
    "cf_pipeline_light_culling_create": [_P, _P, _P, C.POINTER(_P)],
    "cf_pipeline_light_culling_destroy": [_P],
    "cf_pipeline_light_culling_reset_global_index": [_P],
    "cf_pipeline_light_culling_set_cluster_forward_ubo": [_P, C.POINTER(CfClusterForwardUBO)],
    "cf_pipeline_light_culling_fill_command_buffer": [_P, _P],
    "cf_pipeline_light_culling_set_tuning": [_P, _I, _I, _I, _I, _I],
    "cf_pipeline_light_culling_get_tuning": [_P, C.POINTER(_I)],
    "cf_pipeline_light_culling_enable_stage_timing": [_P, _I],
    "cf_pipeline_light_culling_get_stage_times": [_P, C.POINTER(C.c_float)],
    "cf_pipeline_light_culling_enable_work_counters": [_P, _I],
    "cf_pipeline_light_culling_read_work_counters": [_P, _PU64],
    "cf_cull_workspace_size": [C.POINTER(CfClusterForwardUBO), _U32, _U32, _PU64],
    "cf_generate_aabbs": [C.POINTER(CfClusterForwardUBO), _P, _P],
    "cf_animate_light_orbits": [_P, _P, _U64, _U32, _P],
    "cf_shade_clusters": [C.POINTER(CfClusterForwardUBO), C.POINTER(C.c_float), C.POINTER(CfPBRPushConstant), _P, _U32,
                          _U32, _P, _P, _U64, _P, _U32, _P, _P],
    "cf_frustum_cull": [C.POINTER(CfFrustum), _P, _U32, _P, _P, _P],
    "cf_lookup_clusters": [C.POINTER(CfClusterForwardUBO), _P, _U32, _U32, _P, _P, _U64, _P, _U32, _U32, _P, _I, _P,
                           _P],
    "cf_cull_lights": [C.POINTER(CfClusterForwardUBO), _P, _P, _U32, _U32, _P, _P, _U64, _P, _P, _U64, _P],
    "cf_cull_workspace_device_error": [_P, _PU32],
    "cf_cull_lights_static_scratch": [C.POINTER(CfClusterForwardUBO), _P, _P, _U32, _U32, _P, _P, _U64, _P, _P, _P],
    "cf_testing_set_wait_limit_ns": [_U64],
    "cf_testing_inject_stall": [_U32],
    "cf_testing_fail_allocation_after": [C.c_int32],
    "cf_testing_fail_version_writes": [C.c_int32],
    "cf_batch_create": [_P, C.POINTER(_P)],
    "cf_batch_destroy": [_P],
    "cf_batch_set_views": [_P, C.POINTER(CfBatchView), _U32],
    "cf_batch_update_view_matrices": [_P, C.POINTER(CfClusterForwardUBO), _U32, _P],
    "cf_batch_generate_aabbs": [_P, _P],
    "cf_batch_cull": [_P, _P],
    "cf_batch_set_graph": [_P, _I],
    "cf_batch_set_tuning": [_P, _U32, _I, _I, _I, _I],
    "cf_batch_autotune": [_P, _I, _P],
    "cf_batch_get_info": [_P, C.POINTER(CfBatchInfo)],
    "cf_server_create": [_P, C.POINTER(CfServerConfig), C.POINTER(_P)],
    "cf_server_destroy": [_P],
    "cf_server_register_light_set": [_P, _P, _U32, _PU64],
    "cf_server_update_light_set": [_P, _U64, _P, _U32],
    "cf_server_jitter_light_set": [_P, _U64, _U64, C.c_float],
    "cf_server_release_light_set": [_P, _U64],
    "cf_server_is_light_set_resident": [_P, _U64, C.POINTER(_I)],
    "cf_server_submit": [_P, C.POINTER(CfServerRequest), _PU64],
    "cf_server_poll": [_P, C.POINTER(CfServerCompletion), _U32, _PU32, _I],
    "cf_server_release": [_P, _U64],
    "cf_server_release_many": [_P, C.c_void_p, C.c_uint32],
    "cf_server_declare_pinned_host": [_P, C.c_void_p, C.c_size_t],
    "cf_server_set_tuning": [_P, _U32, _I, _I, _I, _I],
    "cf_server_get_stats": [_P, C.POINTER(CfServerStats)],
    "cf_serve_run_load": [_P, C.POINTER(CfServeLoad), C.POINTER(CfServeReport)],
}
_RESTYPE = {"cf_status_string": C.c_char_p, "cf_last_error_message": C.c_char_p}

_lib = None


def declared_symbols():
    """Names declared with CFCULL_API in include/*.h."""
    names = []
    for h in sorted((REPO / "include").glob("*.h")):
        for m in re.finditer(r"CFCULL_API\s+[\w\s\*]+?\b(cf_\w+)\s*\(", h.read_text()):
            names.append(m.group(1))
    return names


def lib():
    """The loaded library; raises if it was not built."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise ImportError(
                "libcfcull.so is not built (%s); run `python -m hellovulkan_gb300.build` "
                "or __graft_entry__.build()" % LIB_PATH)
        L = C.CDLL(str(LIB_PATH))
        for name, args in _SIGS.items():
            f = getattr(L, name)
            f.argtypes = args
            f.restype = _RESTYPE.get(name, C.c_int)
        _lib = L
    return _lib


def check(status: int) -> None:
    if status != 0:
        raise CfError(status, lib().cf_last_error_message().decode(errors="replace"))


def ptr(x) -> int | None:
    """Address of a torch tensor, a numpy array or an int address."""
    if x is None:
        return None
    if isinstance(x, int):
        return x
    if hasattr(x, "data_ptr"):
        return x.data_ptr()
    if isinstance(x, np.ndarray):
        return x.ctypes.data
    raise TypeError("cannot take the address of %r" % type(x))


def stream_handle(stream) -> int | None:
    if stream is None:
        return None
    if isinstance(stream, int):
        return stream
    return stream.cuda_stream
