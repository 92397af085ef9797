"""Shared helpers of the GPU tests: run a view through the C ABI, compare with the oracle."""
from __future__ import annotations

import ctypes as C
import hashlib

import numpy as np


def bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32)


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def run_pipeline(ctx, view, tuning=None, stream=None):
    """ResourcesLight/ResourcesClusterForward + the two pipelines, as the
    reference app drives them per frame; returns (aabbs, cells, indices)."""
    from hellovulkan_gb300.pipelines import (PipelineAABBGenerator, PipelineLightCulling, ResourcesClusterForward,
                                             ResourcesLight)
    rl = ResourcesLight(ctx)
    rl.add_lights(view.lights)
    rc = ResourcesClusterForward(ctx)
    rc.create_buffers(*view.grid, view.cap)
    gen = PipelineAABBGenerator(ctx, rc)
    gen.set_cluster_forward_ubo(view.ubo)
    gen.fill_command_buffer(stream)
    cull = PipelineLightCulling(ctx, rl, rc)
    if tuning:
        cull.set_tuning(*tuning)
    cull.reset_global_index()
    cull.set_cluster_forward_ubo(view.ubo)
    cull.fill_command_buffer(stream)
    aabbs = rc.read_aabbs()
    cells, idx = rc.read_outputs(stream)
    assert ctx.check_device_error() == 0
    for o in (cull, gen, rc, rl):
        o.close()
    return aabbs, cells, idx.copy()


def run_stateless(view, stream=None):
    """cf_generate_aabbs + cf_cull_lights on torch-owned device memory."""
    import torch
    from hellovulkan_gb300._lib import check, lib
    L = lib()
    Cn, cap = view.clusters, view.cap
    aabbs = torch.empty(Cn * 8, dtype=torch.float32, device="cuda")
    lights = torch.from_numpy(np.ascontiguousarray(view.lights)).cuda()
    cells = torch.empty(Cn * 2, dtype=torch.int32, device="cuda")
    idx = torch.empty(Cn * cap, dtype=torch.int32, device="cuda")
    total = torch.zeros(1, dtype=torch.int32, device="cuda")
    n = C.c_uint64()
    check(L.cf_cull_workspace_size(C.byref(view.ubo), view.light_count, cap, C.byref(n)))
    ws = torch.zeros(n.value, dtype=torch.uint8, device="cuda")
    s = (stream or torch.cuda.current_stream()).cuda_stream
    check(L.cf_generate_aabbs(C.byref(view.ubo), aabbs.data_ptr(), s))
    check(L.cf_cull_lights(C.byref(view.ubo), aabbs.data_ptr(), lights.data_ptr() if view.light_count else None,
                           view.light_count, cap, cells.data_ptr(), idx.data_ptr(), Cn * cap, total.data_ptr(),
                           ws.data_ptr(), n.value, s))
    torch.cuda.synchronize()
    err = C.c_uint32()
    check(L.cf_cull_workspace_device_error(ws.data_ptr(), C.byref(err)))
    t = int(total.item())
    return (aabbs.cpu().numpy().reshape(Cn, 8), cells.cpu().numpy().view(np.uint32).reshape(Cn, 2),
            idx[:t].cpu().numpy().view(np.uint32).copy())


def assert_matches_oracle(oracle, view, aabbs, cells, idx):
    a = oracle.generate_aabbs(view.ubo)
    assert np.array_equal(bits(aabbs), bits(a)), "AABB bits differ in %d clusters" % int(
        (bits(aabbs) != bits(a)).any(axis=1).sum())
    oc, oi, _ = oracle.cull(view.ubo, a, view.lights, view.cap)
    if not np.array_equal(cells, oc):
        bad = np.nonzero((cells != oc).any(axis=1))[0]
        raise AssertionError("cells differ in %d clusters, first %s: gpu %s oracle %s" % (
            bad.size, bad[:5], cells[bad[:3]].tolist(), oc[bad[:3]].tolist()))
    assert np.array_equal(idx, oi), "index lists differ"
