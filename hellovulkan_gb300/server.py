"""The culling server (include/cfcull.h, cf_server_*) and its load driver.

    srv = Server(ctx, budget_bytes=8 << 30)
    sid = srv.register(lights)              # (n, 12) float32 LightData records
    rid = srv.submit(ubo, sid)
    for c in srv.poll(wait_ms=10): cells, idx = srv.read(c); srv.release(c.request_id)
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np

from . import scenes
from ._lib import (CfClusterForwardUBO, CfServeLoad, CfServeReport, CfServerCompletion, CfServerConfig,
                   CfServerRequest, CfServerStats, check, lib)


class Server:
    def __init__(self, ctx, budget_bytes: int = 8 << 30, max_batch_views: int = 64, streams: int = 4,
                 max_pending: int = 0, max_groups_per_view: int = 0):
        self.ctx = ctx
        cfg = CfServerConfig(budget_bytes, max_batch_views, streams, max_pending, max_groups_per_view)
        h = C.c_void_p()
        check(lib().cf_server_create(ctx.handle, C.byref(cfg), C.byref(h)))
        self.handle = h

    def register(self, lights: np.ndarray) -> int:
        """A new resident light set.  From pageable memory the lights are
        copied before the call returns; from pinned memory (a pinned tensor's
        numpy view) the server's worker copies them before the next batch, so
        the array must stay alive and unchanged until the first request that
        uses the set has completed."""
        a = np.ascontiguousarray(lights, np.float32).reshape(-1, 12)
        out = C.c_uint64()
        check(lib().cf_server_register_light_set(self.handle, a.ctypes.data if a.size else None, a.shape[0],
                                                 C.byref(out)))
        return int(out.value)

    def update(self, set_id: int, lights: np.ndarray) -> None:
        """A new version of a set for requests submitted from now on (the
        same rule on pinned memory as register)."""
        a = np.ascontiguousarray(lights, np.float32).reshape(-1, 12)
        check(lib().cf_server_update_light_set(self.handle, set_id, a.ctypes.data if a.size else None, a.shape[0]))

    def jitter(self, set_id: int, seed: int, sigma: float) -> None:
        check(lib().cf_server_jitter_light_set(self.handle, set_id, seed, sigma))

    def release_set(self, set_id: int) -> None:
        check(lib().cf_server_release_light_set(self.handle, set_id))

    def resident(self, set_id: int) -> bool:
        v = C.c_int()
        check(lib().cf_server_is_light_set_resident(self.handle, set_id, C.byref(v)))
        return bool(v.value)

    def submit(self, ubo: CfClusterForwardUBO, set_id: int, tag: int = 0, cap: int = 150) -> int:
        r = CfServerRequest()
        r.ubo = ubo
        r.light_set = set_id
        r.user_tag = tag
        r.max_lights_per_cluster = cap
        out = C.c_uint64()
        check(lib().cf_server_submit(self.handle, C.byref(r), C.byref(out)))
        return int(out.value)

    def poll(self, max_count: int = 1024, wait_ms: int = 0):
        buf = (CfServerCompletion * max_count)()
        n = C.c_uint32()
        check(lib().cf_server_poll(self.handle, buf, max_count, C.byref(n), wait_ms))
        return [buf[i] for i in range(n.value)]

    def wait_all(self, count: int, timeout_s: float = 60.0):
        import time
        out, t0 = [], time.time()
        while len(out) < count and time.time() - t0 < timeout_s:
            out += self.poll(wait_ms=5)
        return out

    def release(self, request_id: int) -> None:
        check(lib().cf_server_release(self.handle, request_id))

    def declare_pinned(self, arr) -> None:
        """Declares a pinned host array (a pinned tensor or its numpy view) for
        the server's lifetime: registers and updates from it make no CUDA
        call.  The server object keeps a reference to it."""
        a = arr.numpy() if hasattr(arr, "numpy") else arr
        check(lib().cf_server_declare_pinned_host(self.handle, a.ctypes.data, a.nbytes))
        self._keep_alive = getattr(self, "_keep_alive", []) + [arr]

    def release_many(self, request_ids) -> None:
        """release() for many requests under one acquisition of the server's lock."""
        ids = (C.c_uint64 * len(request_ids))(*request_ids)
        check(lib().cf_server_release_many(self.handle, C.cast(ids, C.c_void_p), len(request_ids)))

    def read(self, c: CfServerCompletion, cap: int = 150):
        """(cells (C,2) uint32, indices (total,) uint32) of a successful completion."""
        from .pipelines import device_view
        total = int(device_view(c.d_total, (1,), "<u4").cpu().numpy().view(np.uint32)[0])
        cells = device_view(c.d_cells, (c.clusters, 2), "<u4").cpu().numpy().view(np.uint32).copy()
        idx = device_view(c.d_indices, (max(total, 1),), "<u4").cpu().numpy().view(np.uint32)[:total].copy()
        return cells, idx

    def stats(self) -> dict:
        s = CfServerStats()
        check(lib().cf_server_get_stats(self.handle, C.byref(s)))
        return {n: getattr(s, n) for n, _ in CfServerStats._fields_ if not n.startswith("_")}

    def close(self):
        if self.handle:
            lib().cf_server_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def projection_ubos():
    """The four projections of the served mix (grid, resolution, fovY 45 deg, near 0.1, far 2000)."""
    out = []
    for g in scenes.GRIDS:
        t = scenes.TILE_PX[g]
        out.append(scenes.custom_view(g, g[0] * t, g[1] * t, 0.1, 2000.0).ubo)
    return out


def _pin(arrays):
    """Page-locked copies of the arrays (torch tensors, kept by the caller), or None without CUDA."""
    try:
        import torch
        if not torch.cuda.is_available():
            return None
        return [torch.from_numpy(a).pin_memory() for a in arrays]
    except ImportError:
        return None


def run_load(server: Server, rate: float, duration: float, seed: int = 4, base_sets=None, p_reuse: float = 0.7,
             sigma: float = 0.1, recent_sets: int = 256, submit_threads: int = 2) -> dict:
    """cf_serve_run_load with the served mix's distributions: base light sets
    drawn like the batch mix (256..65536 blob lights), cameras uniform in
    [-80,80]x[2,40]x[-80,80] looking at targets in [-20,20]^3."""
    if base_sets is None:
        rng = np.random.default_rng(seed)
        base_sets = [scenes.blob_lights(rng, int(round(math.exp(rng.uniform(math.log(256), math.log(65536))))))
                     for _ in range(128)]
    # pinned, as a server keeps the data it registers from: the uploads are then
    # asynchronous copies rather than staged ones (the sets outlive the run)
    base_sets = [np.ascontiguousarray(b, np.float32) for b in base_sets]
    pinned = _pin(base_sets)
    if pinned is not None:
        base_sets = [t.numpy() for t in pinned]
        # the server may still copy from them after the run (a set registered
        # by a request that failed is copied when the worker is next idle)
        server._keep_alive = getattr(server, "_keep_alive", []) + [pinned]
    projs = (CfClusterForwardUBO * 4)(*projection_ubos())
    ptrs = (C.c_void_p * len(base_sets))(*[b.ctypes.data for b in base_sets])
    counts = (C.c_uint32 * len(base_sets))(*[b.shape[0] for b in base_sets])
    ld = CfServeLoad()
    ld.rate_per_s, ld.duration_s, ld.p_reuse, ld.seed = rate, duration, p_reuse, seed
    ld.jitter_sigma, ld.recent_sets, ld.submit_threads, ld.max_lights_per_cluster = sigma, recent_sets, submit_threads, 150
    ld.n_projections, ld.n_base_sets = 4, len(base_sets)
    ld.projections = C.cast(projs, C.c_void_p)
    ld.base_sets = C.cast(ptrs, C.c_void_p)
    ld.base_counts = C.cast(counts, C.c_void_p)
    ld.eye_lo[:], ld.eye_hi[:] = [-80, 2, -80], [80, 40, 80]
    ld.target_lo[:], ld.target_hi[:] = [-20, -20, -20], [20, 20, 20]
    rep = CfServeReport()
    check(lib().cf_serve_run_load(server.handle, C.byref(ld), C.byref(rep)))
    out = {n: getattr(rep, n) for n, _ in CfServeReport._fields_}
    out["views_per_s"] = out["achieved_rate"]
    out["tests_per_s"] = out["tests_brute_force"] / max(out["wall_s"], 1e-9)
    return out
