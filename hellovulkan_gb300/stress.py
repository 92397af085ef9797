"""Animated many-view culling: the stress workload over the C ABI.

Every frame moves every light of every view one step along its orbit on the
device (cf_animate_light_orbits, in place) and culls all views in one batched
pass (cf_batch_cull, a CUDA-graph replay).  Every `frames_per_projection`
frames the projection of every view changes (its grid flips between 16x9x24
and 32x18x48 and fovY between 45 and 60 degrees): the batch is re-planned
(cf_batch_set_views) and the AABBs of all views are regenerated in one launch
(cf_batch_generate_aabbs).

Device layout: the lights of all views in one (views * lights, 12) float32
buffer and their orbits in one (views * lights, 8) buffer; the outputs in two
pools, one per grid, of views / 2 slots each.  In epoch e view i writes slot
i // 2 of pool (i + e) % 2, so exactly half of the views use each grid in
every epoch and neither pool changes size.
"""
from __future__ import annotations

import time

import numpy as np

from . import scenes
from ._lib import CfBatchView, check, lib, stream_handle
from .batch import Batch


def stress_device_bytes(n_views: int, n_lights: int, cap: int = 150) -> int:
    """Device memory the stress workload holds outside the batch's workspace."""
    per_slot = [c * (32 + 8 + 4 * cap) + 4 for c in (int(np.prod(g)) for g in scenes.STRESS_GRIDS)]
    return n_views * n_lights * (48 + 32) + (n_views // 2) * sum(per_slot)


class StressAnimation:
    def __init__(self, ctx, n_views: int = 4096, n_lights: int = 4096, seed: int = 5,
                 frames_per_projection: int = 60, cap: int = 150):
        import torch
        if n_views < 2 or n_views % 2:
            raise ValueError("an even number of views is needed (half on each grid)")
        self.ctx, self.n_views, self.n_lights, self.cap = ctx, n_views, n_lights, cap
        self.frames_per_projection = frames_per_projection
        rng = np.random.default_rng(seed)
        self.cameras = [scenes.random_camera(rng) for _ in range(n_views)]
        lights, orbits = scenes.orbit_lights(rng, n_views, n_lights)
        self.h_orbits0 = orbits  # frame-0 orbit state, for the checks
        self.d_lights = torch.from_numpy(lights).cuda()
        self.d_orbits = torch.from_numpy(orbits).cuda()
        del lights
        slots = n_views // 2
        self.pools = []
        for g in scenes.STRESS_GRIDS:
            c = int(np.prod(g))
            self.pools.append({
                "clusters": c,
                "aabbs": torch.empty((slots, c * 8), dtype=torch.float32, device="cuda"),
                "cells": torch.empty((slots, c * 2), dtype=torch.int32, device="cuda"),
                "indices": torch.empty((slots, c * cap), dtype=torch.int32, device="cuda"),
                "totals": torch.zeros(slots, dtype=torch.int32, device="cuda"),
            })
        self.batch = Batch(ctx)
        self.epoch = -1
        self.ubos = []
        self.frame_index = 0

    # -- layout ---------------------------------------------------------------
    def slot(self, view: int, epoch: int | None = None):
        e = self.epoch if epoch is None else epoch
        return self.pools[(view + e) % 2], view // 2

    def set_epoch(self, epoch: int, stream=None) -> None:
        """Re-plans the batch for the projections of `epoch` and regenerates
        every view's AABBs (one launch on `stream`)."""
        self.plan_epoch(epoch)
        self.batch.generate_aabbs(stream)

    def plan_epoch(self, epoch: int) -> None:
        """Points the batch at the projections and output slots of `epoch`
        (host work; synchronous)."""
        L = self.n_lights
        views, ubos = [], []
        lp = self.d_lights.data_ptr()
        for i in range(self.n_views):
            ubo = scenes.stress_ubo(i, epoch, self.cameras[i])
            pool, s = self.slot(i, epoch)
            bv = CfBatchView()
            bv.ubo = ubo
            bv.d_lights = lp + i * L * 48
            bv.d_aabbs = pool["aabbs"][s].data_ptr()
            bv.d_cells = pool["cells"][s].data_ptr()
            bv.d_indices = pool["indices"][s].data_ptr()
            bv.d_total = pool["totals"][s:s + 1].data_ptr()
            bv.index_capacity = pool["clusters"] * self.cap
            bv.light_count = L
            bv.max_lights_per_cluster = self.cap
            views.append(bv)
            ubos.append(ubo)
        self.batch.set_views(views)
        self.epoch, self.ubos = epoch, ubos

    def animate(self, frames: int = 1, stream=None) -> None:
        check(lib().cf_animate_light_orbits(self.d_lights.data_ptr(), self.d_orbits.data_ptr(),
                                            self.n_views * self.n_lights, frames, stream_handle(stream)))

    def tests_per_frame(self) -> int:
        return sum(int(np.prod(scenes.STRESS_GRIDS[(i + max(self.epoch, 0)) % 2])) for i in range(self.n_views)) * \
            self.n_lights

    # -- state for checking -------------------------------------------------
    def view_state(self, view: int) -> dict:
        """View `view` at the current frame, read back to the host: its
        lights, the orbits it started from, its AABBs, cells and index list,
        its UBO and cap.  A checker (the tests, the benchmark) compares them
        with a host restatement; this package only reads them."""
        import torch
        torch.cuda.synchronize()
        L = self.n_lights
        pool, s = self.slot(view)
        c = pool["clusters"]
        total = int(pool["totals"][s].item())
        return {"frame": self.frame_index, "view": view,
                "lights": self.d_lights[view * L:(view + 1) * L].cpu().numpy(),
                "orbits0": self.h_orbits0[view * L:(view + 1) * L],
                "aabbs": pool["aabbs"][s].cpu().numpy().reshape(c, 8),
                "cells": pool["cells"][s].cpu().numpy().view(np.uint32).reshape(c, 2),
                "indices": pool["indices"][s][:total].cpu().numpy().view(np.uint32),
                "ubo": self.ubos[view], "cap": self.cap}

    # -- the run --------------------------------------------------------------
    def run(self, frames: int, stream, check_frames=(), check_views=(), check=None, autotune: bool = True) -> dict:
        """`frames` frames from frame 0: each frame animates one step, then
        culls every view; a new projection epoch starts every
        frames_per_projection frames.  Every frame is timed with CUDA events on
        `stream`: the frames that start an epoch include the AABB
        regeneration and the capture of the re-planned pass into a CUDA graph;
        the host-side re-planning before them is timed apart.  With `check`
        (a callable taking view_state(v) and returning a dict of booleans
        "lights", "aabbs", "cells", "indices"), the views in check_views are
        checked after the frames in check_frames."""
        import torch
        ev = [[torch.cuda.Event(enable_timing=True) for _ in range(3)] for _ in range(frames)]
        plan_ms, checks, tests = [], [], 0
        self.frame_index = 0
        for f in range(frames):
            if f % self.frames_per_projection == 0:
                # the re-plan waits for the frames already queued; drain them first so
                # that the time below is the host's own planning work
                stream.synchronize()
                t0 = time.perf_counter()
                self.plan_epoch(f // self.frames_per_projection)
                plan_ms.append(1e3 * (time.perf_counter() - t0))
                if autotune and f == 0:  # untimed: culls frame 0's inputs with each candidate
                    self.batch.generate_aabbs(stream)
                    self.batch.autotune(2, stream)
                ev[f][0].record(stream)
                self.batch.generate_aabbs(stream)
            else:
                ev[f][0].record(stream)
            self.animate(1, stream)
            self.frame_index += 1
            ev[f][1].record(stream)
            self.batch.cull(stream)
            ev[f][2].record(stream)
            tests += self.tests_per_frame()
            if check is not None and f in check_frames:
                for v in check_views:
                    checks.append(check(self.view_state(v)))
        torch.cuda.synchronize()
        frame_ms = np.array([a.elapsed_time(c) for a, _, c in ev])
        anim_ms = np.array([a.elapsed_time(b) for a, b, _ in ev])
        cull_ms = np.array([b.elapsed_time(c) for _, b, c in ev])
        steady = [f for f in range(frames) if f % self.frames_per_projection]
        total_s = float(frame_ms.sum()) * 1e-3
        slowest = np.argsort(frame_ms)[::-1][:5]
        return {
            "frames": frames, "views": self.n_views, "lights_per_view": self.n_lights,
            "frames_per_projection": self.frames_per_projection,
            "ms_per_frame": float(frame_ms.mean()), "ms_per_frame_p50": float(np.median(frame_ms)),
            "ms_per_frame_max": float(frame_ms.max()),
            "ms_per_frame_steady": float(frame_ms[steady].mean()) if steady else None,
            "animate_ms_per_frame": float(anim_ms[steady].mean()) if steady else float(anim_ms.mean()),
            "cull_ms_per_frame": float(cull_ms[steady].mean()) if steady else float(cull_ms.mean()),
            "projection_frame_ms": [float(frame_ms[f]) for f in range(0, frames, self.frames_per_projection)],
            "replan_host_ms": plan_ms,
            "slowest_frames": [[int(f), float(frame_ms[f])] for f in slowest],
            "device_error": self.ctx.check_device_error(),
            "views_per_s": self.n_views * frames / total_s, "tests_per_s": tests / total_s,
            "checks": checks, "parity": all(all(c[k] for k in ("lights", "aabbs", "cells", "indices"))
                                            for c in checks) if checks else None,
            "batch": self.batch.info(),
        }

    def close(self):
        self.batch.close()
