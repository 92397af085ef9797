#!/usr/bin/env python
"""Benchmark of the clustered-forward light-culling path on one GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload plain_large|plain_small]

A step is one culling pass over one view: light transform, sphere-AABB
culling and the offset scan (the per-frame work of PipelineLightCulling; the
AABBs are generated once per projection, as the reference's dirty flag does).
The default workload is the 2560x1600, 32x18x48-cluster view with 16384
lights in Gaussian blobs.  The metric is light-cluster tests per second
counted brute force (clusters x lights per view); views/s is the same rate
per view.

ours       value: device-resident inputs, each step timed with CUDA events on
           the launching stream, L2 flushed (256 MiB write) between steps.
           e2e:   the same step through the C ABI with host buffers: pinned
           LightData upload, the pipeline call, and the LightCell + index
           read-back into pinned memory, timed on the host clock, with two
           pipelines in flight (and with one, reported beside it).
           roofline: the culling kernel's own event-timed duration against the
           FP32 issue rate (16 ops per executed test).
           cpu_baseline: the reference's LightCulling.comp compiled as C++
           (or the oracle port where that is unavailable) on all host cores.
reference  the same CPU implementation alone, timed per step on a bounded
           sample (a run of depth slices) of the same view.
"""
from __future__ import annotations

import argparse
import json
import os
import platform
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

REPO = Path(__file__).resolve().parent
sys.path.insert(0, str(REPO))

import numpy as np  # noqa: E402

METRIC = "light-cluster tests/s"
UNIT = "tests/s"
OPS_PER_TEST = 16
L2_FLUSH_BYTES = 256 << 20
FP32_LANES_PER_SM = 128
REF_BUDGET_S = 150.0  # the reference arm's whole run stays within this
PLAIN_SMALL = (1, 8, 512, 4, 0)  # brute-force culling configurations
PLAIN_LARGE = (2, 8, 512, 4, 0)


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=1000)
    p.add_argument("--warmup", type=int, default=10)
    p.add_argument("--impl", choices=["ours", "reference"], default="ours")
    p.add_argument("--workload", choices=["plain_large", "plain_small"], default="plain_large")
    p.add_argument("--tuning", type=str, default="", help="K,warps,tile,stages,binned of the culling kernel")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-batch", action="store_true", help="skip the 256-view batched measurement")
    p.add_argument("--no-serve", action="store_true", help="skip the served-stream measurement")
    p.add_argument("--serve-seconds", type=float, default=10.0, help="length of each served-stream run")
    p.add_argument("--no-stress", action="store_true", help="skip the animated many-view measurement")
    p.add_argument("--stress-views", type=int, default=4096)
    p.add_argument("--stress-lights", type=int, default=4096)
    p.add_argument("--stress-frames", type=int, default=600)
    p.add_argument("--cpu-seconds", type=float, default=12.0, help="CPU baseline budget")
    p.add_argument("--e2e-in-flight", type=int, default=2, help="pipelines (frames) in flight in the e2e loop")
    return p.parse_args()


def make_view(name: str, rank: int):
    from hellovulkan_gb300 import scenes
    if name == "plain_small":
        return scenes.plain_small(1 + 1000 * rank)
    return scenes.plain_large(2 + 1000 * rank)


def workload_config(view, name):
    """The workload only (the same dict in both arms); how it is measured
    goes under the line's "measurement" key."""
    x, y, z = view.grid
    w, h = view.ubo.screenSize
    return {"workload": "%s: %dx%d, grid %dx%dx%d = %d clusters, %d lights, cap %d" % (
        name, w, h, x, y, z, view.clusters, view.light_count, view.cap),
        "clusters": view.clusters, "lights": view.light_count, "cap": view.cap,
        "tests_per_view": view.clusters * view.light_count}


def fp32_peak_tops(sm_count: int, sm_mhz: float) -> float:
    """Nominal FP32 issue rate: SMs x 128 lanes x SM clock, in Tops/s."""
    return sm_count * FP32_LANES_PER_SM * sm_mhz * 1e6 / 1e12


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def max_over_ranks(values, device="cpu"):
    """Per-rank timings reduced to the slowest rank's (the whole job ends when
    its last replica does); the identity with one process."""
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(x) for x in values], dtype=torch.float64, device=device)
    if dist.is_available() and dist.is_initialized() and dist.get_world_size() > 1:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return [float(x) for x in t]


# --------------------------------------------------------------------------- clocks
class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 100 ms."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.file = None

    def start(self):
        try:
            self.file = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=self.file, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        self.proc.wait(timeout=5)
        self.file.flush()
        rows = [l.split(",") for l in Path(self.file.name).read_text().splitlines() if l.strip()]
        os.unlink(self.file.name)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            r = [c.strip() for c in r]
            if len(r) < 9:
                continue
            try:
                sm.append(float(r[1]))
                smax.append(float(r[2]))
            except ValueError:
                continue
            for n, v in zip(names, r[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# --------------------------------------------------------------------------- CPU side
def cpu_impl():
    """(kind, object with .cull(ubo, aabbs, lights, threads)) — the reference's
    shaders compiled as C++ when available, else the oracle port."""
    from oracle import Oracle, Reference
    ref = Reference.load()
    if ref is not None:
        return "reference", lambda ubo, a, L, cap, t: ref.cull(ubo, a, L, threads=t)
    o = Oracle()
    return "port", lambda ubo, a, L, cap, t: o.cull(ubo, a, L, cap, threads=t)[:2]


def sub_view(ubo, aabbs, k0: int, nz: int):
    """The clusters of depth slices [k0, k0+nz) as a view of their own."""
    import copy
    u = copy.copy(ubo)
    u.sliceCountZ = nz
    per = int(ubo.sliceCountX) * int(ubo.sliceCountY)
    return u, aabbs[k0 * per:(k0 + nz) * per]


def cpu_threads() -> int:
    return len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else (os.cpu_count() or 1)


def time_cpu(view, aabbs, budget_s: float, steps: int | None = None, warmup: int = 1):
    """Times the CPU implementation, each step the whole view when
    (warmup + steps) whole views fit the budget, else a run of depth slices
    sized to it; returns a dict."""
    kind, cull = cpu_impl()
    threads = cpu_threads()
    X, Y, Z = view.grid
    t0 = time.perf_counter()
    cull(view.ubo, aabbs, view.lights, view.cap, threads)  # one whole view: sizes the sample, warms the caches
    full = max(time.perf_counter() - t0, 1e-4)
    n_steps = steps if steps is not None else 5
    per_step = budget_s / max(n_steps + warmup, 1)
    nz = Z if full <= per_step else int(max(1, min(Z, per_step / (full / Z))))
    times, tests = [], 0
    for i in range(warmup + n_steps):
        k0 = (i * nz) % max(1, Z - nz + 1)
        u, a = sub_view(view.ubo, aabbs, k0, nz)
        t0 = time.perf_counter()
        cull(u, a, view.lights, view.cap, threads)
        dt = time.perf_counter() - t0
        if i >= warmup:
            times.append(dt)
            tests += X * Y * nz * view.light_count
    total = sum(times)
    return {"kind": kind, "cores": threads, "value": tests / total, "ms_per_step": 1e3 * total / len(times),
            "sample": "%d of %d depth slices (%d clusters x %d lights) per step, %d steps, %s threads" % (
                nz, Z, X * Y * nz, view.light_count, len(times), threads),
            "cpu": platform.processor() or platform.machine()}


def run_reference_arm(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    from oracle import Oracle
    view = make_view(args.workload, 0)
    aabbs = Oracle().generate_aabbs(view.ubo)
    r = time_cpu(view, aabbs, REF_BUDGET_S, steps=args.steps, warmup=args.warmup)
    cfg = workload_config(view, args.workload)
    line = {"metric": METRIC, "value": r["value"], "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": r["ms_per_step"], "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)", "impl": "reference",
            "config": cfg,
            "measurement": {"sample": r["sample"], "timing": "host clock per step, all host threads"},
            "cpu_baseline": {"value": r["value"], "unit": UNIT, "cores": r["cores"], "kind": r["kind"],
                             "sample": r["sample"]},
            "e2e": {"value": r["value"], "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# --------------------------------------------------------------------------- GPU side
def measure_batch(ctx, stream, n_views=256, passes=20, seed=3, sample_views=6):
    """The batched form on the 256-view uneven mix (grids 8x8x16 .. 32x18x48,
    256..65536 blob lights each): one pass culls every view (a CUDA-graph
    replay of the batched launches, autotuned per grid), against the same views
    culled one after another with one launch sequence per view
    (cf_cull_lights).  Inputs (lights, AABBs, outputs) exceed the L2, so no
    flush is needed between passes."""
    import ctypes as C

    import torch

    from hellovulkan_gb300 import scenes
    from hellovulkan_gb300._lib import check, lib
    from hellovulkan_gb300.batch import Batch, BatchBuffers

    views = scenes.batch_mix(seed, n_views)
    bufs = BatchBuffers(views)
    b = Batch(ctx)
    b.set_views(bufs.batch_views())
    b.generate_aabbs(stream)
    t0 = time.perf_counter()
    b.autotune(2, stream)
    tune_s = time.perf_counter() - t0

    def timed(fn, n):
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(n)]
        for s, e in ev:
            s.record(stream)
            fn()
            e.record(stream)
        torch.cuda.synchronize()
        return [s.elapsed_time(e) for s, e in ev]

    for _ in range(3):
        b.cull(stream)
    batch_ms = timed(lambda: b.cull(stream), passes)

    L = lib()
    sizes = []
    for v in views:
        nb = C.c_uint64()
        check(L.cf_cull_workspace_size(C.byref(v.ubo), v.light_count, v.cap, C.byref(nb)))
        sizes.append(nb.value)
    ws = torch.zeros(max(sizes), dtype=torch.uint8, device="cuda")
    sh = stream.cuda_stream

    def per_view_pass():
        for i, v in enumerate(views):
            check(L.cf_cull_lights(C.byref(v.ubo), bufs.aabbs[i].data_ptr(),
                                   bufs.lights[i].data_ptr() if v.light_count else None, v.light_count, v.cap,
                                   bufs.cells[i].data_ptr(), bufs.indices[i].data_ptr(), v.clusters * v.cap,
                                   bufs.totals[i].data_ptr(), ws.data_ptr(), ws.numel(), sh))

    per_view_pass()
    per_view_ms = timed(per_view_pass, 3)

    # the plain brute-force kernel (every light against every cluster), one
    # pipeline and one launch sequence per view, as the reference records one
    # LightCulling dispatch per view
    from hellovulkan_gb300.pipelines import (PipelineAABBGenerator, PipelineLightCulling, ResourcesClusterForward,
                                             ResourcesLight)
    plain = []
    for v in views:
        rl = ResourcesLight(ctx)
        rl.add_lights(v.lights)
        rc = ResourcesClusterForward(ctx)
        rc.create_buffers(*v.grid, v.cap)
        gen = PipelineAABBGenerator(ctx, rc)
        gen.set_cluster_forward_ubo(v.ubo)
        gen.fill_command_buffer(stream)
        cu = PipelineLightCulling(ctx, rl, rc)
        cu.set_cluster_forward_ubo(v.ubo)
        cu.set_tuning(*(PLAIN_SMALL if v.clusters <= 8192 else PLAIN_LARGE))
        plain.append((rl, rc, gen, cu))

    def plain_pass():
        for _, _, _, cu in plain:
            cu.fill_command_buffer(stream)

    plain_pass()
    plain_ms = timed(plain_pass, 3)
    b.cull(stream)  # leave the batch's own outputs in the buffers for the parity check
    torch.cuda.synchronize()

    from oracle import Oracle
    o = Oracle()
    order = sorted(range(n_views), key=lambda i: views[i].light_count)
    sample = sorted({order[0], order[-1], order[n_views // 2]} | set(
        np.random.default_rng(seed).choice(n_views, sample_views - 3, replace=False).tolist()))
    parity = True
    for i in sample:
        a, cells, idx = bufs.read(i)
        oa = o.generate_aabbs(views[i].ubo)
        oc, oi, _ = o.cull(views[i].ubo, oa, views[i].lights, views[i].cap)
        parity &= bool(np.array_equal(a.view(np.uint32), oa.view(np.uint32)) and np.array_equal(cells, oc)
                       and np.array_equal(idx, oi))
        pc, pi = plain[i][1].read_outputs(stream)
        parity &= bool(np.array_equal(pc, oc) and np.array_equal(pi, oi))
    for objs in plain:
        for o_ in reversed(objs):
            o_.close()
    tests = sum(v.clusters * v.light_count for v in views)
    bm, pm, plm = float(np.mean(batch_ms)), float(np.mean(per_view_ms)), float(np.mean(plain_ms))
    info = b.info()
    b.close()
    return {
        "workload": "%d views, grids {8x8x16,16x9x24,24x14x32,32x18x48}, %d..%d lights (total %d), cap 150, "
                    "seed %d" % (n_views, min(v.light_count for v in views), max(v.light_count for v in views),
                                 sum(v.light_count for v in views), seed),
        "ms_per_batch": bm, "views_per_s": n_views / (bm * 1e-3),
        "tests_per_s": tests / (bm * 1e-3),
        "per_view_launch_ms": pm, "per_view_launch_views_per_s": n_views / (pm * 1e-3),
        "speedup_vs_per_view_launch": pm / bm,
        "plain_per_view_ms": plm, "plain_per_view_views_per_s": n_views / (plm * 1e-3),
        "speedup_vs_plain_per_view": plm / bm,
        "per_view_note": "per_view_launch: cf_cull_lights (binned) once per view; plain_per_view: the brute-force "
                         "kernel through PipelineLightCulling once per view",
        "passes": passes, "graph": True, "autotune_s": tune_s, "buckets": info["bucket_configs"],
        "items": info["items"], "parity_sampled_views": parity, "sampled_views": sample,
        "l2": "inputs larger than L2 (%.0f MB of buffers), no flush" % (bufs.device_bytes / 1e6),
    }


def event_floor_ms(stream, flush, reps):
    """The same bracket as a timed step (L2 flush, start event, work, end
    event) around one 1-element torch kernel: the part of an event-timed step
    that is not the step's own kernels."""
    import torch
    tiny = torch.zeros(1, device="cuda")
    out = []
    for _ in range(reps):
        with torch.cuda.stream(stream):
            flush.zero_()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        with torch.cuda.stream(stream):
            tiny.add_(1.0)
        b.record(stream)
        torch.cuda.synchronize()
        out.append(a.elapsed_time(b))
    return float(np.median(out))


def measure_plain_small(ctx, stream, flush, steps, warmup, rank, sm_count, sm_mhz, traffic):
    """The 1920x1080, 16x9x24-cluster view with 1024 lights through
    PipelineLightCulling: one launch per view (the one-launch kernel).  Each
    step is event-timed on the launching stream with L2 flushed before it;
    event_floor_ms is the same bracket around a 1-element kernel.  The FP32
    fraction counts the reference loop's executed tests x 16 ops against the
    step, and against the step less that floor."""
    import torch

    from hellovulkan_gb300 import scenes
    from hellovulkan_gb300.pipelines import (PipelineAABBGenerator, PipelineLightCulling, ResourcesClusterForward,
                                             ResourcesLight)
    from oracle import Oracle
    v = scenes.plain_small(1 + 1000 * rank)
    rl = ResourcesLight(ctx)
    rl.add_lights(v.lights)
    rc = ResourcesClusterForward(ctx)
    rc.create_buffers(*v.grid, v.cap)
    gen = PipelineAABBGenerator(ctx, rc)
    gen.set_cluster_forward_ubo(v.ubo)
    gen.fill_command_buffer(stream)
    cu = PipelineLightCulling(ctx, rl, rc)
    cu.set_cluster_forward_ubo(v.ubo)
    tuning = cu.tuning()
    for _ in range(max(3, warmup)):
        cu.fill_command_buffer(stream)
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
    for i in range(steps):
        with torch.cuda.stream(stream):
            flush.zero_()
        starts[i].record(stream)
        cu.fill_command_buffer(stream)
        ends[i].record(stream)
    torch.cuda.synchronize()
    ms = [a.elapsed_time(b) for a, b in zip(starts, ends)]
    step_ms = float(np.mean(ms))
    floor_ms = event_floor_ms(stream, flush, max(10, min(steps, 100)))
    cells, idx = rc.read_outputs(stream)
    o = Oracle()
    oa = o.generate_aabbs(v.ubo)
    oc, oi, executed = o.cull(v.ubo, oa, v.lights, v.cap)
    parity = bool(np.array_equal(cells, oc) and np.array_equal(idx, oi))
    for obj in (cu, gen, rc, rl):
        obj.close()
    peak = fp32_peak_tops(sm_count, sm_mhz)
    ops = executed * OPS_PER_TEST
    ach = ops / (step_ms * 1e-3) / 1e12
    kernel_ms = max(step_ms - floor_ms, 1e-6)
    ach_k = ops / (kernel_ms * 1e-3) / 1e12
    kname = ("one_launch_kernel (%d clusters per CTA, %d warps)" % (tuning[0], tuning[1]) if tuning[4] == 2 else
             "cull_kernel<%d,%d,%d,%d> + transform + copy" % tuple(tuning[:4]))
    return {"workload": workload_config(v, "plain_small")["workload"],
            "tuning": list(tuning), "kernels_per_step": 1 if tuning[4] == 2 else 3,
            "ms_per_step": step_ms, "ms_per_step_min": float(np.min(ms)), "steps": steps,
            "value": v.clusters * v.light_count / (step_ms * 1e-3), "unit": UNIT,
            "views_per_s": 1e3 / step_ms, "parity_with_oracle": parity,
            "event_floor_ms": floor_ms,
            "executed_tests_per_view_reference_loop": executed,
            "roofline": {"bound": "fp32", "achieved": ach, "peak": peak, "unit": "Tops/s", "frac": ach / peak,
                         "kernel": kname, "ops_per_launch": ops, "traffic": traffic.get("one_launch_kernel"),
                         "peak_source": "nominal FP32 issue rate, %d SMs (device attribute) x %d lanes x %.0f MHz" % (
                             sm_count, FP32_LANES_PER_SM, sm_mhz),
                         "note": "executed tests x 16 ops over the event-timed step (one launch)"},
            "roofline_less_event_floor": {"achieved": ach_k, "frac": ach_k / peak, "kernel_ms": kernel_ms,
                                          "note": "the same ops over the step less event_floor_ms"},
            "l2": "flushed between timed steps (256 MiB write)"}


HOST_STALL_MS = 10.0


def host_stall_ms(run) -> float:
    """The longest single CUDA call inside a served run's register / jitter /
    submit entry points, in ms.  A host-side copy or launch normally returns
    in tens of microseconds, so one that blocked for over HOST_STALL_MS means
    the CUDA driver stopped taking work from every thread of the process at
    once."""
    return max(run["register_call_max_us"], run["jitter_call_max_us"], run["submit_call_max_us"]) / 1e3


def measured_once_more_after_stall(run_fn):
    """One served run (run_fn() -> dict with "sustained" and the call maxima).
    A run that misses the bound while one of its CUDA calls blocked for over
    HOST_STALL_MS is recorded under "stalled_run" of a second run, which is
    the one reported, as a clock-throttled run would be measured again; any
    other run is reported as it is."""
    x = run_fn()
    x["host_stall_ms"] = host_stall_ms(x)
    if not x["sustained"] and x["host_stall_ms"] > HOST_STALL_MS:
        y = run_fn()
        y["host_stall_ms"] = host_stall_ms(y)
        y["stalled_run"] = {k: x[k] for k in ("latency_p99_ms", "latency_max_ms", "host_stall_ms", "achieved_rate")}
        x = y
    return x


def measure_serve(ctx, seconds, rates=(2000.0, 10000.0, 50000.0), sweep=(60000.0, 80000.0, 90000.0, 100000.0,
                                                                        110000.0, 120000.0, 130000.0, 140000.0,
                                                                        150000.0, 200000.0),
                  sweep_seconds=10.0, submit_threads=4):
    """The served stream: Poisson arrivals at each rate for `seconds`, requests
    drawn like the batched mix (4 projections, random cameras, 128 base light
    sets of 256..65536 blob lights), light sets re-referenced with p = 0.7 and
    jittered on the device by N(0, 0.1) per request, an 8 GiB device budget.
    Latency runs from the scheduled arrival to the completion callback.  A
    sweep of 10 s runs then finds the highest offered rate the server
    sustains with p99 <= 2 ms (stopping at the first rate that misses)."""
    from hellovulkan_gb300.server import Server, run_load
    keep = ("offered_rate", "achieved_rate", "scheduled", "completed", "failed", "latency_p50_ms", "latency_p90_ms",
            "latency_p99_ms", "latency_p999_ms", "latency_max_ms", "queue_p50_ms", "queue_p99_ms", "exec_p50_ms",
            "exec_p99_ms", "submit_lag_p99_ms", "register_call_p50_us", "jitter_call_p50_us", "submit_call_p50_us",
            "register_call_max_us", "jitter_call_max_us", "submit_call_max_us", "worst_lag_arrival_s",
            "tests_per_s", "new_sets", "reused_sets")

    def one(rate, dur, thr):
        srv = Server(ctx, budget_bytes=8 << 30, max_batch_views=64, streams=4)
        rep = run_load(srv, rate=rate, duration=dur, submit_threads=thr)
        st = srv.stats()
        srv.close()
        r = {"rate": rate, "seconds": dur, "submit_threads": thr}
        r.update({k: rep[k] for k in keep})
        r.update({"views_per_s": rep["achieved_rate"], "batches": st["batches"],
                  "mean_views_per_batch": st["views_launched"] / max(1, st["batches"]),
                  "max_batch_views": st["max_batch_views"], "arena_peak_bytes": st["arena_peak_bytes"],
                  "evictions": st["evictions"],
                  "sustained": rep["latency_p99_ms"] <= 2.0 and rep["failed"] == 0 and
                  rep["achieved_rate"] >= 0.98 * rep["offered_rate"]})
        return r

    def measured(rate, dur):
        return measured_once_more_after_stall(lambda: one(rate, dur, submit_threads))

    runs = [measured(r, seconds) for r in rates]
    swept, best = [], 0.0
    for r in sweep:
        x = measured(r, sweep_seconds)
        swept.append({k: x[k] for k in ("rate", "achieved_rate", "latency_p50_ms", "latency_p99_ms",
                                         "mean_views_per_batch", "sustained", "host_stall_ms", "stalled_run")
                      if k in x})
        if not x["sustained"]:
            break
        best = x["achieved_rate"]
    return {"workload": "Poisson arrivals, 4 projections {8x8x16,16x9x24,24x14x32,32x18x48}, 128 base sets of "
                        "256..65536 blob lights, p_reuse 0.7 with device jitter sigma 0.1, 8 GiB budget, "
                        "64 views per batch, 4 streams",
            "runs": runs, "sweep": swept, "sweep_seconds": sweep_seconds,
            "max_sustained_views_per_s": best,
            "note": "sustained = p99 <= 2 ms, no failures, achieved >= 98% of offered; host_stall_ms = the "
                    "longest CUDA call inside the register/jitter/submit entry points; a run that missed "
                    "while one blocked > 10 ms is kept under stalled_run and measured once more"}


def measure_lookup(ctx, stream, reps=20):
    """Scene.frag's cluster lookup (cf_lookup_clusters) over a 1920x1080 depth
    buffer of log-uniform linear depths, on the 1920x1080 16x9x24 view with 1024
    lights culled by the pipeline: the lookup alone (timed), then once with
    every light tested (the drop-in check: a light containing a fragment but
    missing from its list only where the fragment leaves its cluster's box)."""
    import torch

    from hellovulkan_gb300._lib import FRAGMENT_CAPPED, FRAGMENT_OUTSIDE_AABB
    from hellovulkan_gb300.consumer import lookup_clusters, samples_to_numpy
    from hellovulkan_gb300.pipelines import (PipelineAABBGenerator, PipelineLightCulling, ResourcesClusterForward,
                                             ResourcesLight)
    from hellovulkan_gb300 import scenes
    v = scenes.plain_small(1)
    rl = ResourcesLight(ctx)
    rl.add_lights(v.lights)
    rc = ResourcesClusterForward(ctx)
    rc.create_buffers(*v.grid, v.cap)
    gen = PipelineAABBGenerator(ctx, rc)
    gen.set_cluster_forward_ubo(v.ubo)
    gen.fill_command_buffer(stream)
    cu = PipelineLightCulling(ctx, rl, rc)
    cu.set_cluster_forward_ubo(v.ubo)
    cu.fill_command_buffer(stream)
    b = rc.buffers()
    stream.synchronize()
    _, idx = rc.read_outputs(stream)
    w, h = 1920, 1080
    depth = torch.from_numpy(scenes.depth_log_uniform(np.random.default_rng(7), w, h, 0.1, 1000.0)).cuda()
    def run(check_all):
        return lookup_clusters(v.ubo, depth, b.light_cells, b.light_indices, rl.device_buffer, idx.size,
                               v.light_count, v.cap, b.aabbs, check_all, stream)

    for _ in range(3):
        run(False)
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(reps)]
    for a, c in ev:
        a.record(stream)
        run(False)
        c.record(stream)
    torch.cuda.synchronize()
    ms = float(np.median([a.elapsed_time(c) for a, c in ev]))
    a, c = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record(stream)
    out = run(True)
    c.record(stream)
    torch.cuda.synchronize()
    check_ms = a.elapsed_time(c)
    s = samples_to_numpy(out, h, w)
    f = s["flags"]
    explained = (f & (FRAGMENT_OUTSIDE_AABB | FRAGMENT_CAPPED)) > 0

    # Scene.frag's direct clustered lighting over a 1920x1080 G-buffer
    from hellovulkan_gb300._lib import CfPBRPushConstant
    from hellovulkan_gb300.consumer import shade_clusters
    pc = CfPBRPushConstant(1.75, 0.01, 0.0, 0.1, 0.1)
    g = torch.from_numpy(scenes.gbuffer(np.random.default_rng(8), v.ubo)).cuda()
    cam = scenes.camera_position(v.ubo)

    def shade():
        return shade_clusters(v.ubo, cam, pc, g, b.light_cells, b.light_indices, idx.size, rl.device_buffer,
                              v.light_count, stream)

    for _ in range(3):
        shade()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(reps)]
    for a, c in ev:
        a.record(stream)
        shade()
        c.record(stream)
    torch.cuda.synchronize()
    shade_ms = float(np.median([a.elapsed_time(c) for a, c in ev]))
    for o in (cu, gen, rc, rl):
        o.close()
    moved = w * h * (4 + 32)  # depth read + sample written; cells, indices and lights come from L2
    return {"workload": "1920x1080 depth buffer, 16x9x24 grid, 1024 lights (plain_small)",
            "ms": ms, "pixels_per_s": w * h / (ms * 1e-3), "gbs_depth_and_samples": moved / (ms * 1e-3) / 1e9,
            "check_all_lights_ms": check_ms, "mean_listed_lights": float(s["count"].mean()),
            "mean_covering_lights": float(s["covering"].mean()),
            "pixels_outside_their_box": int((f & FRAGMENT_OUTSIDE_AABB > 0).sum()),
            "pixels_missing_a_light": int((s["missing"] > 0).sum()),
            "unexplained_misses": int(((s["missing"] > 0) & ~explained).sum()),
            "shading": {"workload": "1920x1080 G-buffer, direct clustered lighting (Radiance.glsl) over the culled "
                                    "lists", "ms": shade_ms, "texels_per_s": w * h / (shade_ms * 1e-3),
                        "gbs_gbuffer_and_output": w * h * (48 + 16) / (shade_ms * 1e-3) / 1e9}}


def measure_frustum(stream, reps=50):
    """FrustumCulling.comp (cf_frustum_cull) on 10 000 random boxes, the case
    the reference's README quotes (under 25 microseconds on an RTX 3070
    Mobile, whole dispatch), and on 16 M boxes (768 MB of boxes and commands,
    larger than L2), whose cost is HBM traffic: 32 bytes read + 4 written per
    box.  Checked against the oracle on the 10 000-box case."""
    import math

    import torch

    from hellovulkan_gb300 import scenes
    from hellovulkan_gb300.camera import frustum_ubo
    from hellovulkan_gb300.consumer import frustum_cull
    from oracle import Oracle
    rng = np.random.default_rng(11)
    f = frustum_ubo(math.radians(45.0), 16.0 / 9.0, 0.1, 500.0, scenes.random_camera(rng))
    peaks = {}
    try:
        peaks = json.loads((REPO / "MEASURED_PEAKS.json").read_text())
    except (OSError, ValueError):
        pass
    hbm_peak = peaks.get("hbm_gbs", 6800.0)
    out = {}
    for n in (10000, 16 << 20):
        boxes = torch.from_numpy(scenes.random_boxes(rng, n)).cuda()
        cmds = torch.zeros((n, 4), dtype=torch.int32, device="cuda")
        for _ in range(3):
            frustum_cull(f, boxes, cmds, None, stream)
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(reps)]
        for a, c in ev:
            a.record(stream)
            frustum_cull(f, boxes, cmds, None, stream)
            c.record(stream)
        torch.cuda.synchronize()
        ms = float(np.median([a.elapsed_time(c) for a, c in ev]))
        r = {"boxes": n, "us": ms * 1e3, "boxes_per_s": n / (ms * 1e-3),
             "kept": float(cmds[:, 1].float().mean().item())}
        if n == 10000:
            r["parity_with_oracle"] = bool(np.array_equal(cmds[:, 1].cpu().numpy().astype(np.uint32),
                                                          Oracle().frustum_cull(f, boxes.cpu().numpy())))
            r["reference_published_us"] = 25.0
            r["reference_hardware"] = "RTX 3070 Mobile, 'less than 25 microseconds' (README.md:63)"
        else:
            gbs = n * 36 / (ms * 1e-3) / 1e9
            traffic = None
            try:  # DRAM bytes of one launch at this size, from an ncu capture
                traffic = json.loads((REPO / "profiles" / "dram_bytes_per_launch.json").read_text())[
                    "frustum_16M"]["frustum_kernel"] if n == 16 << 20 else None
            except (OSError, ValueError, KeyError):
                traffic = None
            r["roofline"] = {"bound": "hbm", "achieved": gbs, "peak": hbm_peak, "unit": "GB/s", "frac": gbs / hbm_peak,
                             "bytes_per_launch": n * 36, "traffic": traffic,
                             "peak_source": "MEASURED_PEAKS.json hbm_gbs (measured)"}
            if traffic:
                r["roofline"]["traffic_gbs"] = traffic / (ms * 1e-3) / 1e9
                r["roofline"]["traffic_frac"] = r["roofline"]["traffic_gbs"] / hbm_peak
                r["roofline"]["note"] = ("36 algorithmic bytes per box; DRAM moves 64 (the 16-byte command's sector "
                                         "is read to merge the 4-byte store, then written back)")
        out["boxes_%d" % n] = r
        del boxes, cmds
    return out


def check_stress_view(state, oracle):
    """One animated view (StressAnimation.view_state) against the host
    restatement of the orbit animation and the oracle's AABBs and culling."""
    from oracle import animate_orbits
    _, pos = animate_orbits(state["orbits0"], state["frame"])
    lights = state["lights"]
    oa = oracle.generate_aabbs(state["ubo"])
    oc, oi, _ = oracle.cull(state["ubo"], oa, lights, state["cap"])
    return {"frame": state["frame"], "view": state["view"],
            "lights": bool(np.array_equal(lights[:, :4].view(np.uint32), pos.view(np.uint32))),
            "aabbs": bool(np.array_equal(state["aabbs"].view(np.uint32), oa.view(np.uint32))),
            "cells": bool(np.array_equal(state["cells"], oc)), "indices": bool(np.array_equal(state["indices"], oi))}


def measure_stress(ctx, stream, n_views, n_lights, frames, seed=5):
    """The animated workload: n_views views x n_lights lights, every light moved
    one step along its orbit in place on the device each frame, every view
    culled each frame in one batched pass; the projection of every view changes
    every 60 frames (grid 16x9x24 <-> 32x18x48, fovY 45 <-> 60 degrees), which
    regenerates all AABBs.  Sampled frames and views are checked against the
    oracle (lights against the host restatement of the animation)."""
    import torch

    from hellovulkan_gb300.stress import StressAnimation, stress_device_bytes
    from oracle import Oracle
    free, _ = torch.cuda.mem_get_info()
    need = stress_device_bytes(n_views, n_lights) + n_views // 2 * (4_200_000 + 20_800_000) * n_lights // 4096
    if need > 0.8 * free:
        return {"skipped": "needs about %.1f GB of device memory, %.1f GB free" % (need / 1e9, free / 1e9)}
    t0 = time.perf_counter()
    st = StressAnimation(ctx, n_views=n_views, n_lights=n_lights, seed=seed)
    setup_s = time.perf_counter() - t0
    check_frames = {f for f in (0, 59, 60, 61, 299, frames - 1) if 0 <= f < frames}
    check_views = sorted({0, 1, n_views // 2 + 1, n_views - 1})
    o = Oracle()
    rep = st.run(frames, stream, check_frames=check_frames, check_views=check_views,
                 check=lambda state: check_stress_view(state, o))
    st.close()
    del st
    torch.cuda.empty_cache()
    rep["setup_s"] = setup_s
    rep["device_bytes"] = need
    rep["workload"] = ("%d views x %d lights, %d frames, projection change every 60 frames (grids 16x9x24 / "
                       "32x18x48 alternating per view and per epoch, fovY 45 / 60), lights on circles r U[1,10], "
                       "omega U[0.1,2] rad/s at 60 Hz, moved in place on the device" % (n_views, n_lights, frames))
    rep["l2"] = "inputs larger than L2 (%.0f MB of lights per frame), no flush" % (n_views * n_lights * 48 / 1e6)
    return rep


def run_summary(line: dict) -> dict:
    """The run's headline figures in one small object (placed last in the
    JSON line): each measured form of the path with its parity flag."""
    def pick(d, *keys):
        for k in keys:
            if not isinstance(d, dict) or k not in d:
                return None
            d = d[k]
        return d
    e2e = line.get("e2e", {})
    out = {"plain_large_ms_per_step": line.get("ms_per_step"), "plain_large_parity": line.get("parity_with_oracle"),
           "e2e_ms_per_frame_pipelined": e2e.get("ms_per_step"), "e2e_ms_one_frame": e2e.get("one_in_flight_ms_per_step"),
           "roofline_frac": pick(line, "roofline", "frac"),
           "cpu_baseline_tests_per_s": pick(line, "cpu_baseline", "value"),
           "plain_small_ms_per_step": pick(line, "plain_small", "ms_per_step"),
           "plain_small_frac": pick(line, "plain_small", "roofline", "frac"),
           "plain_small_frac_less_event_floor": pick(line, "plain_small", "roofline_less_event_floor", "frac"),
           "plain_small_parity": pick(line, "plain_small", "parity_with_oracle"),
           "batch_views_per_s": pick(line, "batched", "views_per_s"),
           "batch_speedup_vs_per_view_launch": pick(line, "batched", "speedup_vs_per_view_launch"),
           "batch_speedup_vs_plain_per_view": pick(line, "batched", "speedup_vs_plain_per_view"),
           "batch_parity": pick(line, "batched", "parity_sampled_views"),
           "served_max_sustained_views_per_s": pick(line, "served", "max_sustained_views_per_s"),
           "served_speedup_vs_plain_per_view": pick(line, "served", "speedup_vs_plain_per_view"),
           "stress_views_per_s": pick(line, "stress", "views_per_s"), "stress_parity": pick(line, "stress", "parity"),
           "lookup_unexplained_misses": pick(line, "cluster_lookup", "unexplained_misses"),
           "frustum_10k_us": pick(line, "frustum_culling", "boxes_10000", "us")}
    runs = pick(line, "served", "runs") or []
    out["served_p50_p99_ms"] = {str(int(r["rate"])): [r["latency_p50_ms"], r["latency_p99_ms"]] for r in runs}
    return out


def run_ours(args):
    import torch

    ws, rank, local = dist_env()
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    sm_count = torch.cuda.get_device_properties(local).multi_processor_count
    from hellovulkan_gb300 import build as cuda_build
    cuda_build.build()
    from hellovulkan_gb300.pipelines import (Context, PipelineAABBGenerator, PipelineLightCulling,
                                             ResourcesClusterForward, ResourcesLight)

    view = make_view(args.workload, rank)
    ctx = Context(local)
    rl = ResourcesLight(ctx)
    rl.add_lights(view.lights)
    rc = ResourcesClusterForward(ctx)
    rc.create_buffers(*view.grid, view.cap)
    gen = PipelineAABBGenerator(ctx, rc)
    cull = PipelineLightCulling(ctx, rl, rc)
    if args.tuning:
        cull.set_tuning(*[int(t) for t in args.tuning.split(",")])
    stream = torch.cuda.Stream()
    flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device="cuda")

    # AABBs: once per projection (timed for information)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    gen.set_cluster_forward_ubo(view.ubo)
    with torch.cuda.stream(stream):
        e0.record(stream)
        gen.fill_command_buffer(stream)
        e1.record(stream)
    stream.synchronize()
    aabb_ms = e0.elapsed_time(e1)

    cull.set_cluster_forward_ubo(view.ubo)
    cull_cfg_used = cull.tuning()

    def timed_steps(n, stages=False):
        """n steps, L2 flushed before each, each bracketed by CUDA events on the
        launching stream; returns (sum of step ms, per-step stage ms).  With
        stages, the pipeline also records its per-stage events (which add a
        little device time) and each step is read back before the next."""
        cull.enable_stage_timing(stages)
        starts = [torch.cuda.Event(enable_timing=True) for _ in range(n)]
        ends = [torch.cuda.Event(enable_timing=True) for _ in range(n)]
        stage = np.zeros((n, 3))
        for i in range(n):
            with torch.cuda.stream(stream):
                flush.zero_()
            starts[i].record(stream)
            cull.fill_command_buffer(stream)
            ends[i].record(stream)
            if stages:
                stage[i] = cull.stage_times_ms()
        torch.cuda.synchronize()
        cull.enable_stage_timing(False)
        return float(sum(s.elapsed_time(e) for s, e in zip(starts, ends))), stage

    for _ in range(args.warmup):
        cull.fill_command_buffer(stream)
    stream.synchronize()

    sampler = ClockSampler(local).start()
    if ws > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    total_ms, _ = timed_steps(args.steps)
    _, stage = timed_steps(max(3, min(args.steps, 100)), stages=True)  # the per-stage breakdown, untimed

    # e2e through the C ABI with host buffers: every step uploads its lights
    # from pinned memory, culls, and reads its cells and indices back into
    # pinned memory.  k pipelines (resources, culling pipeline, stream) are in
    # flight, as a renderer keeps frames in flight: step i + k - 1 is enqueued
    # before the host waits for step i's result.
    b = rc.buffers()
    h_lights = torch.from_numpy(np.ascontiguousarray(view.lights)).pin_memory()
    in_flight = max(2, args.e2e_in_flight)
    sets = [(rl, rc, cull, stream)]
    for _ in range(in_flight - 1):
        rl2 = ResourcesLight(ctx)
        rl2.add_lights(view.lights)
        rc2 = ResourcesClusterForward(ctx)
        rc2.create_buffers(*view.grid, view.cap)
        gen2 = PipelineAABBGenerator(ctx, rc2)
        gen2.set_cluster_forward_ubo(view.ubo)
        gen2.fill_command_buffer(stream)
        cull2 = PipelineLightCulling(ctx, rl2, rc2)
        if args.tuning:
            cull2.set_tuning(*[int(t) for t in args.tuning.split(",")])
        sets.append((rl2, rc2, cull2, torch.cuda.Stream()))
    pinned = []
    pipes = []
    for p_rl, p_rc, p_cull, p_st in sets:
        hc = torch.empty((b.cluster_count, 2), dtype=torch.int32).pin_memory()
        hi = torch.empty(b.index_capacity, dtype=torch.int32).pin_memory()
        pinned += [hc, hi]
        pipes.append((p_rl, p_rc, p_cull, p_st, hc.numpy().view(np.uint32), hi.numpy().view(np.uint32)))
    e2e_steps = max(200, min(args.steps, 500))  # ~10 ms, so that filling and draining the pipelines weigh little
    cull.enable_stage_timing(False)

    def enqueue(p):
        p_rl, _, p_cull, p_st = p[:4]
        p_rl.upload_async(h_lights, view.light_count, p_st)
        p_cull.set_cluster_forward_ubo(view.ubo)
        p_cull.fill_command_buffer(p_st)

    def e2e_run(n, k):
        """n steps with k pipelines in flight (k = 1: each step waits for its own)."""
        got = None
        for i in range(min(k - 1, n)):
            enqueue(pipes[i])
        for i in range(n):
            if i + k - 1 < n:
                enqueue(pipes[(i + k - 1) % k])
            p = pipes[i % k]
            _, got = p[1].read_outputs(p[3], p[4], p[5])
        return got

    e2e_run(2 * in_flight, in_flight)
    e2e_run(3, 1)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    got = e2e_run(e2e_steps, 1)
    torch.cuda.synchronize()
    e2e_serial_s = time.perf_counter() - t0
    t0 = time.perf_counter()
    got = e2e_run(e2e_steps, in_flight)
    torch.cuda.synchronize()
    e2e_s = time.perf_counter() - t0
    total_indices = got.size
    clocks = sampler.stop()

    # untimed: the tests the kernels executed in one step (work counters), and
    # the brute-force kernel on the same view (every light against every cluster)
    cull.enable_work_counters(True)
    cull.fill_command_buffer(stream)
    work_filter, work_cluster = cull.read_work_counters()
    cull.enable_work_counters(False)
    plain_steps = max(3, min(args.steps, 200))
    cull.set_tuning(*(PLAIN_SMALL if view.clusters <= 8192 else PLAIN_LARGE))
    for _ in range(3):
        cull.fill_command_buffer(stream)
    plain_ms, _ = timed_steps(plain_steps)
    _, plain_stage = timed_steps(max(3, min(plain_steps, 50)), stages=True)
    cull.set_tuning(0)

    traffic_all = {}
    try:
        traffic_all = json.loads((REPO / "profiles" / "dram_bytes_per_launch.json").read_text())
    except (OSError, ValueError):
        traffic_all = {}
    small = None
    if args.workload == "plain_large" and rank == 0:  # the 1920x1080 view, one launch per view
        small = measure_plain_small(ctx, stream, flush, max(3, args.steps), args.warmup, rank, sm_count,
                                    clocks.get("sm_max_mhz") or 2070.0, traffic_all.get("plain_small", {}))

    batched = None
    if not args.no_batch and rank == 0:
        batched = measure_batch(ctx, stream)
    lookup = frustum = None
    if rank == 0:
        lookup = measure_lookup(ctx, stream)
        frustum = measure_frustum(stream)
    stress = None
    if not args.no_stress and rank == 0:
        stress = measure_stress(ctx, stream, args.stress_views, args.stress_lights, args.stress_frames)
    served = None
    if not args.no_serve and rank == 0:
        served = measure_serve(ctx, args.serve_seconds)
        if batched:
            served["speedup_vs_plain_per_view"] = (served["max_sustained_views_per_s"] /
                                                   batched["plain_per_view_views_per_s"])
            served["speedup_vs_per_view_launch"] = (served["max_sustained_views_per_s"] /
                                                    batched["per_view_launch_views_per_s"])

    tests_per_view = view.clusters * view.light_count
    total_ms, e2e_s = max_over_ranks([total_ms, e2e_s], device="cuda")
    if rank != 0:
        torch.distributed.destroy_process_group()
        return

    # correctness of what was timed (rank 0, last e2e result) against the oracle
    from oracle import Oracle
    o = Oracle()
    o_aabbs = o.generate_aabbs(view.ubo)
    o_cells, o_idx, executed = o.cull(view.ubo, o_aabbs, view.lights, view.cap)
    # both pipelines' last read-backs (pinned host buffers)
    parity = total_indices == o_idx.size and all(
        np.array_equal(p[4], o_cells) and np.array_equal(p[5][: o_idx.size], o_idx) for p in pipes)

    value = ws * tests_per_view * args.steps / (total_ms * 1e-3)
    X, Y, Z = view.grid
    if cull_cfg_used[4] == 2:  # the one-launch kernel
        kernels_per_step = 1
    else:
        gw = cull_cfg_used[0] * cull_cfg_used[1]
        groups = Z * -(-(X * Y) // gw) if cull_cfg_used[4] else -(-view.clusters // gw)
        kernels_per_step = (4 if cull_cfg_used[4] else 3) + (1 if groups > 8192 else 0)
    sm_max = clocks.get("sm_max_mhz") or 2070.0
    fp32_peak = fp32_peak_tops(sm_count, sm_max)
    peak_note = ("nominal FP32 issue rate, %d SMs (device attribute) x %d lanes x %.0f MHz (no measured FP32 peak "
                 "exists in MEASURED_PEAKS.json)" % (sm_count, FP32_LANES_PER_SM, sm_max))
    peaks = {}
    try:
        peaks = json.loads((REPO / "MEASURED_PEAKS.json").read_text())
    except (OSError, ValueError):
        pass
    hbm_peak = peaks.get("hbm_gbs", 6800.0)
    traffic = {}
    prof = REPO / "profiles" / "dram_bytes_per_launch.json"
    if prof.exists():
        try:
            traffic = json.loads(prof.read_text()).get(args.workload, {})
        except ValueError:
            traffic = {}
    st_x, st_c, st_f = (float(np.mean(stage[:, i])) for i in range(3))
    H = o_idx.size
    cull_ops = (work_filter + work_cluster) * OPS_PER_TEST
    fin_bytes = 12 * view.clusters + 8 * H
    auto_cfg = cull_cfg_used
    if auto_cfg[4] == 2:
        cull_kernel_name = "one_launch_kernel (%d clusters per CTA, %d warps)" % tuple(auto_cfg[:2])
    else:
        cull_kernel_name = ("bin_slices_kernel + cull_pipe_kernel<%d,%d,%d,%d> (binned)" if auto_cfg[4] else
                            "cull_kernel<%d,%d,%d,%d> (brute force)") % tuple(auto_cfg[:4])
    if st_c >= st_f:
        ach = cull_ops / (st_c * 1e-3) / 1e12
        roof = {"bound": "fp32", "achieved": ach, "peak": fp32_peak, "unit": "Tops/s", "frac": ach / fp32_peak,
                "traffic": traffic.get("cull"), "kernel": cull_kernel_name,
                "ops_per_launch": cull_ops, "peak_source": peak_note,
                "work": "executed sphere-box tests x %d ops (work counters): %d slab/union + %d cluster" % (
                    OPS_PER_TEST, work_filter, work_cluster)}
    else:
        ach = fin_bytes / (st_f * 1e-3) / 1e9
        roof = {"bound": "hbm", "achieved": ach, "peak": hbm_peak, "unit": "GB/s", "frac": ach / hbm_peak,
                "traffic": traffic.get("finalize"), "kernel": "finalize_kernel", "bytes_per_launch": fin_bytes,
                "peak_source": "MEASURED_PEAKS.json hbm_gbs (measured)"}
    # the whole step against HBM: the algorithmic bytes of one view (lights
    # read, AABBs read, LightCells and indices written, the UBO) per step
    step_bytes = 48 * view.light_count + 32 * view.clusters + 8 * view.clusters + 4 * H + 176
    hbm_ach = step_bytes / (total_ms / args.steps * 1e-3) / 1e9
    roof_hbm = {"bound": "hbm", "achieved": hbm_ach, "peak": hbm_peak, "unit": "GB/s", "frac": hbm_ach / hbm_peak,
                "bytes_per_step": step_bytes, "peak_source": "MEASURED_PEAKS.json hbm_gbs (measured)",
                "note": "48 L + 40 C + 4 H + 176 bytes per view over the event-timed step; the path is issue-bound, "
                        "not HBM-bound"}
    p_x, p_c, p_f = (float(np.mean(plain_stage[:, i])) for i in range(3))
    p_ach = executed * OPS_PER_TEST / (p_c * 1e-3) / 1e12
    bi = view.light_count * 48
    bo = view.clusters * 8 + total_indices * 4 + 4
    cpu = None
    if not args.no_cpu_baseline:
        r = time_cpu(view, o_aabbs, args.cpu_seconds)
        cpu = {"value": r["value"], "unit": UNIT, "cores": r["cores"], "kind": r["kind"], "sample": r["sample"],
               "cpu": r["cpu"]}
    cfg = workload_config(view, args.workload)
    measurement = {"parallelism": "replicas x%d" % ws if ws > 1 else "single GPU",
                   "l2": "flushed between timed steps (256 MiB write)",
                   "aabbs": "generated once per projection (%.4f ms, not in the step)" % aabb_ms,
                   "step": ("light transform + culling + offset scan in one launch" if auto_cfg[4] == 2 else
                            "light transform + slice binning + culling + offset scan"),
                   "sm_count": sm_count}
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": total_ms / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic (seeded)", "config": cfg, "measurement": measurement,
        "views_per_s": ws * args.steps / (total_ms * 1e-3),
        "parity_with_oracle": parity,
        "stage_ms": {"light_transform": st_x, "bin_and_cull": st_c, "offset_scan": st_f},
        "executed_tests_per_view_reference_loop": executed,
        "executed_tests_per_view_kernels": work_filter + work_cluster,
        "roofline": roof,
        "roofline_hbm": roof_hbm,
        "plain_kernel": {"note": "brute force: every light against every cluster, same view",
                         "ms_per_step": plain_ms / plain_steps, "value": tests_per_view * plain_steps / (plain_ms * 1e-3),
                         "stage_ms": {"light_transform": p_x, "cull": p_c, "offset_scan": p_f},
                         "roofline": {"bound": "fp32", "achieved": p_ach, "peak": fp32_peak, "unit": "Tops/s",
                                      "frac": p_ach / fp32_peak, "kernel": "cull_kernel (brute force)",
                                      "ops_per_launch": executed * OPS_PER_TEST, "traffic": traffic.get("cull_plain")}},
        "cpu_baseline": cpu,
        "e2e": {"value": ws * tests_per_view * e2e_steps / e2e_s, "unit": UNIT, "h2d_bytes_per_step": bi,
                "d2h_bytes_per_step": bo, "ms_per_step": 1e3 * e2e_s / e2e_steps, "steps": e2e_steps,
                "one_in_flight_ms_per_step": 1e3 * e2e_serial_s / e2e_steps,
                "in_flight": in_flight,
                "kind": "pipelined throughput with %d frames in flight (a renderer's steady state); the latency of "
                        "one frame alone is one_in_flight_ms_per_step" % in_flight,
                "timing": "host clock, pinned host buffers, %d pipelines in flight (step i + %d enqueued before "
                          "the host waits for step i's read-back); one_in_flight: each step waits for its own" % (
                              in_flight, in_flight - 1)},
        # our kernels per step: light transform, [slice binning,] culling, [offset scan, for views of more
        # than 8192 cluster groups,] copy; each e2e step adds the read-back kernel (both e2e runs are timed)
        "gpu_launches": kernels_per_step * args.steps + (kernels_per_step + 1) * 2 * e2e_steps + (
            small["kernels_per_step"] * small["steps"] if small else 0),
        "plain_small": small,
        "clocks": clocks,
        "batched": batched,
        "served": served,
        "stress": stress,
        "cluster_lookup": lookup,
        "frustum_culling": frustum,
    }
    line["summary"] = run_summary(line)  # last, so that a record keeping the line's tail keeps it
    print(json.dumps(line), flush=True)
    if ws > 1:
        torch.distributed.destroy_process_group()


def main():
    args = parse()
    if args.impl == "reference":
        run_reference_arm(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
