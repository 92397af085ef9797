"""Generates the golden fixtures from the reference's own shaders.

    python tests/golden/make_golden.py

The outputs come from oracle/_ref/libcf_ref.so: the reference's shaders
compiled as C++ (oracle/build.py).  It needs the reference checkout to build
that library; the committed fixtures are what the tests read everywhere else.

* golden_cases.npz — AABBGenerator.comp and LightCulling.comp, with their
  workgroups run serially in index order, so the atomicAdd offsets are the
  cluster-order scan.  Each case stores its inputs (UBO bytes, LightData
  records) and the reference's outputs: AABBs as float32 bit patterns,
  LightCells and the index list — in full for the small cases and as SHA-256
  digests for the larger ones.
* golden_consumers.npz — FrustumCulling.comp's instanceCount for a set of
  boxes (random, inverted, degenerate, huge, infinite, NaN, signed-zero) under
  three frusta; Scene.frag's clustered lookup (cluster index, count, offset,
  LinearDepth bits) over a depth buffer, and its direct lighting (Lo bits)
  over a G-buffer, with the cells and indices the reference's culling made;
  and a one-cluster shading case whose albedoMultipler is -0.0 (Radiance's
  own Lo starts at +0, so a -0 term becomes +0).
"""
from __future__ import annotations

import hashlib
import sys
from pathlib import Path

import numpy as np

REPO = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(REPO))

from hellovulkan_gb300 import scenes  # noqa: E402
from hellovulkan_gb300.camera import frustum_ubo, ubo_to_bytes, look_at_rh  # noqa: E402
from oracle import Reference  # noqa: E402

OUT = Path(__file__).resolve().parent / "golden_cases.npz"
OUT_CONSUMERS = Path(__file__).resolve().parent / "golden_consumers.npz"
# PBR push constants of the shading cases: the reference UI's defaults
# (Header/UIData.h:23-29) and the same with albedoMultipler -0.0
PC_DEFAULT = (1.75, 0.01, 0.0, 0.1, 0.1)
PC_NEG_ZERO = (1.75, 0.01, 0.0, 0.1, -0.0)


def sha(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def cases():
    rng = np.random.default_rng(20240601)
    out = {}
    out["plain_small"] = (scenes.plain_small(1), "hash")
    out["zero_lights"] = (scenes.custom_view((16, 9, 24), 1920, 1080, 0.1, 1000.0), "full")
    v = scenes.custom_view((1, 1, 1), 640, 480, 0.5, 50.0,
                           lights=scenes.uniform_box_lights(rng, 37, [-10, -10, -60], [10, 10, 5]))
    out["grid_1x1x1"] = (v, "full")
    v = scenes.custom_view((7, 5, 3), 700, 500, 0.2, 80.0,
                           lights=scenes.uniform_box_lights(rng, 333, [-30, -20, -90], [30, 20, 10], 0.5, 6.0))
    out["odd_grid_odd_lights"] = (v, "full")
    # dense: 1000 large lights in front of the camera -> most clusters hit the cap of 150
    v = scenes.custom_view((8, 8, 16), 1024, 1024, 0.1, 200.0,
                           lights=scenes.uniform_box_lights(rng, 1000, [-15, -15, -40], [15, 15, -1], 3.0, 12.0))
    out["cap_dense"] = (v, "full")
    # everything hits: radius far larger than the frustum -> all clusters capped early
    v = scenes.custom_view((4, 4, 4), 512, 512, 0.1, 100.0,
                           lights=scenes.uniform_box_lights(rng, 700, [-1, -1, -5], [1, 1, -1], 1e4, 1e4))
    out["all_capped"] = (v, "full")
    # non-finite light coordinates: NaN and +-inf in some positions and radii
    L = scenes.uniform_box_lights(rng, 300, [-20, -10, -60], [20, 10, 0], 1.0, 8.0)
    L[5, 0] = np.nan
    L[17, 1] = np.inf
    L[40, 2] = -np.inf
    L[41, :3] = np.nan
    L[90, 8] = np.nan
    L[91, 8] = np.inf
    L[299, 2] = np.inf
    out["nonfinite_lights"] = (scenes.custom_view((16, 9, 24), 1920, 1080, 0.1, 100.0, lights=L), "full")
    # lights behind the camera and a rotated view
    view = look_at_rh((5.0, 3.0, -2.0), (-4.0, 1.0, -30.0))
    L = scenes.uniform_box_lights(rng, 512, [-40, -10, -80], [40, 20, 40], 0.5, 5.0)
    out["behind_and_rotated"] = (scenes.custom_view((16, 9, 24), 1280, 720, 0.1, 300.0, view=view, lights=L), "full")
    out["plain_large_2k"] = (scenes.plain_large(2, n_lights=2048), "hash")
    return out


def frustum_boxes(rng, n: int = 4096) -> np.ndarray:
    """Random boxes followed by the cases a plane test can get wrong."""
    b = scenes.random_boxes(rng, n)
    k = n // 16
    b[:k, [0, 4]] = b[:k, [4, 0]]                  # inverted on x
    b[k:2 * k, 4:7] = b[k:2 * k, 0:3]              # degenerate (a point)
    b[2 * k:2 * k + 32, 0] = -3e20                 # beyond any safe magnitude
    b[2 * k + 32:2 * k + 64, 5] = np.inf
    b[2 * k + 64:2 * k + 96, 2] = np.nan
    b[2 * k + 96:2 * k + 128, 0:3] = -0.0          # signed zeros at the origin
    b[2 * k + 96:2 * k + 128, 4:7] = 0.0
    b[2 * k + 128:2 * k + 160, 0:3] = -1e30        # huge boxes containing everything
    b[2 * k + 128:2 * k + 160, 4:7] = 1e30
    return b


def consumer_cases(ref):
    """golden_consumers.npz: FrustumCulling.comp and Scene.frag's lookup and
    direct lighting run by the reference's own code."""
    from hellovulkan_gb300._lib import CfPBRPushConstant
    rng = np.random.default_rng(20241204)
    a = {}
    boxes = frustum_boxes(rng)
    a["frustum/boxes"] = boxes
    for k in range(3):
        f = frustum_ubo(np.radians(rng.uniform(30, 90)), rng.uniform(1.0, 2.5), 0.1, float(rng.uniform(100, 1000)),
                        scenes.random_camera(rng))
        a["frustum/f%d" % k] = np.frombuffer(bytes(f), np.uint8).copy()
        a["frustum/instance%d" % k] = ref.frustum_cull(f, boxes).astype(np.uint8)
        print("frustum %d: %d of %d boxes kept" % (k, int(a["frustum/instance%d" % k].sum()), boxes.shape[0]))
    # lookup and lighting on a 96x54 screen, 16x9x24 grid, 600 blob lights
    v = scenes.custom_view((16, 9, 24), 96, 54, 0.1, 1000.0, scenes.random_camera(rng), scenes.blob_lights(rng, 600))
    aabbs = ref.generate_aabbs(v.ubo)
    cells, idx = ref.cull(v.ubo, aabbs, v.lights)
    depth = scenes.depth_log_uniform(rng, 96, 54, 0.1, 1000.0, far_plane_fraction=0.03)
    depth[0, :8] = 0.0  # the near plane
    look = ref.lookup_fragments(v.ubo, depth, cells)
    g = scenes.gbuffer(rng, v.ubo, far_plane_fraction=0.03)
    cam = scenes.camera_position(v.ubo).astype(np.float32)
    rgb, cl = ref.shade_fragments(v.ubo, cam, CfPBRPushConstant(*PC_DEFAULT), g, cells, idx, v.lights)
    a.update({"frag/ubo": ubo_to_bytes(v.ubo), "frag/lights": v.lights, "frag/cells": cells, "frag/indices": idx,
              "frag/depth": depth, "frag/lookup_cluster": look["cluster"], "frag/lookup_count": look["count"],
              "frag/lookup_offset": look["offset"], "frag/lookup_linear_depth": look["linear_depth"].view(np.uint32),
              "frag/gbuffer": g, "frag/camera": cam, "frag/pc": np.float32(PC_DEFAULT),
              "frag/shade_rgb": rgb.view(np.uint32), "frag/shade_cluster": cl})
    print("lookup/shade: %d pixels, %d listed indices, %d pixels past the grid" % (
        depth.size, idx.size, int((look["cluster"] >= cells.shape[0]).sum())))
    # one cluster, one light in the plane of the texel: NoL is -0 and so is
    # the light's term; with albedoMultipler -0.0 Lo starts at -0
    v1 = scenes.custom_view((1, 1, 1), 4, 4, 0.1, 100.0)
    g1 = np.zeros((4, 4, 12), np.float32)
    g1[..., 0:3] = (0.0, 0.0, -5.0)
    g1[..., 3] = 0.5
    g1[..., 4:7] = (0.0, 0.0, -1.0)
    g1[..., 7] = 0.3
    g1[..., 8:11] = (-0.0, 0.25, 0.5)
    g1[..., 11] = 0.6
    L1 = scenes.make_lights(np.float32([[-1.0, -1.0, -5.0]]), np.float32([10.0]))
    c1, i1 = np.array([[0, 1]], np.uint32), np.array([0], np.uint32)
    rgb1, _ = ref.shade_fragments(v1.ubo, np.zeros(3, np.float32), CfPBRPushConstant(*PC_NEG_ZERO), g1, c1, i1, L1)
    a.update({"negzero/ubo": ubo_to_bytes(v1.ubo), "negzero/gbuffer": g1, "negzero/lights": L1, "negzero/cells": c1,
              "negzero/indices": i1, "negzero/pc": np.float32(PC_NEG_ZERO), "negzero/shade_rgb": rgb1.view(np.uint32)})
    return a


def main():
    ref = Reference.load()
    if ref is None:
        raise SystemExit("the reference shaders could not be built here")
    cons = consumer_cases(ref)
    np.savez_compressed(OUT_CONSUMERS, **cons)
    print(OUT_CONSUMERS, OUT_CONSUMERS.stat().st_size, "bytes")
    arrays = {}
    names = []
    for name, (v, mode) in cases().items():
        aabbs = ref.generate_aabbs(v.ubo)
        cells, idx = ref.cull(v.ubo, aabbs, v.lights)
        names.append(name)
        arrays[name + "/ubo"] = ubo_to_bytes(v.ubo)
        arrays[name + "/lights"] = v.lights
        arrays[name + "/cap"] = np.array([ref.cap], np.uint32)
        if mode == "full":
            arrays[name + "/aabbs"] = aabbs.view(np.uint32)
            arrays[name + "/cells"] = cells
            arrays[name + "/indices"] = idx
        else:
            arrays[name + "/sha_aabbs"] = np.array(sha(aabbs.view(np.uint32)))
            arrays[name + "/sha_cells"] = np.array(sha(cells))
            arrays[name + "/sha_indices"] = np.array(sha(idx))
            arrays[name + "/total"] = np.array([idx.size], np.uint64)
        print("%-22s C=%6d L=%6d total=%7d max=%3d capped=%d" % (
            name, cells.shape[0], v.lights.shape[0], idx.size, cells[:, 1].max(initial=0),
            int((cells[:, 1] == ref.cap).sum())))
    arrays["names"] = np.array(names)
    np.savez_compressed(OUT, **arrays)
    print(OUT, OUT.stat().st_size, "bytes")


if __name__ == "__main__":
    main()
