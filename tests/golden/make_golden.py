"""Generates tests/golden/golden_cases.npz from the reference's own shaders.

    python tests/golden/make_golden.py

The outputs come from oracle/_ref/libcf_ref.so: the reference's
AABBGenerator.comp and LightCulling.comp compiled as C++ (oracle/build.py),
with their workgroups run serially in index order, so the atomicAdd offsets
are the cluster-order scan.  It needs the reference checkout to build that
library; the committed fixture is what the tests read everywhere else.

Each case stores its inputs (UBO bytes, LightData records) and the
reference's outputs: AABBs as float32 bit patterns, LightCells and the index
list — in full for the small cases and as SHA-256 digests for the
1920x1080 / 1024-light case.
"""
from __future__ import annotations

import hashlib
import sys
from pathlib import Path

import numpy as np

REPO = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(REPO))

from hellovulkan_gb300 import scenes  # noqa: E402
from hellovulkan_gb300.camera import ubo_to_bytes, look_at_rh  # noqa: E402
from oracle import Reference  # noqa: E402

OUT = Path(__file__).resolve().parent / "golden_cases.npz"


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


def main():
    ref = Reference.load()
    if ref is None:
        raise SystemExit("the reference shaders could not be built here")
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
