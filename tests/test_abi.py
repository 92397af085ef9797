"""CPU tests of the C ABI and the host-side logic (no GPU calls)."""
import ctypes as C
import subprocess
from pathlib import Path

import numpy as np
import pytest

REPO = Path(__file__).resolve().parents[1]


def test_every_declared_symbol_is_exported(cflib):
    from hellovulkan_gb300 import _lib
    declared = _lib.declared_symbols()
    assert len(declared) >= 30
    for name in declared:
        assert hasattr(cflib, name), name
    out = subprocess.run(["nm", "-D", "--defined-only", str(_lib.LIB_PATH)], capture_output=True, text=True).stdout
    exported = {l.split()[-1] for l in out.splitlines() if " T " in l}
    assert set(declared) <= exported


def test_library_targets_sm103a_only(cflib):
    from hellovulkan_gb300 import _lib
    out = subprocess.run(["cuobjdump", "--list-elf", str(_lib.LIB_PATH)], capture_output=True, text=True)
    if out.returncode != 0:
        pytest.skip("cuobjdump unavailable")
    elfs = [l for l in out.stdout.splitlines() if "sm_" in l]
    assert elfs and all("sm_103a" in l for l in elfs), elfs


@pytest.mark.parametrize("std", ["c11", "c++17"])
def test_headers_compile_standalone(tmp_path, std):
    src = tmp_path / ("t.c" if std.startswith("c1") else "t.cpp")
    src.write_text('#include "cfcull.h"\n#include "cf_pinned_math.h"\nint main(void){return sizeof(CfClusterForwardUBO)==176?0:1;}\n')
    cc = "gcc" if std == "c11" else "g++"
    r = subprocess.run([cc, "-std=" + std, "-Wall", "-Werror", "-I", str(REPO / "include"), str(src), "-o", str(tmp_path / "a.out")],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    assert subprocess.run([str(tmp_path / "a.out")]).returncode == 0


def test_record_layouts():
    from hellovulkan_gb300 import _lib
    assert C.sizeof(_lib.CfLightData) == 48 and _lib.CfLightData.radius.offset == 32
    assert C.sizeof(_lib.CfAABB) == 32 and _lib.CfAABB.maxPoint.offset == 16
    assert C.sizeof(_lib.CfLightCell) == 8
    U = _lib.CfClusterForwardUBO
    offs = [U.cameraInverseProjection.offset, U.cameraView.offset, U.screenSize.offset, U.sliceScaling.offset,
            U.sliceBias.offset, U.cameraNear.offset, U.cameraFar.offset, U.sliceCountX.offset, U.sliceCountY.offset,
            U.sliceCountZ.offset]
    assert offs == [0, 64, 128, 136, 140, 144, 148, 152, 156, 160]  # std140 of Header.glsl:7-19


def test_status_strings_and_argument_errors_without_gpu(cflib):
    from hellovulkan_gb300 import _lib
    L = cflib
    assert L.cf_status_string(0) == b"success" and L.cf_status_string(4) == b"buffer too small"
    assert L.cf_version() == 10000
    assert L.cf_context_create(0, None) == 1
    assert L.cf_generate_aabbs(None, None, None) == 1
    assert b"null" in L.cf_last_error_message()
    n = C.c_uint64()
    from hellovulkan_gb300 import scenes
    v = scenes.plain_small(1)
    assert L.cf_cull_workspace_size(C.byref(v.ubo), 1024, 150, C.byref(n)) == 0
    # 3.5 M tests: brute force.  Status block + lights + flags + counts +
    # staging + group sums and offsets (432 groups of 8 clusters), each
    # 256-byte aligned
    al = lambda x: (x + 255) // 256 * 256
    assert n.value == (256 + al(1024 * 16) + al(4 * 4) + al(3456 * 4) + al(3456 * 150 * 4) + 2 * al(432 * 4))
    big = scenes.plain_large(2)
    assert L.cf_cull_workspace_size(C.byref(big.ubo), 16384, 150, C.byref(n)) == 0
    # 453 M tests: binned, 48 slices x 36 groups of 16 clusters, plus 48 slice
    # candidate lists (float4 + index), slice counts, slice flags and the
    # groups' union boxes
    assert n.value == (256 + al(16384 * 16) + al(64 * 4) + al(27648 * 4) + al(27648 * 150 * 4) + 2 * al(1728 * 4)
                       + al(48 * 16384 * 16) + al(48 * 16384 * 4) + 2 * al(2 * 48 * 4) + al(1728 * 32))
    ubo = _lib.CfClusterForwardUBO()
    ubo.sliceCountX, ubo.sliceCountY, ubo.sliceCountZ = 0, 9, 24
    assert L.cf_generate_aabbs(C.byref(ubo), C.c_void_p(256), None) == 1
    assert b"zero side" in L.cf_last_error_message()
    ubo.sliceCountX = 16
    assert L.cf_cull_lights(C.byref(ubo), C.c_void_p(256), C.c_void_p(256), 10, 0, C.c_void_p(256), C.c_void_p(256),
                            100, None, C.c_void_p(256), 1 << 30, None) == 1  # cap 0
    assert L.cf_cull_lights(C.byref(ubo), C.c_void_p(256), C.c_void_p(256), 10, 150, C.c_void_p(256), C.c_void_p(256),
                            100, None, C.c_void_p(256), 1 << 30, None) == 4  # index capacity < C * cap
    assert L.cf_cull_lights(C.byref(ubo), C.c_void_p(256), C.c_void_p(256), 10, 150, C.c_void_p(256), C.c_void_p(256),
                            3456 * 150, None, C.c_void_p(256), 64, None) == 4  # workspace too small
    assert L.cf_cull_lights(C.byref(ubo), C.c_void_p(256), C.c_void_p(256), 10, 150, C.c_void_p(256), C.c_void_p(256),
                            3456 * 150, None, C.c_void_p(300), 1 << 30, None) == 1  # misaligned workspace


def test_context_fails_loudly_without_a_gpu(cflib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is visible")
    from hellovulkan_gb300 import CfError
    from hellovulkan_gb300.pipelines import Context
    with pytest.raises(CfError) as e:
        Context(0)
    assert e.value.status == 8


def test_ubo_builder_matches_glm_conventions():
    from hellovulkan_gb300 import camera
    P = camera.perspective_rh_zo(np.pi / 4, 16 / 9, 0.1, 1000.0)
    # a point on the near plane maps to depth 0 and on the far plane to depth 1
    for z, d in ((-0.1, 0.0), (-1000.0, 1.0)):
        c = P.astype(np.float64) @ np.array([0.0, 0.0, z, 1.0])
        assert abs(c[2] / c[3] - d) < 1e-5
    V = camera.look_at_rh((0, 10, 60), (0, 0, 0))
    R = V[:3, :3].astype(np.float64)
    assert np.allclose(R @ R.T, np.eye(3), atol=1e-6)
    assert np.allclose(V.astype(np.float64) @ np.array([0, 10, 60, 1.0]), [0, 0, 0, 1], atol=1e-4)
    u = camera.cluster_forward_ubo(np.pi / 4, 1920, 1080, 0.1, 1000.0, np.eye(4, dtype=np.float32))
    b = camera.ubo_to_bytes(u)
    assert b.size == 176
    invp = np.frombuffer(b[:64].tobytes(), np.float32).reshape(4, 4).T  # column-major storage
    Pf = camera.perspective_rh_zo(np.pi / 4, 1920 / 1080, 0.1, 1000.0)
    Pf[1, 1] *= -1
    assert np.allclose(invp.astype(np.float64) @ Pf, np.eye(4), atol=1e-4)
    assert abs(u.sliceScaling - 24 / np.log2(1e4)) < 1e-5 and abs(u.sliceBias + 24 * np.log2(0.1) / np.log2(1e4)) < 1e-4


def test_scenes_are_seeded_and_shaped():
    from hellovulkan_gb300 import scenes
    a, b = scenes.plain_large(2), scenes.plain_large(2)
    assert np.array_equal(a.lights, b.lights) and a.clusters == 27648 and a.light_count == 16384
    assert (a.lights[:, 8] >= 0.5).all() and (a.lights[:, 8] <= 20).all() and (a.lights[:, 3] == 1).all()
    s = scenes.plain_small(1)
    p = s.lights[:, :3]
    assert s.clusters == 3456 and (p[:, 0] >= -20).all() and (p[:, 2] <= 10).all()
    mix = scenes.batch_mix(3, n_views=64)
    ls = [v.light_count for v in mix]
    assert min(ls) >= 256 and max(ls) <= 65536 and len({v.grid for v in mix}) == 4


@pytest.mark.parametrize("std", ["c11", "c++17"])
def test_testing_header_compiles_standalone(tmp_path, std):
    src = tmp_path / ("t.c" if std.startswith("c1") else "t.cpp")
    src.write_text('#include "cfcull_testing.h"\nint main(void){return CF_TESTING_STALL_ONE_LAUNCH == 1u ? 0 : 1;}\n')
    cc = "gcc" if std == "c11" else "g++"
    r = subprocess.run([cc, "-std=" + std, "-Wall", "-Werror", "-I", str(REPO / "include"), str(src), "-o",
                        str(tmp_path / "a.out")], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    assert subprocess.run([str(tmp_path / "a.out")]).returncode == 0


def test_testing_hooks_validate_without_gpu(cflib):
    assert cflib.cf_testing_inject_stall(0x80) == 1  # unknown bits: CF_ERROR_INVALID_ARGUMENT, no CUDA call
    assert cflib.cf_testing_fail_allocation_after(3) == 0 and cflib.cf_testing_fail_allocation_after(-1) == 0
