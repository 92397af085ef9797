"""CPU tests of the oracle: pinned math, agreement with the reference's own
shaders compiled as C++ (the two culling passes, frustum culling, and
Scene.frag's lookup and direct lighting), the committed golden fixtures and
hand-made cases."""
import hashlib
import math

import numpy as np
import pytest

from hellovulkan_gb300 import scenes
from hellovulkan_gb300.camera import ubo_from_bytes


def bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32)


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


# --- pinned math --------------------------------------------------------------

def test_host_build_does_not_contract_fma(oracle):
    # -ffp-contract=off: a*b + c is rounded twice, like the kernels' intrinsics
    assert oracle.fp_contract_probe() == 1


def test_pow_is_within_glsl_precision(oracle):
    """GLSL specifies pow's precision as that of exp2(y*log2(x)): 3 + 2|t| ulp."""
    rng = np.random.default_rng(0)
    worst = 0.0
    for x in np.concatenate([np.float32([2, 10, 1e3, 1e4, 2e4]), rng.uniform(1.001, 1e5, 500).astype(np.float32)]):
        for k in range(49):
            y = np.float32(np.float32(k) / np.float32(48))
            t = float(x) ** float(y)
            err = abs(oracle.pow(float(x), float(y)) - t) / float(np.spacing(np.float32(t)))
            worst = max(worst, err)
            assert err <= 3 + 2 * abs(float(y) * math.log2(float(x))), (x, y)
    assert worst < 24


def test_exp2_log2_special_values(oracle):
    assert oracle.log2(1.0) == 0.0 and oracle.log2(2.0) == 1.0 and oracle.log2(1024.0) == 10.0
    assert oracle.log2(0.0) == -math.inf and math.isnan(oracle.log2(-1.0)) and math.isnan(oracle.log2(math.nan))
    assert oracle.log2(math.inf) == math.inf
    for k in range(-126, 128):
        assert oracle.exp2(float(k)) == 2.0 ** k
    assert oracle.exp2(200.0) == math.inf and oracle.exp2(-200.0) == 0.0 and math.isnan(oracle.exp2(math.nan))
    assert oracle.exp2(-140.0) == 2.0 ** -140  # subnormal result


# --- oracle == reference shaders ---------------------------------------------

def _views_for_reference():
    rng = np.random.default_rng(7)
    vs = [scenes.plain_small(1), scenes.plain_large(2, n_lights=1024)]
    for _ in range(4):
        v = scenes.batch_view(rng)
        vs.append(scenes.View(v.ubo, v.lights[:1500], v.cap, v.name))
    return vs


@pytest.mark.parametrize("case", range(6))
def test_oracle_matches_reference_shaders(oracle, reference, case):
    v = _views_for_reference()[case]
    a = oracle.generate_aabbs(v.ubo)
    ar = reference.generate_aabbs(v.ubo)
    assert np.array_equal(bits(a), bits(ar))
    cells, idx, _ = oracle.cull(v.ubo, a, v.lights, reference.cap)
    rc, ri = reference.cull(v.ubo, ar, v.lights)
    assert np.array_equal(cells, rc)
    assert np.array_equal(idx, ri)


def test_reference_atomics_give_same_sets_in_any_order(oracle, reference):
    """Run in parallel, the reference's atomicAdd hands out slices in a
    scheduling-dependent order; per-cluster lists are the same."""
    v = scenes.plain_small(5)
    a = oracle.generate_aabbs(v.ubo)
    cells, idx, _ = oracle.cull(v.ubo, a, v.lights)
    rc, ri = reference.cull(v.ubo, a, v.lights, threads=4)
    assert np.array_equal(cells[:, 1], rc[:, 1])
    for c in range(cells.shape[0]):
        o, n = cells[c]
        ro, _ = rc[c]
        assert np.array_equal(idx[o:o + n], ri[ro:ro + n])


# --- golden fixtures ------------------------------------------------------------

def golden_names(golden):
    return [str(n) for n in golden["names"]]


def test_oracle_matches_golden(oracle, golden):
    for name in golden_names(golden):
        ubo = ubo_from_bytes(golden[name + "/ubo"])
        lights = golden[name + "/lights"]
        cap = int(golden[name + "/cap"][0])
        a = oracle.generate_aabbs(ubo)
        cells, idx, _ = oracle.cull(ubo, a, lights, cap)
        if name + "/aabbs" in golden.files:
            assert np.array_equal(bits(a), golden[name + "/aabbs"]), name
            assert np.array_equal(cells, golden[name + "/cells"]), name
            assert np.array_equal(idx, golden[name + "/indices"]), name
        else:
            assert sha(bits(a)) == str(golden[name + "/sha_aabbs"]), name
            assert sha(cells) == str(golden[name + "/sha_cells"]), name
            assert sha(idx) == str(golden[name + "/sha_indices"]), name


# --- hand-made known answers -------------------------------------------------------

def one_cluster_ubo():
    return scenes.custom_view((1, 1, 1), 100, 100, 1.0, 10.0).ubo


def light_rows(pos_r):
    return scenes.make_lights(np.float32([p for p, _ in pos_r]).reshape(-1, 3), np.float32([r for _, r in pos_r]))


def test_strict_less_on_the_face(oracle):
    """TestSphereAABB uses sq < r*r (LightCulling.comp:56): a sphere that just
    touches the box is not a hit."""
    ubo = one_cluster_ubo()
    a = oracle.generate_aabbs(ubo)
    mx = a[0, 4:7]
    x = float(mx[0]) + 2.0  # 2 units beyond the +x face, y/z inside
    y = float((a[0, 1] + a[0, 5]) / 2)
    z = float((a[0, 2] + a[0, 6]) / 2)
    d = np.float32(np.float32(mx[0]) - np.float32(x))
    r_touch = float(np.sqrt(np.float32(d * d)))  # r*r == d*d exactly when representable
    assert np.float32(r_touch) * np.float32(r_touch) == d * d
    lights = light_rows([((x, y, z), r_touch), ((x, y, z), np.nextafter(np.float32(r_touch), np.float32(10))),
                         ((x, y, z), 1.0)])
    cells, idx, _ = oracle.cull(ubo, a, lights)
    assert cells[0, 1] == 1 and list(idx) == [1]


def test_inside_light_hits_and_far_light_misses(oracle):
    ubo = one_cluster_ubo()
    a = oracle.generate_aabbs(ubo)
    centre = tuple(float(v) for v in (a[0, 0:3] + a[0, 4:7]) / 2)
    lights = light_rows([((0.0, 0.0, 50.0), 1.0), (centre, 1e-3), ((0.0, 0.0, -500.0), 5.0)])
    cells, idx, _ = oracle.cull(ubo, a, lights)
    assert list(idx) == [1] and list(cells[0]) == [0, 1]


def test_cap_keeps_the_first_hits_in_ascending_order(oracle):
    ubo = one_cluster_ubo()
    a = oracle.generate_aabbs(ubo)
    centre = tuple(float(v) for v in (a[0, 0:3] + a[0, 4:7]) / 2)
    # 400 lights, every third one misses: the list must be the first 150 hits
    rows = [((0.0, 0.0, 1e4), 1.0) if i % 3 == 0 else (centre, 1.0) for i in range(400)]
    cells, idx, executed = oracle.cull(ubo, a, light_rows(rows), 150)
    want = [i for i in range(400) if i % 3 != 0][:150]
    assert list(idx) == want and cells[0, 1] == 150
    assert executed == want[-1] + 1  # the reference loop stops at the 150th hit


def test_zero_lights_and_cap_of_one(oracle):
    v = scenes.plain_small(3)
    a = oracle.generate_aabbs(v.ubo)
    cells, idx, ex = oracle.cull(v.ubo, a, v.lights[:0])
    assert idx.size == 0 and not cells.any() and ex == 0
    cells, idx, _ = oracle.cull(v.ubo, a, v.lights, 1)
    assert cells[:, 1].max() == 1 and np.array_equal(cells[:, 0], np.cumsum(cells[:, 1]) - cells[:, 1])


def test_oracle_lookup_flags_cells_that_leave_the_index_list(oracle):
    """A cell pointing past the index list, or at a light that does not exist,
    is flagged and nothing is read through it (planted in the oracle's inputs)."""
    from hellovulkan_gb300 import scenes
    from hellovulkan_gb300._lib import FRAGMENT_BAD_CELL
    v = scenes.custom_view((4, 3, 8), 40, 30, 0.1, 100.0, lights=scenes.uniform_box_lights(
        np.random.default_rng(3), 50, [-5, -5, -60], [5, 5, -1]))
    a = oracle.generate_aabbs(v.ubo)
    cells, idx, _ = oracle.cull(v.ubo, a, v.lights, 150)
    depth = scenes.depth_log_uniform(np.random.default_rng(4), 40, 30, 0.1, 100.0)
    good = oracle.lookup_clusters(v.ubo, depth, cells, idx, v.lights, 150, a)
    assert not np.any(good["flags"] & FRAGMENT_BAD_CELL) and np.all(good["missing"][good["flags"] == 0] == 0)
    bad = cells.copy()
    bad[:, 0] = idx.size + 5  # every offset beyond the list
    s = oracle.lookup_clusters(v.ubo, depth, bad, idx, v.lights, 150, a)
    hit = s["count"] == 0
    assert np.all((s["flags"] & FRAGMENT_BAD_CELL) > 0) and np.all(hit)
    wrong = idx.copy()
    wrong[:] = v.light_count + 1  # indices that name no light
    s = oracle.lookup_clusters(v.ubo, depth, cells, wrong, v.lights, 150, a)
    listed = good["count"] > 0
    assert np.all((s["flags"][listed] & FRAGMENT_BAD_CELL) > 0) and np.all(s["covering"] == 0)


def test_oracle_frustum_culling_keeps_what_the_camera_sees():
    """Boxes around points in front of the camera are kept, boxes behind it or
    beyond the far plane are not (oracle only)."""
    from hellovulkan_gb300.camera import frustum_ubo, look_at_rh
    from oracle import Oracle
    o = Oracle()
    f = frustum_ubo(math.radians(60.0), 1.0, 0.1, 100.0, look_at_rh((0.0, 0.0, 0.0), (0.0, 0.0, -1.0)))
    def box(c, h=0.5):
        b = np.zeros(8, np.float32)
        b[0:3] = np.array(c) - h
        b[4:7] = np.array(c) + h
        return b
    boxes = np.stack([box((0, 0, -10)), box((0, 0, 10)), box((0, 0, -200)), box((50, 0, -10)), box((0, 0, -99.9))])
    assert o.frustum_cull(f, boxes).tolist() == [1, 0, 0, 0, 1]


# --- consumer passes: oracle == the reference's shader code --------------------

PC_DEFAULT = (1.75, 0.01, 0.0, 0.1, 0.1)  # the reference UI's defaults (Header/UIData.h:23-29)


def edge_boxes(rng, n):
    """Random boxes, then inverted, degenerate, huge, infinite, NaN and
    signed-zero ones: the cases where the GPU's single-corner plane test must
    fall back to the shader's eight-corner count."""
    b = scenes.random_boxes(rng, n)
    k = n // 16
    b[:k, [0, 4]] = b[:k, [4, 0]]
    b[k:2 * k, 4:7] = b[k:2 * k, 0:3]
    b[2 * k:2 * k + 32, 0] = -3e20
    b[2 * k + 32:2 * k + 64, 5] = np.inf
    b[2 * k + 64:2 * k + 96, 2] = np.nan
    b[2 * k + 96:2 * k + 128, 0:3] = -0.0
    b[2 * k + 96:2 * k + 128, 4:7] = 0.0
    b[2 * k + 128:2 * k + 160, 0:3] = -1e30
    b[2 * k + 128:2 * k + 160, 4:7] = 1e30
    return b


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_oracle_frustum_matches_reference_shader(oracle, reference, seed):
    """cfo_frustum_cull == FrustumCulling.comp:14-57 compiled as C++."""
    from hellovulkan_gb300.camera import frustum_ubo
    rng = np.random.default_rng(seed)
    boxes = edge_boxes(rng, 20000)
    for _ in range(3):
        f = frustum_ubo(math.radians(rng.uniform(30, 90)), rng.uniform(1.0, 2.5), 0.1, float(rng.uniform(100, 1000)),
                        scenes.random_camera(rng))
        want = reference.frustum_cull(f, boxes, threads=4)
        assert np.array_equal(oracle.frustum_cull(f, boxes), want)
        assert 0 < want.sum() < boxes.shape[0]


def _fragment_views():
    rng = np.random.default_rng(31)
    return [scenes.custom_view((16, 9, 24), 320, 180, 0.1, 1000.0, scenes.random_camera(rng),
                               scenes.blob_lights(rng, 2000)),
            scenes.custom_view((7, 5, 3), 140, 100, 0.2, 80.0, np.eye(4, dtype=np.float32),
                               scenes.uniform_box_lights(rng, 333, [-30, -20, -90], [30, 20, 10], 0.5, 6.0))]


@pytest.mark.parametrize("case", range(2))
def test_oracle_lookup_matches_reference_fragment_code(oracle, reference, case):
    """cfo_lookup_clusters' cluster, count, offset and LinearDepth ==
    Scene.frag:54-78 compiled as C++ (a fragment past the grid reads a zero
    cell there, and is flagged OUTSIDE_GRID with count 0 here)."""
    from hellovulkan_gb300._lib import FRAGMENT_OUTSIDE_GRID
    v = _fragment_views()[case]
    a = oracle.generate_aabbs(v.ubo)
    cells, idx, _ = oracle.cull(v.ubo, a, v.lights, 150)
    w, h = int(v.ubo.screenSize[0]), int(v.ubo.screenSize[1])
    depth = scenes.depth_log_uniform(np.random.default_rng(5 + case), w, h, float(v.ubo.cameraNear),
                                     float(v.ubo.cameraFar), far_plane_fraction=0.02)
    depth[0, :10] = 0.0
    got = oracle.lookup_clusters(v.ubo, depth, cells, idx, v.lights, 150, a)
    ref = reference.lookup_fragments(v.ubo, depth, cells, threads=4)
    inside = ref["cluster"] < cells.shape[0]
    assert np.array_equal((got["flags"] & FRAGMENT_OUTSIDE_GRID) == 0, inside)
    assert np.array_equal(got["cluster"][inside], ref["cluster"][inside])
    assert np.array_equal(got["count"], ref["count"]) and np.array_equal(got["offset"], ref["offset"])
    assert np.array_equal(bits(got["linear_depth"]), bits(ref["linear_depth"]))
    assert inside.mean() > 0.9 and (~inside).any()


@pytest.mark.parametrize("case", range(2))
def test_oracle_shading_matches_reference_fragment_code(oracle, reference, case):
    """cfo_shade_clusters' Lo == Scene.frag's direct lighting (Radiance.glsl
    and PBRHeader.glsl) compiled as C++, bit for bit; alpha is 1 exactly where
    the lookup lands in the grid."""
    from hellovulkan_gb300._lib import CfPBRPushConstant
    v = _fragment_views()[case]
    a = oracle.generate_aabbs(v.ubo)
    cells, idx, _ = oracle.cull(v.ubo, a, v.lights, 150)
    g = scenes.gbuffer(np.random.default_rng(9 + case), v.ubo, far_plane_fraction=0.02)
    cam = scenes.camera_position(v.ubo)
    pc = CfPBRPushConstant(*PC_DEFAULT)
    got = oracle.shade_clusters(v.ubo, cam, pc, g, cells, idx, v.lights)
    rgb, cl = reference.shade_fragments(v.ubo, cam, pc, g, cells, idx, v.lights, threads=4)
    assert np.array_equal(bits(got[..., :3]), bits(rgb))
    assert np.array_equal(got[..., 3] == 1.0, cl < cells.shape[0])


def test_oracle_shading_signed_zero_matches_reference(oracle, reference):
    """Radiance's own Lo starts at vec3(0.0) (Radiance.glsl:13,55), so a light
    whose term is -0 (NoL = -0: N = -z, the light in the texel's plane) adds
    +0: with albedoMultipler -0.0, Scene.frag's Lo ends +0, not -0."""
    from hellovulkan_gb300._lib import CfPBRPushConstant
    v = scenes.custom_view((1, 1, 1), 4, 4, 0.1, 100.0)
    g = np.zeros((4, 4, 12), np.float32)
    g[..., 0:3] = (0.0, 0.0, -5.0)
    g[..., 3] = 0.5
    g[..., 4:7] = (0.0, 0.0, -1.0)
    g[..., 7] = 0.3
    g[..., 8:11] = (-0.0, 0.25, 0.5)
    g[..., 11] = 0.6
    L = scenes.make_lights(np.float32([[-1.0, -1.0, -5.0]]), np.float32([10.0]))
    cells, idx = np.array([[0, 1]], np.uint32), np.array([0], np.uint32)
    for mult in (0.0, -0.0, 0.1):
        pc = CfPBRPushConstant(1.75, 0.01, 0.0, 0.1, mult)
        got = oracle.shade_clusters(v.ubo, np.zeros(3), pc, g, cells, idx, L)
        rgb, _ = reference.shade_fragments(v.ubo, np.zeros(3), pc, g, cells, idx, L)
        assert np.array_equal(bits(got[..., :3]), bits(rgb)), mult
    assert not np.signbit(got[..., :3]).any()


def test_oracle_consumers_match_golden(oracle, golden_consumers):
    """The oracle's frustum culling, lookup and lighting against the outputs
    the reference's own shader code produced (golden_consumers.npz)."""
    from hellovulkan_gb300._lib import CfFrustum, CfPBRPushConstant, FRAGMENT_OUTSIDE_GRID
    g = golden_consumers
    boxes = g["frustum/boxes"]
    for k in range(3):
        f = CfFrustum.from_buffer_copy(g["frustum/f%d" % k].tobytes())
        assert np.array_equal(oracle.frustum_cull(f, boxes), g["frustum/instance%d" % k].astype(np.uint32)), k
    ubo = ubo_from_bytes(g["frag/ubo"])
    cells, idx, lights = g["frag/cells"], g["frag/indices"], g["frag/lights"]
    s = oracle.lookup_clusters(ubo, g["frag/depth"], cells, idx, lights, 150)
    inside = g["frag/lookup_cluster"] < cells.shape[0]
    assert np.array_equal((s["flags"] & FRAGMENT_OUTSIDE_GRID) == 0, inside)
    assert np.array_equal(s["cluster"][inside], g["frag/lookup_cluster"][inside])
    assert np.array_equal(s["count"], g["frag/lookup_count"]) and np.array_equal(s["offset"], g["frag/lookup_offset"])
    assert np.array_equal(bits(s["linear_depth"]), g["frag/lookup_linear_depth"])
    out = oracle.shade_clusters(ubo, g["frag/camera"], CfPBRPushConstant(*g["frag/pc"].tolist()), g["frag/gbuffer"],
                                cells, idx, lights)
    assert np.array_equal(bits(out[..., :3]), g["frag/shade_rgb"])
    assert np.array_equal(out[..., 3] == 1.0, g["frag/shade_cluster"] < cells.shape[0])
    out = oracle.shade_clusters(ubo_from_bytes(g["negzero/ubo"]), np.zeros(3), CfPBRPushConstant(
        *g["negzero/pc"].tolist()), g["negzero/gbuffer"], g["negzero/cells"], g["negzero/indices"], g["negzero/lights"])
    assert np.array_equal(bits(out[..., :3]), g["negzero/shade_rgb"])


def test_jitter_restatement_follows_the_documented_formula():
    """oracle.jitter_lights (the host restatement the server's GPU tests check
    against) against the formula documented at cf_server_jitter_light_set in
    include/cfcull.h, restated here independently with Python integers and
    float32 scalars, one rounding per operation."""
    import numpy as np

    from hellovulkan_gb300 import scenes
    from oracle import jitter_lights
    M = (1 << 64) - 1

    def mix(x):
        x ^= x >> 30
        x = (x * 0xBF58476D1CE4E5B9) & M
        x ^= x >> 27
        x = (x * 0x94D049BB133111EB) & M
        return x ^ (x >> 31)

    rng = np.random.default_rng(41)
    lights = scenes.uniform_box_lights(rng, 9, [-20, -10, -60], [20, 10, -1], 1.0, 6.0)
    for seed, sigma in ((0, 0.1), (123456789, 0.75), ((1 << 64) - 3, 2.5)):
        got = jitter_lights(lights, seed, sigma)
        for i in range(lights.shape[0]):
            for a in range(3):
                s = np.float32(0.0)
                for k in range(12):
                    h = mix((seed + i * 0x9E3779B97F4A7C15 + (a * 12 + k) * 0xD1B54A32D192ED03) & M)
                    s = np.float32(s + np.float32(np.float32(h >> 40) * np.float32(2.0 ** -24)))
                want = np.float32(lights[i, a] + np.float32(np.float32(sigma) * np.float32(s - np.float32(6.0))))
                assert got[i, a].view(np.uint32) == want.view(np.uint32), (seed, i, a)
        assert np.array_equal(got[:, 3:].view(np.uint32), lights[:, 3:].view(np.uint32))  # only x, y, z move


def test_orbit_restatement_follows_the_documented_rotation():
    """oracle.animate_orbits (what the animated workload's GPU checks compare
    against) against CfLightOrbit's documented step, offset' = R * offset with
    R = [[cos, -sin], [sin, cos]], then position = (cx + x, cy, cz + z, cw):
    restated per light with float32 scalars, products before the difference
    or sum, one rounding per operation."""
    import numpy as np
    from oracle import animate_orbits
    rng = np.random.default_rng(43)
    n = 7
    o = np.zeros((n, 8), np.float32)
    o[:, 0:2] = rng.uniform(-10, 10, (n, 2))
    ang = rng.uniform(0.001, 0.05, n)
    o[:, 2], o[:, 3] = np.cos(ang), np.sin(ang)
    o[:, 4:7] = rng.uniform(-50, 50, (n, 3))
    o[:, 7] = 1.0
    got_o, got_p = animate_orbits(o, 13)
    for i in range(n):
        x, z, c, s = o[i, 0], o[i, 1], o[i, 2], o[i, 3]
        for _ in range(13):
            x, z = (np.float32(np.float32(c * x) - np.float32(s * z)), np.float32(np.float32(s * x) + np.float32(c * z)))
        want_p = np.array([np.float32(o[i, 4] + x), o[i, 5], np.float32(o[i, 6] + z), o[i, 7]], np.float32)
        assert got_o[i, 0].view(np.uint32) == np.float32(x).view(np.uint32)
        assert got_o[i, 1].view(np.uint32) == np.float32(z).view(np.uint32)
        assert np.array_equal(got_p[i].view(np.uint32), want_p.view(np.uint32)), i
