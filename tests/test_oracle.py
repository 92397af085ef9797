"""CPU tests of the oracle: pinned math, agreement with the reference's own
shaders compiled as C++, the committed golden fixtures and hand-made cases."""
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
