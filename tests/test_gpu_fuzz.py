"""Randomised parity against the oracle: seeded random views through every
kernel configuration, the stateless entry point and the batch.

Each view draws an odd-sized grid (up to 40x24x50 clusters), a random
resolution, depth range, field of view and camera, a light count (0, 1, the
32-light and 1024-light boundaries, or up to 5000) and a cap from 1 to 255;
the lights mix uniform boxes, blobs and tiny near lights, and some carry NaN
or infinite coordinates, zero, negative, NaN, infinite or huge radii, huge
coordinates or a w other than 1.  Every output must equal the oracle's bit for
bit (the AABBs, the cells and the packed index list).  The same generator
also passes on 4 000 views of up to 48 000 clusters and 20 000 lights; the
suite runs a few seconds' worth."""
import numpy as np
import pytest

from gpu_helpers import bits, run_pipeline, run_stateless
from hellovulkan_gb300 import scenes
from hellovulkan_gb300.camera import cluster_forward_ubo, look_at_rh
from test_gpu_parity import TUNINGS

pytestmark = pytest.mark.gpu


def random_lights(rng, n):
    kind = int(rng.integers(0, 3))
    if kind == 0:
        L = scenes.uniform_box_lights(rng, n, [-40, -25, -150], [40, 25, 5], float(rng.uniform(0.05, 2)),
                                      float(rng.uniform(2, 40)))
    elif kind == 1:
        L = scenes.blob_lights(rng, n, n_blobs=int(rng.integers(1, 40)), sigma=float(rng.uniform(1, 20)))
    else:
        L = scenes.uniform_box_lights(rng, n, [-5, -5, -30], [5, 5, -0.05], 0.01, 3.0)
    if n and rng.random() < 0.6:
        for i in rng.integers(0, n, int(rng.integers(1, max(2, n // 20)))):
            c = int(rng.integers(0, 10))
            axis = int(rng.integers(0, 3))
            if c == 0:
                L[i, axis] = np.nan
            elif c == 1:
                L[i, axis] = np.inf
            elif c == 2:
                L[i, axis] = -np.inf
            elif c == 3:
                L[i, 8] = 0.0
            elif c == 4:
                L[i, 8] = -float(rng.uniform(0, 5))
            elif c == 5:
                L[i, 8] = np.nan
            elif c == 6:
                L[i, 8] = np.inf
            elif c == 7:
                L[i, axis] = float(rng.choice([1e30, -1e30, 3e19, -3e19]))
            elif c == 8:
                L[i, 3] = float(rng.uniform(-2, 2))
            else:
                L[i, 8] = 1e20
    return L


def random_view(rng, max_clusters=20000, max_lights=5000):
    while True:
        X, Y, Z = int(rng.integers(1, 41)), int(rng.integers(1, 25)), int(rng.integers(1, 51))
        if X * Y * Z <= max_clusters:
            break
    W, H = int(rng.integers(16, 4000)), int(rng.integers(16, 2500))
    near = float(10 ** rng.uniform(-3, 0))
    far = near * float(10 ** rng.uniform(0.5, 4))
    eye = rng.uniform(-50, 50, 3)
    eye[1] = rng.uniform(-10, 40)
    view = look_at_rh(tuple(eye), tuple(rng.uniform(-20, 20, 3)))
    n = int(rng.integers(1, max_lights)) if rng.random() < 0.7 else int(
        rng.choice([0, 1, 31, 32, 33, 64, 65, 1023, 1024, 1025, 2048, 2049]))
    cap = int(rng.choice([1, 2, 7, 32, 150, 150, 150, 255, int(rng.integers(1, 256))]))
    ubo = cluster_forward_ubo(float(rng.uniform(20, 120)), W, H, near, far, view, (X, Y, Z))
    return scenes.View(ubo, random_lights(rng, n), cap, "random %dx%dx%d L=%d cap=%d" % (X, Y, Z, n, cap))


def mismatch(oracle, v, aabbs, cells, idx):
    a = oracle.generate_aabbs(v.ubo)
    if not np.array_equal(bits(aabbs), bits(a)):
        return "AABBs differ"
    oc, oi, _ = oracle.cull(v.ubo, a, v.lights, v.cap)
    if not np.array_equal(cells, oc):
        bad = np.nonzero((cells != oc).any(axis=1))[0]
        return "cells differ in %d clusters, first %d: gpu %s oracle %s" % (
            bad.size, bad[0], cells[bad[0]].tolist(), oc[bad[0]].tolist())
    if not np.array_equal(idx, oi):
        return "index lists differ"
    return None


@pytest.mark.parametrize("seed", [11, 12])
def test_random_views_through_every_configuration(gpu, oracle, seed):
    rng = np.random.default_rng(seed)
    configs = [None] + TUNINGS
    failures = []
    for case in range(120):
        v = random_view(rng)
        tuning = configs[int(rng.integers(0, len(configs)))]
        m = mismatch(oracle, v, *run_pipeline(gpu, v, tuning))
        if m:
            failures.append((case, v.name, tuning, m))
        if rng.random() < 0.3:
            m = mismatch(oracle, v, *run_stateless(v))
            if m:
                failures.append((case, v.name, "cf_cull_lights", m))
    assert not failures, failures[:5]


def test_random_batches(gpu, oracle):
    import torch

    from hellovulkan_gb300.batch import Batch, BatchBuffers
    rng = np.random.default_rng(13)
    for b in range(4):
        views = [random_view(rng, 12000, 3000) for _ in range(int(rng.integers(1, 12)))]
        bufs = BatchBuffers(views)
        batch = Batch(gpu)
        batch.set_views(bufs.batch_views())
        s = torch.cuda.Stream()
        batch.generate_aabbs(s)
        batch.cull(s)
        torch.cuda.synchronize()
        for i, v in enumerate(views):
            m = mismatch(oracle, v, *bufs.read(i))
            assert m is None, (b, i, v.name, m)
        assert gpu.check_device_error() == 0
        batch.close()
