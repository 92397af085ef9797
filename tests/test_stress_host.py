"""Host-side checks of the animated workload: the orbit restatement and the
per-epoch projections (no GPU)."""
import math

import numpy as np

from hellovulkan_gb300 import scenes
from hellovulkan_gb300.camera import cluster_forward_ubo
from oracle import animate_orbits


def test_orbit_restatement_composes_and_keeps_the_radius():
    rng = np.random.default_rng(1)
    lights, orbits = scenes.orbit_lights(rng, 2, 500)
    o0, p0 = animate_orbits(orbits, 0)
    assert np.array_equal(p0[:, :3], lights[:, :3]) and np.array_equal(o0, orbits)
    o5, p5 = animate_orbits(orbits, 5)
    o3, _ = animate_orbits(orbits, 3)
    o32, p32 = animate_orbits(o3, 2)
    assert np.array_equal(o5.view(np.uint32), o32.view(np.uint32)) and np.array_equal(p5, p32)
    r0 = np.hypot(orbits[:, 0], orbits[:, 1])
    o600, _ = animate_orbits(orbits, 600)
    assert np.allclose(np.hypot(o600[:, 0], o600[:, 1]), r0, rtol=1e-4)
    assert np.array_equal(p5[:, 1], orbits[:, 5]) and np.all(p5[:, 3] == 1.0)  # height and w kept


def test_stress_projections_alternate_grids_and_fov():
    cam = scenes.random_camera(np.random.default_rng(2))
    for i, e in [(0, 0), (1, 0), (0, 1), (5, 2), (6, 7)]:
        u = scenes.stress_ubo(i, e, cam)
        grid = scenes.STRESS_GRIDS[(i + e) % 2]
        t = 120 if grid == (16, 9, 24) else 80
        ref = cluster_forward_ubo(math.radians(45.0 if e % 2 == 0 else 60.0), grid[0] * t, grid[1] * t, 0.1, 2000.0,
                                  cam, grid)
        assert bytes(u) == bytes(ref)
    # half of the views on each grid in every epoch
    for e in range(3):
        grids = [scenes.STRESS_GRIDS[(i + e) % 2] for i in range(8)]
        assert grids.count((16, 9, 24)) == 4


def test_stress_checker_accepts_a_correct_view_and_flags_a_planted_error():
    """bench.check_stress_view on a view state built on the CPU from the
    oracle itself: all parts match; a flipped index (planted in the oracle's
    own output) and a moved light are reported."""
    from bench import check_stress_view
    from oracle import Oracle
    o = Oracle()
    rng = np.random.default_rng(3)
    lights0, orbits = scenes.orbit_lights(rng, 1, 300)
    _, pos = animate_orbits(orbits, 4)
    lights = lights0.copy()
    lights[:, 0:4] = pos
    ubo = scenes.stress_ubo(0, 0, scenes.random_camera(rng))
    a = o.generate_aabbs(ubo)
    cells, idx, _ = o.cull(ubo, a, lights, 150)
    state = {"frame": 4, "view": 0, "lights": lights, "orbits0": orbits, "aabbs": a, "cells": cells,
             "indices": idx, "ubo": ubo, "cap": 150}
    assert all(check_stress_view(state, o)[k] for k in ("lights", "aabbs", "cells", "indices"))
    bad = dict(state, indices=idx.copy())
    bad["indices"][0] ^= 1
    assert not check_stress_view(bad, o)["indices"]
    moved = dict(state, lights=lights.copy())
    moved["lights"][7, 0] += 1.0
    r = check_stress_view(moved, o)
    assert not r["lights"]


def test_the_package_never_imports_the_oracle():
    """The oracle is the checker: nothing under hellovulkan_gb300/ imports it."""
    import re
    from pathlib import Path
    pkg = Path(__file__).resolve().parents[1] / "hellovulkan_gb300"
    pat = re.compile(r"^\s*(from\s+oracle\b|import\s+oracle\b)", re.M)
    offenders = [str(p) for p in pkg.rglob("*.py") if pat.search(p.read_text())]
    assert not offenders, offenders
