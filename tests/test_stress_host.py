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
