"""Seeded synthetic workloads of the clustered-forward culling path.

No public dataset is involved: every workload is generated here from a seed
with the shapes, sizes and value distributions of the benchmark
configurations.

  plain_small    1920x1080, 16x9x24 grid, fovY 45 deg, near 0.1, far 1000,
                 camera at the origin looking down -Z (identity view);
                 1024 lights, position U([-20,20]x[0,15]x[-40,10]) (w = 1),
                 color U[0,1]^3, radius U[1,5]
  plain_large    2560x1600, 32x18x48 grid, near 0.1, far 2000, camera at
                 (0,10,60) looking at the origin; 16384 lights from 32
                 Gaussian blobs (sigma 8) whose centres are uniform in
                 x in [-100,100], z in [-100,100], height y in [0,30] (y is
                 up, as in the reference scenes); radius lognormal(ln 3, 0.5)
                 clipped to [0.5, 20]; cap 150
  batch_mix      256 views; grid drawn from {8x8x16, 16x9x24, 24x14x32,
                 32x18x48} with a resolution of matching aspect; light count
                 log-uniform in [256, 65536], lights as plain_large; camera
                 uniform in [-80,80]x[2,40]x[-80,80] looking at a uniform
                 target in [-20,20]^3; near 0.1, far 2000

  stress         n_views views x n_lights lights each (4096 x 4096 at full
                 size), lights drawn like plain_large around per-view blobs and
                 moving on horizontal circles of radius U[1,10] at angular speed
                 U[0.1,2] rad/s, 60 frames per second; the projection changes
                 every 60 frames: view i uses grid STRESS_GRIDS[(i + epoch) % 2]
                 (16x9x24 at 1920x1080, 32x18x48 at 2560x1440) and fovY
                 alternates 45 / 60 degrees; cameras as batch_mix

LightData records are numpy float32 arrays of shape (n, 12): position xyzw,
color rgba, radius, 3 pad words (the 48-byte std430 record).
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

from .camera import cluster_forward_ubo, look_at_rh
from ._lib import CfClusterForwardUBO

FOVY = math.radians(45.0)
GRIDS = ((8, 8, 16), (16, 9, 24), (24, 14, 32), (32, 18, 48))
# pixel size of a cluster tile for each grid, so that resolution matches aspect
TILE_PX = {(8, 8, 16): 128, (16, 9, 24): 120, (24, 14, 32): 120, (32, 18, 48): 80}
CAP = 150


@dataclass
class View:
    ubo: CfClusterForwardUBO
    lights: np.ndarray  # (n, 12) float32
    cap: int = CAP
    name: str = ""
    meta: dict = field(default_factory=dict)

    @property
    def grid(self):
        return int(self.ubo.sliceCountX), int(self.ubo.sliceCountY), int(self.ubo.sliceCountZ)

    @property
    def clusters(self) -> int:
        x, y, z = self.grid
        return x * y * z

    @property
    def light_count(self) -> int:
        return int(self.lights.shape[0])


def make_lights(pos: np.ndarray, radius: np.ndarray, color: np.ndarray | None = None) -> np.ndarray:
    n = pos.shape[0]
    out = np.zeros((n, 12), np.float32)
    out[:, 0:3] = pos
    out[:, 3] = 1.0
    out[:, 4:7] = color if color is not None else 1.0
    out[:, 7] = 1.0
    out[:, 8] = radius
    return out


def uniform_box_lights(rng: np.random.Generator, n: int, lo, hi, rmin=1.0, rmax=5.0) -> np.ndarray:
    pos = rng.uniform(lo, hi, size=(n, 3)).astype(np.float32)
    color = rng.uniform(0.0, 1.0, size=(n, 3)).astype(np.float32)
    radius = rng.uniform(rmin, rmax, size=n).astype(np.float32)
    return make_lights(pos, radius, color)


def blob_lights(rng: np.random.Generator, n: int, n_blobs: int = 32, sigma: float = 8.0) -> np.ndarray:
    centres = np.stack([rng.uniform(-100, 100, n_blobs), rng.uniform(0, 30, n_blobs),
                        rng.uniform(-100, 100, n_blobs)], axis=1)
    which = rng.integers(0, n_blobs, size=n)
    pos = (centres[which] + rng.normal(0.0, sigma, size=(n, 3))).astype(np.float32)
    radius = np.clip(rng.lognormal(math.log(3.0), 0.5, size=n), 0.5, 20.0).astype(np.float32)
    color = rng.uniform(0.0, 1.0, size=(n, 3)).astype(np.float32)
    return make_lights(pos, radius, color)


def plain_small(seed: int = 1, n_lights: int = 1024) -> View:
    rng = np.random.default_rng(seed)
    ubo = cluster_forward_ubo(FOVY, 1920, 1080, 0.1, 1000.0, np.eye(4, dtype=np.float32), (16, 9, 24))
    lights = uniform_box_lights(rng, n_lights, [-20, 0, -40], [20, 15, 10])
    return View(ubo, lights, CAP, "plain_small 1920x1080 16x9x24 L=%d" % n_lights)


def plain_large(seed: int = 2, n_lights: int = 16384, grid=(32, 18, 48)) -> View:
    rng = np.random.default_rng(seed)
    view = look_at_rh((0.0, 10.0, 60.0), (0.0, 0.0, 0.0))
    ubo = cluster_forward_ubo(FOVY, 2560, 1600, 0.1, 2000.0, view, grid)
    lights = blob_lights(rng, n_lights)
    return View(ubo, lights, CAP, "plain_large 2560x1600 %dx%dx%d L=%d" % (*grid, n_lights))


def random_camera(rng: np.random.Generator):
    eye = (rng.uniform(-80, 80), rng.uniform(2, 40), rng.uniform(-80, 80))
    target = tuple(rng.uniform(-20, 20, 3))
    return look_at_rh(eye, target)


def batch_view(rng: np.random.Generator, light_set: np.ndarray | None = None) -> View:
    grid = GRIDS[int(rng.integers(0, len(GRIDS)))]
    t = TILE_PX[grid]
    w, h = grid[0] * t, grid[1] * t
    ubo = cluster_forward_ubo(FOVY, w, h, 0.1, 2000.0, random_camera(rng), grid)
    if light_set is None:
        n = int(round(math.exp(rng.uniform(math.log(256), math.log(65536)))))
        light_set = blob_lights(rng, n)
    return View(ubo, light_set, CAP, "batch %dx%dx%d L=%d" % (*grid, light_set.shape[0]))


def batch_mix(seed: int = 3, n_views: int = 256) -> list[View]:
    rng = np.random.default_rng(seed)
    return [batch_view(rng) for _ in range(n_views)]


def custom_view(grid, width, height, near, far, view=None, lights=None, cap=CAP, fovy=FOVY) -> View:
    view = np.eye(4, dtype=np.float32) if view is None else view
    ubo = cluster_forward_ubo(fovy, width, height, near, far, view, grid)
    lights = np.zeros((0, 12), np.float32) if lights is None else lights
    return View(ubo, lights, cap, "custom")


STRESS_GRIDS = ((16, 9, 24), (32, 18, 48))
STRESS_FPS = 60.0


def orbit_lights(rng: np.random.Generator, n_views: int, n_lights: int, n_blobs: int = 32, sigma: float = 8.0):
    """(lights (n_views * n_lights, 12), orbits (n_views * n_lights, 8)) float32:
    each view's lights around its own 32 Gaussian blobs, each light on a
    horizontal circle (CfLightOrbit: offset x/z, cos/sin of the angle per frame,
    centre xyz + position w).  Positions are centre + offset, rounded to float32
    like the device does."""
    centres = np.stack([rng.uniform(-100, 100, (n_views, n_blobs)), rng.uniform(0, 30, (n_views, n_blobs)),
                        rng.uniform(-100, 100, (n_views, n_blobs))], axis=2)
    which = rng.integers(0, n_blobs, size=(n_views, n_lights))
    centre = np.take_along_axis(centres, which[..., None], axis=1).reshape(-1, 3)
    centre = (centre + rng.normal(0.0, sigma, size=centre.shape)).astype(np.float32)
    n = n_views * n_lights
    radius = np.clip(rng.lognormal(math.log(3.0), 0.5, size=n), 0.5, 20.0).astype(np.float32)
    color = rng.uniform(0.0, 1.0, size=(n, 3)).astype(np.float32)
    rho = rng.uniform(1.0, 10.0, n)
    omega = rng.uniform(0.1, 2.0, n)
    phase = rng.uniform(0.0, 2.0 * math.pi, n)
    orbits = np.empty((n, 8), np.float32)
    orbits[:, 0] = rho * np.cos(phase)
    orbits[:, 1] = rho * np.sin(phase)
    orbits[:, 2] = np.cos(omega / STRESS_FPS)
    orbits[:, 3] = np.sin(omega / STRESS_FPS)
    orbits[:, 4:7] = centre
    orbits[:, 7] = 1.0
    pos = np.empty((n, 3), np.float32)
    pos[:, 0] = orbits[:, 4] + orbits[:, 0]
    pos[:, 1] = orbits[:, 5]
    pos[:, 2] = orbits[:, 6] + orbits[:, 1]
    return make_lights(pos, radius, color), orbits


_STRESS_PROJ = {}


def stress_ubo(view_index: int, epoch: int, camera) -> CfClusterForwardUBO:
    """The UBO of stress view `view_index` during projection epoch `epoch`."""
    grid = STRESS_GRIDS[(view_index + epoch) % 2]
    key = (grid, epoch % 2)
    if key not in _STRESS_PROJ:  # two projections per epoch: build each once
        t = 120 if grid == (16, 9, 24) else 80
        fovy = math.radians(45.0 if epoch % 2 == 0 else 60.0)
        _STRESS_PROJ[key] = bytes(cluster_forward_ubo(fovy, grid[0] * t, grid[1] * t, 0.1, 2000.0,
                                                      np.eye(4, dtype=np.float32), grid))
    u = CfClusterForwardUBO.from_buffer_copy(_STRESS_PROJ[key])
    u.cameraView[:] = np.asarray(camera, np.float32).T.reshape(-1).tolist()
    return u


def depth_log_uniform(rng: np.random.Generator, width: int, height: int, near: float, far: float,
                      far_plane_fraction: float = 0.0) -> np.ndarray:
    """A synthetic (height, width) ZO depth buffer: linear depth log-uniform in
    [near, far), turned into window depth by inverting Scene.frag's
    LinearDepth; a fraction of the pixels sits on the far plane (depth 1)."""
    lin = np.exp(rng.uniform(math.log(near), math.log(far), size=(height, width)))
    z = (near * far / lin - far) / (near - far)
    z = np.clip(z, 0.0, np.nextafter(np.float32(1.0), np.float32(0.0))).astype(np.float32)
    if far_plane_fraction > 0:
        z[rng.uniform(size=z.shape) < far_plane_fraction] = 1.0
    return z


def camera_position(ubo) -> np.ndarray:
    """World-space eye position of a UBO's view matrix (float64)."""
    view = np.array(list(ubo.cameraView), np.float64).reshape(4, 4).T
    return np.linalg.inv(view)[:3, 3]


def gbuffer(rng: np.random.Generator, ubo, far_plane_fraction: float = 0.0) -> np.ndarray:
    """A synthetic (height, width, 12) float32 G-buffer of CfGBufferTexel
    records for the UBO's screen: log-uniform linear depths, each texel's world
    position unprojected from its pixel centre and depth, a random unit normal
    facing the camera, albedo U[0,1]^3, metallic U[0,1], roughness U[0.05,1]."""
    w, h = int(ubo.screenSize[0]), int(ubo.screenSize[1])
    z = depth_log_uniform(rng, w, h, float(ubo.cameraNear), float(ubo.cameraFar), far_plane_fraction)
    inv_p = np.array(list(ubo.cameraInverseProjection), np.float64).reshape(4, 4).T
    view = np.array(list(ubo.cameraView), np.float64).reshape(4, 4).T
    xs = (np.arange(w) + 0.5) / w * 2.0 - 1.0
    ys = (np.arange(h) + 0.5) / h * 2.0 - 1.0
    clip = np.stack([np.broadcast_to(xs[None, :], (h, w)), np.broadcast_to(ys[:, None], (h, w)),
                     z.astype(np.float64), np.ones((h, w))], axis=-1)
    v = clip @ inv_p.T
    v = v / v[..., 3:4]
    world = v @ np.linalg.inv(view).T
    eye = camera_position(ubo)
    n = rng.normal(size=(h, w, 3))
    n /= np.linalg.norm(n, axis=-1, keepdims=True)
    to_eye = eye - world[..., :3]
    n = np.where((np.sum(n * to_eye, axis=-1) < 0)[..., None], -n, n)
    out = np.empty((h, w, 12), np.float32)
    out[..., 0:3] = world[..., :3]
    out[..., 3] = z
    out[..., 4:7] = n
    out[..., 7] = rng.uniform(0.0, 1.0, (h, w))
    out[..., 8:11] = rng.uniform(0.0, 1.0, (h, w, 3))
    out[..., 11] = rng.uniform(0.05, 1.0, (h, w))
    return out


def random_boxes(rng: np.random.Generator, n: int, extent: float = 200.0, size_lo: float = 0.5,
                 size_hi: float = 10.0) -> np.ndarray:
    """n axis-aligned boxes (CfAABB records, (n, 8) float32, w = 0) with
    centres uniform in [-extent, extent]^3 and sides uniform in
    [size_lo, size_hi] — the objects of a frustum-culling scene."""
    c = rng.uniform(-extent, extent, size=(n, 3))
    h = rng.uniform(size_lo, size_hi, size=(n, 3)) / 2.0
    out = np.zeros((n, 8), np.float32)
    out[:, 0:3] = c - h
    out[:, 4:7] = c + h
    return out
