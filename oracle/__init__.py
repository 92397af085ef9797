"""Python access to the CPU oracle and to the reference shaders compiled as C++.

TEST INFRASTRUCTURE ONLY: imported by the tests, by ``__graft_entry__.smoke()``
and by the CPU-baseline leg of ``bench.py``, as the checker of the CUDA path.

* ``Oracle`` wraps ``oracle/_build/libcf_oracle.so`` (cf_oracle.cpp, the
  restatement of AABBGenerator.comp and LightCulling.comp).
* ``Reference`` wraps ``oracle/_ref/libcf_ref.so``: the reference's own
  shaders compiled as C++ (AABBGenerator.comp, LightCulling.comp,
  FrustumCulling.comp and Scene.frag's lookup and direct lighting; see
  oracle/build.py); available only where their generated translation unit
  exists.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

from . import build as _build

_P = C.c_void_p


def _ubo_ptr(ubo):
    return C.byref(ubo)


class Oracle:
    def __init__(self, path: Path | None = None):
        path = path or _build.build_oracle()
        L = C.CDLL(str(path))
        L.cfo_generate_aabbs.argtypes = [_P, _P, C.c_int]
        L.cfo_cull.argtypes = [_P, _P, _P, C.c_uint32, C.c_uint32, _P, _P, C.c_uint64,
                               C.POINTER(C.c_uint64), C.POINTER(C.c_uint64), C.c_int]
        for f in ("cfo_pow", "cfo_log2", "cfo_exp2"):
            getattr(L, f).restype = C.c_float
        L.cfo_pow.argtypes = [C.c_float, C.c_float]
        L.cfo_log2.argtypes = [C.c_float]
        L.cfo_exp2.argtypes = [C.c_float]
        L.cfo_lookup_clusters.argtypes = [_P, _P, C.c_uint32, C.c_uint32, _P, _P, C.c_uint64, _P, C.c_uint32,
                                          C.c_uint32, _P, C.c_int, _P, C.c_int]
        L.cfo_shade_clusters.argtypes = [_P, _P, _P, _P, C.c_uint32, C.c_uint32, _P, _P, C.c_uint64, _P, C.c_uint32,
                                         _P, C.c_int]
        L.cfo_frustum_cull.argtypes = [_P, _P, C.c_uint32, _P, C.c_int]
        L.cfo_fp_contract_probe.argtypes = []
        L.cfo_max_threads.argtypes = []
        self.lib = L

    def generate_aabbs(self, ubo, threads: int = 0) -> np.ndarray:
        C_ = int(ubo.sliceCountX) * int(ubo.sliceCountY) * int(ubo.sliceCountZ)
        out = np.empty((C_, 8), np.float32)
        st = self.lib.cfo_generate_aabbs(_ubo_ptr(ubo), out.ctypes.data, threads)
        assert st == 0, st
        return out

    def cull(self, ubo, aabbs: np.ndarray, lights: np.ndarray, cap: int = 150, threads: int = 0):
        """Returns (cells (C,2) uint32, indices (total,) uint32, executed_tests)."""
        C_ = int(ubo.sliceCountX) * int(ubo.sliceCountY) * int(ubo.sliceCountZ)
        aabbs = np.ascontiguousarray(aabbs, np.float32)
        lights = np.ascontiguousarray(lights, np.float32).reshape(-1, 12)
        cells = np.empty((C_, 2), np.uint32)
        cap_total = C_ * cap
        idx = np.empty(max(cap_total, 1), np.uint32)
        total = C.c_uint64()
        executed = C.c_uint64()
        st = self.lib.cfo_cull(_ubo_ptr(ubo), aabbs.ctypes.data, lights.ctypes.data if lights.size else None,
                               lights.shape[0], cap, cells.ctypes.data, idx.ctypes.data, cap_total,
                               C.byref(total), C.byref(executed), threads)
        assert st == 0, st
        return cells, idx[: total.value].copy(), int(executed.value)

    def lookup_clusters(self, ubo, depth: np.ndarray, cells: np.ndarray, indices: np.ndarray, lights: np.ndarray,
                        cap: int = 150, aabbs: np.ndarray | None = None, check_all: bool = True, threads: int = 0):
        """Scene.frag's cluster lookup per pixel (cfo_lookup_clusters); a
        structured array of shape depth.shape with CfFragmentSample fields."""
        from hellovulkan_gb300._lib import FRAGMENT_DTYPE
        depth = np.ascontiguousarray(depth, np.float32)
        h, w = depth.shape
        cells = np.ascontiguousarray(cells, np.uint32)
        indices = np.ascontiguousarray(indices, np.uint32)
        lights = np.ascontiguousarray(lights, np.float32).reshape(-1, 12)
        out = np.zeros(depth.shape, FRAGMENT_DTYPE)
        ab = None if aabbs is None else np.ascontiguousarray(aabbs, np.float32)
        st = self.lib.cfo_lookup_clusters(_ubo_ptr(ubo), depth.ctypes.data, w, h, cells.ctypes.data,
                                          indices.ctypes.data if indices.size else None, indices.size,
                                          lights.ctypes.data if lights.size else None, lights.shape[0], cap,
                                          None if ab is None else ab.ctypes.data, int(check_all), out.ctypes.data,
                                          threads)
        assert st == 0, st
        return out

    def shade_clusters(self, ubo, camera_position, pc, gbuffer: np.ndarray, cells: np.ndarray, indices: np.ndarray,
                       lights: np.ndarray, threads: int = 0) -> np.ndarray:
        """Scene.frag's direct clustered lighting per G-buffer texel
        (cfo_shade_clusters): gbuffer (h, w, 12) float32 CfGBufferTexel
        records; returns (h, w, 4) float32 (Lo, alpha)."""
        g = np.ascontiguousarray(gbuffer, np.float32)
        h, w = g.shape[:2]
        cells = np.ascontiguousarray(cells, np.uint32)
        indices = np.ascontiguousarray(indices, np.uint32)
        lights = np.ascontiguousarray(lights, np.float32).reshape(-1, 12)
        cam = (C.c_float * 3)(*[float(v) for v in camera_position[:3]])
        out = np.zeros((h, w, 4), np.float32)
        st = self.lib.cfo_shade_clusters(_ubo_ptr(ubo), cam, C.byref(pc), g.ctypes.data, w, h, cells.ctypes.data,
                                         indices.ctypes.data if indices.size else None, indices.size,
                                         lights.ctypes.data if lights.size else None, lights.shape[0],
                                         out.ctypes.data, threads)
        assert st == 0, st
        return out

    def frustum_cull(self, frustum, boxes: np.ndarray, threads: int = 0) -> np.ndarray:
        """FrustumCulling.comp per box (cfo_frustum_cull): the instanceCount
        (0 or 1) of each box's draw command."""
        b = np.ascontiguousarray(boxes, np.float32).reshape(-1, 8)
        out = np.zeros(b.shape[0], np.uint32)
        st = self.lib.cfo_frustum_cull(C.byref(frustum), b.ctypes.data if b.size else None, b.shape[0],
                                       out.ctypes.data if out.size else None, threads)
        assert st == 0, st
        return out

    def pow(self, x: float, y: float) -> float:
        return self.lib.cfo_pow(x, y)

    def log2(self, x: float) -> float:
        return self.lib.cfo_log2(x)

    def exp2(self, x: float) -> float:
        return self.lib.cfo_exp2(x)

    def fp_contract_probe(self) -> int:
        return self.lib.cfo_fp_contract_probe()

    def max_threads(self) -> int:
        return self.lib.cfo_max_threads()


class Reference:
    """The reference's shaders run on the CPU: AABBGenerator.comp,
    LightCulling.comp, FrustumCulling.comp, and Scene.frag's clustered lookup
    and direct lighting."""

    def __init__(self, path: Path):
        L = C.CDLL(str(path))
        L.cfr_generate_aabbs.argtypes = [_P, _P, C.c_int]
        L.cfr_cull.argtypes = [_P, _P, _P, C.c_uint32, _P, _P, C.c_uint64, C.POINTER(C.c_uint32), C.c_int]
        L.cfr_max_lights_per_cluster.restype = C.c_uint32
        L.cfr_frustum_cull.argtypes = [_P, _P, C.c_uint32, _P, C.c_int]
        L.cfr_lookup_fragments.argtypes = [_P, _P, C.c_uint32, C.c_uint32, _P, C.c_uint32, _P, _P, _P, _P, C.c_int]
        L.cfr_shade_fragments.argtypes = [_P, _P, _P, _P, C.c_uint32, C.c_uint32, _P, C.c_uint32, _P, C.c_uint64, _P,
                                          C.c_uint32, _P, _P, C.c_int]
        self.lib = L
        self.cap = int(L.cfr_max_lights_per_cluster())

    @classmethod
    def load(cls):
        """The reference library, or None where it cannot be built."""
        try:
            p = _build.build_ref()
        except Exception:
            return None
        return cls(p) if p else None

    def generate_aabbs(self, ubo, threads: int = 1) -> np.ndarray:
        C_ = int(ubo.sliceCountX) * int(ubo.sliceCountY) * int(ubo.sliceCountZ)
        out = np.empty((C_, 8), np.float32)
        assert self.lib.cfr_generate_aabbs(_ubo_ptr(ubo), out.ctypes.data, threads) == 0
        return out

    def cull(self, ubo, aabbs: np.ndarray, lights: np.ndarray, threads: int = 1):
        """Returns (cells (C,2) uint32, indices (total,) uint32); threads=1 runs
        the workgroups in index order, so offsets are the cluster-order scan."""
        C_ = int(ubo.sliceCountX) * int(ubo.sliceCountY) * int(ubo.sliceCountZ)
        aabbs = np.ascontiguousarray(aabbs, np.float32)
        lights = np.ascontiguousarray(lights, np.float32).reshape(-1, 12)
        cells = np.empty((C_, 2), np.uint32)
        cap_total = C_ * self.cap
        idx = np.zeros(max(cap_total, 1), np.uint32)
        total = C.c_uint32()
        st = self.lib.cfr_cull(_ubo_ptr(ubo), aabbs.ctypes.data, lights.ctypes.data if lights.size else None,
                               lights.shape[0], cells.ctypes.data, idx.ctypes.data, cap_total, C.byref(total), threads)
        assert st == 0, st
        return cells, idx[: total.value].copy()

    def frustum_cull(self, frustum, boxes: np.ndarray, threads: int = 1) -> np.ndarray:
        """FrustumCulling.comp's instanceCount (0 or 1) for each box."""
        b = np.ascontiguousarray(boxes, np.float32).reshape(-1, 8)
        out = np.zeros(b.shape[0], np.uint32)
        st = self.lib.cfr_frustum_cull(C.byref(frustum), b.ctypes.data if b.size else None, b.shape[0],
                                       out.ctypes.data if out.size else None, threads)
        assert st == 0, st
        return out

    def lookup_fragments(self, ubo, depth: np.ndarray, cells: np.ndarray, threads: int = 1):
        """Scene.frag's clustered lookup per pixel: dict of cluster, count,
        offset (uint32) and linear_depth (float32), each shaped like depth.
        A fragment past the grid reads a zero cell (robust buffer access)."""
        depth = np.ascontiguousarray(depth, np.float32)
        h, w = depth.shape
        cells = np.ascontiguousarray(cells, np.uint32).reshape(-1, 2)
        out = {k: np.zeros(depth.shape, np.uint32) for k in ("cluster", "count", "offset")}
        out["linear_depth"] = np.zeros(depth.shape, np.float32)
        st = self.lib.cfr_lookup_fragments(_ubo_ptr(ubo), depth.ctypes.data, w, h, cells.ctypes.data, cells.shape[0],
                                           out["cluster"].ctypes.data, out["count"].ctypes.data,
                                           out["offset"].ctypes.data, out["linear_depth"].ctypes.data, threads)
        assert st == 0, st
        return out

    def shade_fragments(self, ubo, camera_position, pc, gbuffer: np.ndarray, cells: np.ndarray, indices: np.ndarray,
                        lights: np.ndarray, threads: int = 1):
        """Scene.frag's direct clustered lighting per G-buffer texel: (Lo as
        (h, w, 3) float32, the looked-up cluster index as (h, w) uint32)."""
        g = np.ascontiguousarray(gbuffer, np.float32)
        h, w = g.shape[:2]
        cells = np.ascontiguousarray(cells, np.uint32).reshape(-1, 2)
        indices = np.ascontiguousarray(indices, np.uint32)
        lights = np.ascontiguousarray(lights, np.float32).reshape(-1, 12)
        cam = (C.c_float * 3)(*[float(v) for v in camera_position[:3]])
        rgb = np.zeros((h, w, 3), np.float32)
        cl = np.zeros((h, w), np.uint32)
        st = self.lib.cfr_shade_fragments(_ubo_ptr(ubo), cam, C.byref(pc), g.ctypes.data, w, h, cells.ctypes.data,
                                          cells.shape[0], indices.ctypes.data if indices.size else None, indices.size,
                                          lights.ctypes.data if lights.size else None, lights.shape[0],
                                          rgb.ctypes.data, cl.ctypes.data, threads)
        assert st == 0, st
        return rgb, cl


def jitter_lights(lights: np.ndarray, seed: int, sigma: float) -> np.ndarray:
    """Host restatement of the server's light jitter (cf_server_jitter_light_set,
    hellovulkan_gb300/csrc/cf_kernels.cu jitter_light), bit for bit."""
    L = np.array(lights, np.float32, copy=True).reshape(-1, 12)
    n = L.shape[0]
    i = np.arange(n, dtype=np.uint64)
    with np.errstate(over="ignore"):
        for a in range(3):
            s = np.zeros(n, np.float32)
            for k in range(12):
                x = np.uint64(seed) + i * np.uint64(0x9E3779B97F4A7C15) + np.uint64(a * 12 + k) * np.uint64(
                    0xD1B54A32D192ED03)
                x ^= x >> np.uint64(30)
                x *= np.uint64(0xBF58476D1CE4E5B9)
                x ^= x >> np.uint64(27)
                x *= np.uint64(0x94D049BB133111EB)
                x ^= x >> np.uint64(31)
                s = s + (x >> np.uint64(40)).astype(np.float32) * np.float32(2.0 ** -24)
            L[:, a] = L[:, a] + np.float32(sigma) * (s - np.float32(6.0))
    return L


def animate_orbits(orbits: np.ndarray, frames: int):
    """Host restatement of cf_animate_light_orbits (hellovulkan_gb300/csrc/
    cf_kernels.cu orbit_kernel), bit for bit: returns (orbits after `frames`
    steps, positions (n, 4)).  numpy float32 products and sums round to nearest
    one operation at a time, as the kernel's __fmul_rn / __fadd_rn do."""
    o = np.array(orbits, np.float32, copy=True).reshape(-1, 8)
    x, z, c, s = o[:, 0].copy(), o[:, 1].copy(), o[:, 2], o[:, 3]
    for _ in range(frames):
        x, z = c * x - s * z, s * x + c * z
    o[:, 0], o[:, 1] = x, z
    pos = np.stack([o[:, 4] + x, o[:, 5], o[:, 6] + z, o[:, 7]], axis=1).astype(np.float32)
    return o, pos
