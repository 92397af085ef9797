"""Builds the per-view ClusterForwardUBO from camera parameters.

Mirrors Camera::UpdateInternal and Camera::GetClusterForwardUBO
(HelloVulkan/Source/Camera.cpp:113-139, 178-197): a right-handed perspective
with depth in [0, 1] (the reference builds with GLM_FORCE_DEPTH_ZERO_TO_ONE,
HelloVulkan/CMakeLists.txt:24) whose [1][1] entry is negated for Vulkan's
flipped Y, its inverse, a right-handed look-at view matrix, and the slice
scale/bias of the fragment shader's cluster lookup.  glm is not available, so
the formulas are written out from their definitions; the culling kernels and
the oracle consume the same UBO bytes, so the rounding of this builder does
not affect parity.

Matrices are numpy float32 arrays M[row, col]; the UBO stores them
column-major (element (col, row) at col*4 + row), like GLSL and glm.
"""
from __future__ import annotations

import math

import numpy as np

from ._lib import CfClusterForwardUBO

UBO_BYTES = 176


def perspective_rh_zo(fovy: float, aspect: float, near: float, far: float) -> np.ndarray:
    t = math.tan(fovy / 2.0)
    P = np.zeros((4, 4), np.float64)
    P[0, 0] = 1.0 / (aspect * t)
    P[1, 1] = 1.0 / t
    P[2, 2] = far / (near - far)
    P[3, 2] = -1.0
    P[2, 3] = -(far * near) / (far - near)
    return P.astype(np.float32)


def look_at_rh(eye, center, up=(0.0, 1.0, 0.0)) -> np.ndarray:
    eye = np.asarray(eye, np.float64)
    f = np.asarray(center, np.float64) - eye
    f /= np.linalg.norm(f)
    s = np.cross(f, np.asarray(up, np.float64))
    s /= np.linalg.norm(s)
    u = np.cross(s, f)
    M = np.eye(4)
    M[0, :3] = s
    M[1, :3] = u
    M[2, :3] = -f
    M[0, 3] = -np.dot(s, eye)
    M[1, 3] = -np.dot(u, eye)
    M[2, 3] = np.dot(f, eye)
    return M.astype(np.float32)


def column_major(M: np.ndarray) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(M, np.float32).T).reshape(16)


def cluster_forward_ubo(fovy: float, width: float, height: float, near: float, far: float, view: np.ndarray,
                        grid=(16, 9, 24)) -> CfClusterForwardUBO:
    """Camera::GetClusterForwardUBO for the given camera and cluster grid."""
    P = perspective_rh_zo(fovy, float(width) / float(height), near, far)
    P[1, 1] *= -1.0
    inv_p = np.linalg.inv(P.astype(np.float64)).astype(np.float32)
    X, Y, Z = (int(g) for g in grid)
    zf = np.float32(Z)
    log2_fn = np.log2(np.float32(far) / np.float32(near)).astype(np.float32)
    log2_n = np.log2(np.float32(near)).astype(np.float32)
    u = CfClusterForwardUBO()
    u.cameraInverseProjection[:] = column_major(inv_p).tolist()
    u.cameraView[:] = column_major(view).tolist()
    u.screenSize[:] = [float(width), float(height)]
    u.sliceScaling = float(np.float32(zf / log2_fn))
    u.sliceBias = float(np.float32(-(zf * log2_n / log2_fn)))
    u.cameraNear = float(near)
    u.cameraFar = float(far)
    u.sliceCountX, u.sliceCountY, u.sliceCountZ = X, Y, Z
    return u


def ubo_to_bytes(u: CfClusterForwardUBO) -> np.ndarray:
    return np.frombuffer(bytes(u), np.uint8).copy()


def ubo_from_bytes(b) -> CfClusterForwardUBO:
    """A UBO from its 176 bytes (bytes, or a uint8 array as stored in fixtures)."""
    if not isinstance(b, (bytes, bytearray)):
        b = np.asarray(b, np.uint8).tobytes()
    return CfClusterForwardUBO.from_buffer_copy(bytes(b))


def ubo_grid(u: CfClusterForwardUBO):
    return int(u.sliceCountX), int(u.sliceCountY), int(u.sliceCountZ)


def frustum_ubo(fovy: float, aspect: float, near: float, far: float, view: np.ndarray):
    """Camera::GetFrustumUBO (Source/Camera.cpp:199-230): with PV = P * V (P
    with the Vulkan y flip), the planes are row 3 +/- rows 0, 1, 2 of PV (left,
    right, bottom, top, near, far) and the corners are the clip cube's
    (+/-1, +/-1, +/-1) unprojected by inverse(PV) and divided by w.  Computed in
    float64 and stored as float32 (the kernel and the oracle read the same
    bytes, so the rounding here does not affect parity)."""
    from ._lib import CfFrustum
    P = perspective_rh_zo(fovy, aspect, near, far).astype(np.float64)
    P[1, 1] *= -1.0
    PV = P @ np.asarray(view, np.float64)
    planes = [PV[3] + PV[0], PV[3] - PV[0], PV[3] + PV[1], PV[3] - PV[1], PV[3] + PV[2], PV[3] - PV[2]]
    inv = np.linalg.inv(PV)
    ndc = [(-1, -1, -1), (1, -1, -1), (1, 1, -1), (-1, 1, -1), (-1, -1, 1), (1, -1, 1), (1, 1, 1), (-1, 1, 1)]
    f = CfFrustum()
    for i, p in enumerate(planes):
        f.planes[i][:] = [float(np.float32(x)) for x in p]
    for i, c in enumerate(ndc):
        q = inv @ np.array([c[0], c[1], c[2], 1.0])
        f.corners[i][:] = [float(np.float32(x)) for x in q / q[3]]
    return f
