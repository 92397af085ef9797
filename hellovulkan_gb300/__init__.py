"""GB300-native clustered-forward light culling (HelloVulkan's AABB generator and
light-culling compute passes) as sm_103a CUDA kernels behind a C ABI."""
from ._lib import (CfAABB, CfClusterForwardBuffers, CfClusterForwardUBO, CfError, CfLightCell, CfLightData,
                   LIB_PATH, check, lib)
from .camera import cluster_forward_ubo, look_at_rh, perspective_rh_zo, ubo_from_bytes, ubo_to_bytes

__all__ = [
    "CfAABB", "CfClusterForwardBuffers", "CfClusterForwardUBO", "CfError", "CfLightCell", "CfLightData", "LIB_PATH",
    "check", "lib", "cluster_forward_ubo", "look_at_rh", "perspective_rh_zo", "ubo_from_bytes", "ubo_to_bytes",
]
