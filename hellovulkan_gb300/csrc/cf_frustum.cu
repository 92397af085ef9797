// cf_frustum.cu — compute frustum culling of draw commands
// (HelloVulkan/Shaders/FrustumCulling.comp:14-57): one thread per AABB, the
// shader's two tests in its order, and a 4-byte store of the command's
// instanceCount.  Each box costs 32 bytes read and 4 written, so the kernel
// is HBM-bound at scale: boxes are read as two float4 per thread, coalesced,
// and the plane test takes one corner per plane instead of eight.
#include <cuda_runtime.h>

#include "cf_pinned_math.h"
#include "cf_runtime_internal.h"
#include "cfcull.h"

namespace {

constexpr unsigned kFullMask = 0xffffffffu;

// dot(plane, vec4(x, y, z, 1)) summed x, y, z, w in order
__device__ __forceinline__ float plane_dot(const float* p, float x, float y, float z)
{
    return cf_fadd(cf_fadd(cf_fadd(cf_fmul(p[0], x), cf_fmul(p[1], y)), cf_fmul(p[2], z)), cf_fmul(p[3], 1.0f));
}

// Coordinates below this magnitude keep every product and sum of a plane
// test finite (for planes of the same bound), so no rounded dot is NaN.
constexpr float kSafeMagnitude = 1e18f;

__device__ __forceinline__ bool safe(float v) { return fabsf(v) <= kSafeMagnitude; }  // false for NaN too

// IsBoxInFrustum (FrustumCulling.comp:14-45)
__device__ __forceinline__ bool box_in_frustum(const CfFrustum& f, float4 lo, float4 hi, bool planes_safe)
{
    if (planes_safe && safe(lo.x) && safe(lo.y) && safe(lo.z) && safe(hi.x) && safe(hi.y) && safe(hi.z)) {
        // All eight corners lie behind a plane exactly when the corner that
        // maximises the plane's dot does: with no NaN in play the rounded dot
        // (x, y, z, w summed in order) is monotone in each coordinate, rising
        // with it where the plane's coefficient is positive and falling where
        // it is negative (a zero coefficient contributes a zero either way).
#pragma unroll
        for (int i = 0; i < 6; ++i) {
            const float* p = f.planes[i];
            const float x = p[0] >= 0.0f ? fmaxf(lo.x, hi.x) : fminf(lo.x, hi.x);  // also for min > max
            const float y = p[1] >= 0.0f ? fmaxf(lo.y, hi.y) : fminf(lo.y, hi.y);
            const float z = p[2] >= 0.0f ? fmaxf(lo.z, hi.z) : fminf(lo.z, hi.z);
            if (plane_dot(p, x, y, z) < 0.0f) return false;
        }
    } else {  // the shader's eight-corner count
#pragma unroll
        for (int i = 0; i < 6; ++i) {
            const float* p = f.planes[i];
            int r = 0;
            r += plane_dot(p, lo.x, lo.y, lo.z) < 0.0f ? 1 : 0;
            r += plane_dot(p, hi.x, lo.y, lo.z) < 0.0f ? 1 : 0;
            r += plane_dot(p, lo.x, hi.y, lo.z) < 0.0f ? 1 : 0;
            r += plane_dot(p, hi.x, hi.y, lo.z) < 0.0f ? 1 : 0;
            r += plane_dot(p, lo.x, lo.y, hi.z) < 0.0f ? 1 : 0;
            r += plane_dot(p, hi.x, lo.y, hi.z) < 0.0f ? 1 : 0;
            r += plane_dot(p, lo.x, hi.y, hi.z) < 0.0f ? 1 : 0;
            r += plane_dot(p, hi.x, hi.y, hi.z) < 0.0f ? 1 : 0;
            if (r == 8) return false;
        }
    }
    int gx = 0, lx = 0, gy = 0, ly = 0, gz = 0, lz = 0;
#pragma unroll
    for (int i = 0; i < 8; ++i) {
        const float* c = f.corners[i];
        gx += c[0] > hi.x ? 1 : 0;
        lx += c[0] < lo.x ? 1 : 0;
        gy += c[1] > hi.y ? 1 : 0;
        ly += c[1] < lo.y ? 1 : 0;
        gz += c[2] > hi.z ? 1 : 0;
        lz += c[2] < lo.z ? 1 : 0;
    }
    return !(gx == 8 || lx == 8 || gy == 8 || ly == 8 || gz == 8 || lz == 8);
}

__global__ void __launch_bounds__(256) frustum_kernel(const CfFrustum f, bool planes_safe,
                                                      const float4* __restrict__ boxes, uint32_t n,
                                                      CfDrawIndirectCommand* __restrict__ cmds,
                                                      uint32_t* __restrict__ visible)
{
    const uint32_t i = blockIdx.x * 256u + threadIdx.x;
    bool in = false;
    if (i < n) {
        in = box_in_frustum(f, __ldg(&boxes[2 * (size_t)i]), __ldg(&boxes[2 * (size_t)i + 1]), planes_safe);
        cmds[i].instanceCount = in ? 1u : 0u;
    }
    if (visible) {
        const uint32_t m = __ballot_sync(kFullMask, in);
        if ((threadIdx.x & 31) == 0 && m) atomicAdd(visible, (uint32_t)__popc(m));
    }
}

}  // namespace

extern "C" int cf_frustum_cull(const CfFrustum* frustum, const CfAABB* d_boxes, uint32_t count,
                               CfDrawIndirectCommand* d_commands, uint32_t* d_visible, void* stream)
{
    using namespace cfrt;
    if (!frustum || (count && (!d_boxes || !d_commands)))
        return fail(CF_ERROR_INVALID_ARGUMENT, "cf_frustum_cull: null argument");
    if (reinterpret_cast<uintptr_t>(d_boxes) & 15) return fail(CF_ERROR_INVALID_ARGUMENT, "boxes must be 16-byte aligned");
    if (count == 0) return CF_SUCCESS;
    bool planes_safe = true;  // the positive-vertex test needs finite products, so bounded planes too
    for (int i = 0; i < 6; ++i)
        for (int c = 0; c < 4; ++c) {
            const float v = frustum->planes[i][c];
            planes_safe = planes_safe && v == v && v <= 1e18f && v >= -1e18f;
        }
    frustum_kernel<<<(count + 255) / 256, 256, 0, (cudaStream_t)stream>>>(
        *frustum, planes_safe, reinterpret_cast<const float4*>(d_boxes), count, d_commands, d_visible);
    const cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? CF_SUCCESS : cuda_fail(e, "frustum culling launch");
}
