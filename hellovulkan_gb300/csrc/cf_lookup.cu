// cf_lookup.cu — the consumer side of the culled lists: Scene.frag's cluster
// lookup (HelloVulkan/Shaders/ClusteredForward/Scene.frag:54-78) for every
// pixel of a depth buffer, as a check that the (offset, count) cells and the
// index list drop into the reference's fragment pass.
//
// One thread per pixel: LinearDepth of the pixel's depth, the exponential
// slice index from log2 (pinned: cf_log2_pinned), the tile from the pixel
// centre, then the cluster's cell.  The fragment's view-space position is
// reconstructed the way AABBGenerator.comp's ScreenToView unprojects a screen
// point, and every listed light is tested for containing it (the lights a
// shading loop over the list would find in range).  In check mode every light
// of the set is tested as well, to count the ones the list lacks.
#include <cuda_runtime.h>

#include "cf_pinned_math.h"
#include "cf_runtime_internal.h"
#include "cfcull.h"

namespace {

// p = the view-space position of light L (cameraView * position, pinned order).
__device__ __forceinline__ void light_view(const float* V, const CfLightData* __restrict__ L, float p[3], float* r2)
{
    const float4 q = __ldg(reinterpret_cast<const float4*>(&L->position[0]));
    p[0] = cf_mat4_row(V, 0, q.x, q.y, q.z, q.w);
    p[1] = cf_mat4_row(V, 1, q.x, q.y, q.z, q.w);
    p[2] = cf_mat4_row(V, 2, q.x, q.y, q.z, q.w);
    const float r = __ldg(&L->radius);
    *r2 = cf_fmul(r, r);
}

// |f - c|^2 < r^2, summed x, y, z in order.
__device__ __forceinline__ bool contains(const float f[3], const float c[3], float r2)
{
    const float dx = cf_fsub(f[0], c[0]), dy = cf_fsub(f[1], c[1]), dz = cf_fsub(f[2], c[2]);
    return cf_fadd(cf_fadd(cf_fmul(dx, dx), cf_fmul(dy, dy)), cf_fmul(dz, dz)) < r2;
}

__global__ void __launch_bounds__(256) lookup_kernel(const CfClusterForwardUBO u, const float* __restrict__ depth,
                                                     uint32_t width, uint32_t n_pixels,
                                                     const CfLightCell* __restrict__ cells,
                                                     const uint32_t* __restrict__ indices, uint64_t index_count,
                                                     const CfLightData* __restrict__ lights, uint32_t light_count,
                                                     uint32_t cap, const float4* __restrict__ aabbs, int check_all,
                                                     CfFragmentSample* __restrict__ out)
{
    const uint32_t pix = blockIdx.x * 256u + threadIdx.x;
    if (pix >= n_pixels) return;
    const uint32_t x = pix % width, y = pix / width;
    const float z = __ldg(&depth[pix]);
    const float n = u.cameraNear, f = u.cameraFar;
    // LinearDepth (Scene.frag:54-57): near * far / (far + z * (near - far))
    const float lin = cf_fdiv(cf_fmul(n, f), cf_fadd(f, cf_fmul(z, cf_fsub(n, f))));
    // zIndex (Scene.frag:63): max(log2(linDepth) * sliceScaling + sliceBias, 0)
    const float zf = cf_glsl_max(cf_fadd(cf_fmul(cf_log2_pinned(lin), u.sliceScaling), u.sliceBias), 0.0f);
    // tile (Scene.frag:64-70): gl_FragCoord.xy / (screenSize / sliceCount)
    const float fx = (float)x + 0.5f, fy = (float)y + 0.5f;
    const float xf = cf_fdiv(fx, cf_fdiv(u.screenSize[0], (float)u.sliceCountX));
    const float yf = cf_fdiv(fy, cf_fdiv(u.screenSize[1], (float)u.sliceCountY));
    // the fragment in view space: ScreenToView of (fx / width, fy / height, z, 1)
    const float cx = cf_fsub(cf_fmul(cf_fdiv(fx, u.screenSize[0]), 2.0f), 1.0f);
    const float cy = cf_fsub(cf_fmul(cf_fdiv(fy, u.screenSize[1]), 2.0f), 1.0f);
    const float* IP = u.cameraInverseProjection;
    const float vw = cf_mat4_row(IP, 3, cx, cy, z, 1.0f);
    const float frag[3] = {cf_fdiv(cf_mat4_row(IP, 0, cx, cy, z, 1.0f), vw),
                           cf_fdiv(cf_mat4_row(IP, 1, cx, cy, z, 1.0f), vw),
                           cf_fdiv(cf_mat4_row(IP, 2, cx, cy, z, 1.0f), vw)};
    CfFragmentSample s;
    s.view_z = frag[2];
    s.linear_depth = lin;
    s.covering = 0;
    s.missing = 0;
    s.flags = 0;
    uint32_t off = 0, cnt = 0;
    const float* V = u.cameraView;
    // NaN compares false: a NaN index leaves the grid too
    if (zf < (float)u.sliceCountZ && xf < (float)u.sliceCountX && yf < (float)u.sliceCountY) {
        const uint32_t c = (uint32_t)xf + (uint32_t)yf * u.sliceCountX +
                           (uint32_t)zf * u.sliceCountX * u.sliceCountY;
        const CfLightCell cell = cells[c];
        off = cell.offset;
        cnt = cell.count;
        s.cluster = c;
        if ((uint64_t)off + cnt > index_count) {  // not a cell of this index list: read nothing through it
            s.flags |= CF_FRAGMENT_BAD_CELL;
            cnt = 0;
        }
        if (cnt >= cap) s.flags |= CF_FRAGMENT_CAPPED;
        if (aabbs) {
            const float4 lo = aabbs[2 * (size_t)c], hi = aabbs[2 * (size_t)c + 1];
            if (frag[0] < lo.x || frag[1] < lo.y || frag[2] < lo.z || frag[0] > hi.x || frag[1] > hi.y ||
                frag[2] > hi.z)
                s.flags |= CF_FRAGMENT_OUTSIDE_AABB;
        }
        for (uint32_t j = 0; j < cnt; ++j) {
            const uint32_t li = indices[off + j];
            if (li >= light_count) {
                s.flags |= CF_FRAGMENT_BAD_CELL;
                continue;
            }
            float p[3], r2;
            light_view(V, &lights[li], p, &r2);
            s.covering += contains(frag, p, r2) ? 1u : 0u;
        }
    } else {
        s.cluster = 0xFFFFFFFFu;
        s.flags |= CF_FRAGMENT_OUTSIDE_GRID;
    }
    s.offset = off;
    s.count = (s.flags & CF_FRAGMENT_BAD_CELL) ? 0u : cnt;
    if (check_all) {
        uint32_t j = 0;  // the list is ascending: walk it beside the lights
        for (uint32_t i = 0; i < light_count; ++i) {
            if (j < cnt && indices[off + j] == i) {
                ++j;
                continue;
            }
            float p[3], r2;
            light_view(V, &lights[i], p, &r2);
            s.missing += contains(frag, p, r2) ? 1u : 0u;
        }
    }
    out[pix] = s;
}

}  // namespace

extern "C" int cf_lookup_clusters(const CfClusterForwardUBO* ubo, const float* d_depth, uint32_t width, uint32_t height,
                                  const CfLightCell* d_cells, const uint32_t* d_indices, uint64_t index_count,
                                  const CfLightData* d_lights, uint32_t light_count, uint32_t cap,
                                  const CfAABB* d_aabbs, int check_all_lights, CfFragmentSample* d_out, void* stream)
{
    using namespace cfrt;
    if (!ubo || !d_depth || !d_cells || !d_out || (light_count && !d_lights) || (index_count && !d_indices))
        return fail(CF_ERROR_INVALID_ARGUMENT, "cf_lookup_clusters: null argument");
    uint32_t C = 0;
    const int st = validate_grid(ubo->sliceCountX, ubo->sliceCountY, ubo->sliceCountZ, cap ? cap : 1, &C);
    if (st) return st;
    if ((float)width != ubo->screenSize[0] || (float)height != ubo->screenSize[1])
        return fail(CF_ERROR_INVALID_ARGUMENT, "depth buffer %ux%u does not match the UBO's screen %gx%g", width, height,
                    (double)ubo->screenSize[0], (double)ubo->screenSize[1]);
    const uint64_t n = (uint64_t)width * height;
    if (n == 0) return CF_SUCCESS;
    if (n > (1ull << 31)) return fail(CF_ERROR_INVALID_ARGUMENT, "depth buffer of %llu pixels", (unsigned long long)n);
    if (reinterpret_cast<uintptr_t>(d_lights) & 15 || reinterpret_cast<uintptr_t>(d_aabbs) & 15)
        return fail(CF_ERROR_INVALID_ARGUMENT, "lights and AABBs must be 16-byte aligned");
    lookup_kernel<<<(unsigned)((n + 255) / 256), 256, 0, (cudaStream_t)stream>>>(
        *ubo, d_depth, width, (uint32_t)n, d_cells, d_indices, index_count, d_lights, light_count,
        cap ? cap : 0xFFFFFFFFu,
        reinterpret_cast<const float4*>(d_aabbs), check_all_lights, d_out);
    const cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? CF_SUCCESS : cuda_fail(e, "cluster lookup launch");
}
