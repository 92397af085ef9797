// cf_lookup.cu — the consumer side of the culled lists: Scene.frag's cluster
// lookup (HelloVulkan/Shaders/ClusteredForward/Scene.frag:54-78) for every
// pixel of a depth buffer, as a check that the (offset, count) cells and the
// index list drop into the reference's fragment pass, and the pass's direct
// clustered lighting (Radiance.glsl) over a G-buffer.
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

// Scene.frag:54-71 for the fragment at pixel (x, y) with window depth z: the
// linear depth and, when it lies inside the grid, the cluster index.
__device__ __forceinline__ bool fragment_cluster(const CfClusterForwardUBO& u, uint32_t x, uint32_t y, float z,
                                                 uint32_t* cluster, float* linear_depth)
{
    const float n = u.cameraNear, f = u.cameraFar;
    // LinearDepth (Scene.frag:54-57): near * far / (far + z * (near - far))
    const float lin = cf_fdiv(cf_fmul(n, f), cf_fadd(f, cf_fmul(z, cf_fsub(n, f))));
    // zIndex (Scene.frag:63): max(log2(linDepth) * sliceScaling + sliceBias, 0)
    const float zf = cf_glsl_max(cf_fadd(cf_fmul(cf_log2_pinned(lin), u.sliceScaling), u.sliceBias), 0.0f);
    // tile (Scene.frag:64-70): gl_FragCoord.xy / (screenSize / sliceCount)
    const float xf = cf_fdiv((float)x + 0.5f, cf_fdiv(u.screenSize[0], (float)u.sliceCountX));
    const float yf = cf_fdiv((float)y + 0.5f, cf_fdiv(u.screenSize[1], (float)u.sliceCountY));
    *linear_depth = lin;
    // NaN compares false: a NaN index leaves the grid too
    if (!(zf < (float)u.sliceCountZ && xf < (float)u.sliceCountX && yf < (float)u.sliceCountY)) return false;
    *cluster = (uint32_t)xf + (uint32_t)yf * u.sliceCountX + (uint32_t)zf * u.sliceCountX * u.sliceCountY;
    return true;
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
    uint32_t c = 0;
    float lin = 0.0f;
    const bool inside = fragment_cluster(u, x, y, z, &c, &lin);
    const float fx = (float)x + 0.5f, fy = (float)y + 0.5f;
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
    if (inside) {
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

struct V3 {
    float x, y, z;
};

__device__ __forceinline__ V3 v3_sub(V3 a, V3 b) { return {cf_fsub(a.x, b.x), cf_fsub(a.y, b.y), cf_fsub(a.z, b.z)}; }
__device__ __forceinline__ V3 v3_add(V3 a, V3 b) { return {cf_fadd(a.x, b.x), cf_fadd(a.y, b.y), cf_fadd(a.z, b.z)}; }
__device__ __forceinline__ float v3_dot(V3 a, V3 b)
{
    return cf_fadd(cf_fadd(cf_fmul(a.x, b.x), cf_fmul(a.y, b.y)), cf_fmul(a.z, b.z));
}
// normalize(v) = v / sqrt(dot(v, v)), componentwise division
__device__ __forceinline__ V3 v3_normalize(V3 v)
{
    const float l = cf_fsqrt(v3_dot(v, v));
    return {cf_fdiv(v.x, l), cf_fdiv(v.y, l), cf_fdiv(v.z, l)};
}

constexpr float kPi = 3.14159265358979323846f;  // PBRHeader.glsl's PI as a GLSL float

// Radiance (Radiance.glsl:2-57) of one light at world position P, in the
// shader's operation order; adds to lo.
__device__ __forceinline__ void radiance(const CfLightData* __restrict__ light, V3 P, V3 N, V3 V, V3 albedo, V3 F0,
                                         float metallic, float roughness, float alpha_r, float NoV,
                                         const CfPBRPushConstant& pc, V3& lo)
{
    const float4 q = __ldg(reinterpret_cast<const float4*>(&light->position[0]));
    const float4 col = __ldg(reinterpret_cast<const float4*>(&light->color[0]));
    const float radius = __ldg(&light->radius);
    const V3 d = v3_sub(V3{q.x, q.y, q.z}, P);
    const V3 L = v3_normalize(d);
    const V3 H = v3_normalize(v3_add(V, L));
    const float NoH = cf_glsl_max(v3_dot(N, H), 0.0f);
    const float NoL = cf_glsl_max(v3_dot(N, L), 0.0f);
    const float HoV = cf_glsl_max(v3_dot(H, V), 0.0f);
    const float dist = cf_fsqrt(v3_dot(d, d));
    const float att = cf_fdiv(cf_glsl_max(cf_fsub(1.0f, cf_fdiv(dist, radius)), 0.0f), cf_pow_pinned(dist, pc.lightFalloff));
    const V3 rad = {cf_fmul(cf_fmul(col.x, att), pc.lightIntensity), cf_fmul(cf_fmul(col.y, att), pc.lightIntensity),
                    cf_fmul(cf_fmul(col.z, att), pc.lightIntensity)};
    // DistributionGGX (PBRHeader.glsl:17-28)
    const float a = cf_fmul(roughness, roughness);
    const float a2 = cf_fmul(a, a);
    const float den0 = cf_fadd(cf_fmul(cf_fmul(NoH, NoH), cf_fsub(a2, 1.0f)), 1.0f);
    const float D = cf_fdiv(a2, cf_fmul(cf_fmul(kPi, den0), den0));
    // GeometrySchlickGGX (PBRHeader.glsl:41-46)
    const float one_a = cf_fsub(1.0f, alpha_r);
    const float G = cf_fmul(cf_fdiv(NoL, cf_fadd(cf_fmul(NoL, one_a), alpha_r)),
                            cf_fdiv(NoV, cf_fadd(cf_fmul(NoV, one_a), alpha_r)));
    // FresnelSchlick (PBRHeader.glsl:50-53)
    const float p5 = cf_pow_pinned(cf_glsl_min(cf_glsl_max(cf_fsub(1.0f, HoV), 0.0f), 1.0f), 5.0f);
    const V3 F = {cf_fadd(F0.x, cf_fmul(cf_fsub(1.0f, F0.x), p5)), cf_fadd(F0.y, cf_fmul(cf_fsub(1.0f, F0.y), p5)),
                  cf_fadd(F0.z, cf_fmul(cf_fsub(1.0f, F0.z), p5))};
    const float DG = cf_fmul(D, G);
    const float denom = cf_fadd(cf_fmul(cf_fmul(4.0f, NoV), NoL), 0.0001f);
    const float km = cf_fsub(1.0f, metallic);
    const float fc[3] = {F.x, F.y, F.z}, ac[3] = {albedo.x, albedo.y, albedo.z}, rc[3] = {rad.x, rad.y, rad.z};
    float out[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        const float spec = cf_fdiv(cf_fmul(DG, fc[c]), denom);
        const float kd = cf_fmul(cf_fsub(1.0f, fc[c]), km);
        const float diff = cf_fdiv(cf_fmul(kd, ac[c]), kPi);
        // Radiance's own Lo starts at vec3(0.0) (Radiance.glsl:13,55): the
        // term is added to zero before Scene.frag adds it to its Lo, which
        // turns a -0 term into +0
        out[c] = cf_fadd(0.0f, cf_fmul(cf_fmul(cf_fadd(diff, spec), rc[c]), NoL));
    }
    lo = V3{cf_fadd(lo.x, out[0]), cf_fadd(lo.y, out[1]), cf_fadd(lo.z, out[2])};
}

__global__ void __launch_bounds__(256) shade_kernel(const CfClusterForwardUBO u, const float3 cam,
                                                    const CfPBRPushConstant pc,
                                                    const CfGBufferTexel* __restrict__ gbuf, uint32_t width,
                                                    uint32_t n_pixels, const CfLightCell* __restrict__ cells,
                                                    const uint32_t* __restrict__ indices, uint64_t index_count,
                                                    const CfLightData* __restrict__ lights, uint32_t light_count,
                                                    float4* __restrict__ out)
{
    const uint32_t pix = blockIdx.x * 256u + threadIdx.x;
    if (pix >= n_pixels) return;
    const float4* t = reinterpret_cast<const float4*>(&gbuf[pix]);
    const float4 pos = __ldg(&t[0]), nrm = __ldg(&t[1]), alb = __ldg(&t[2]);
    const V3 P = {pos.x, pos.y, pos.z}, N = {nrm.x, nrm.y, nrm.z}, A = {alb.x, alb.y, alb.z};
    const float metallic = nrm.w, roughness = alb.w;
    // Scene.frag:82-115: V, NoV, F0 = mix(baseReflectivity, albedo, metallic), Lo = albedo * albedoMultipler
    const V3 V = v3_normalize(v3_sub(V3{cam.x, cam.y, cam.z}, P));
    const float NoV = cf_glsl_max(v3_dot(N, V), 0.0f);
    const float mi = cf_fsub(1.0f, metallic);
    const V3 F0 = {cf_fadd(cf_fmul(pc.baseReflectivity, mi), cf_fmul(A.x, metallic)),
                   cf_fadd(cf_fmul(pc.baseReflectivity, mi), cf_fmul(A.y, metallic)),
                   cf_fadd(cf_fmul(pc.baseReflectivity, mi), cf_fmul(A.z, metallic))};
    const float r1 = cf_fadd(roughness, 1.0f);
    const float alpha_r = cf_fdiv(cf_fmul(r1, r1), 8.0f);  // AlphaDirectLighting (PBRHeader.glsl:32-37)
    V3 lo = {cf_fmul(A.x, pc.albedoMultipler), cf_fmul(A.y, pc.albedoMultipler), cf_fmul(A.z, pc.albedoMultipler)};
    uint32_t c = 0;
    float lin = 0.0f;
    float alpha = 0.0f;
    if (fragment_cluster(u, pix % width, pix / width, pos.w, &c, &lin)) {
        const CfLightCell cell = cells[c];
        if ((uint64_t)cell.offset + cell.count <= index_count) {
            alpha = 1.0f;
            for (uint32_t j = 0; j < cell.count; ++j) {
                const uint32_t li = indices[cell.offset + j];
                if (li >= light_count) {
                    alpha = 0.0f;
                    continue;
                }
                radiance(&lights[li], P, N, V, A, F0, metallic, roughness, alpha_r, NoV, pc, lo);
            }
        }
    }
    out[pix] = make_float4(lo.x, lo.y, lo.z, alpha);
}

}  // namespace

extern "C" int cf_shade_clusters(const CfClusterForwardUBO* ubo, const float camera_position[3],
                                 const CfPBRPushConstant* pc, const CfGBufferTexel* d_gbuffer, uint32_t width,
                                 uint32_t height, const CfLightCell* d_cells, const uint32_t* d_indices,
                                 uint64_t index_count, const CfLightData* d_lights, uint32_t light_count,
                                 float* d_out, void* stream)
{
    using namespace cfrt;
    if (!ubo || !camera_position || !pc || !d_gbuffer || !d_cells || !d_out || (light_count && !d_lights) ||
        (index_count && !d_indices))
        return fail(CF_ERROR_INVALID_ARGUMENT, "cf_shade_clusters: null argument");
    uint32_t C = 0;
    const int st = validate_grid(ubo->sliceCountX, ubo->sliceCountY, ubo->sliceCountZ, 1, &C);
    if (st) return st;
    if ((float)width != ubo->screenSize[0] || (float)height != ubo->screenSize[1])
        return fail(CF_ERROR_INVALID_ARGUMENT, "G-buffer %ux%u does not match the UBO's screen %gx%g", width, height,
                    (double)ubo->screenSize[0], (double)ubo->screenSize[1]);
    const uint64_t n = (uint64_t)width * height;
    if (n == 0) return CF_SUCCESS;
    if (n > (1ull << 31)) return fail(CF_ERROR_INVALID_ARGUMENT, "G-buffer of %llu texels", (unsigned long long)n);
    if ((reinterpret_cast<uintptr_t>(d_lights) | reinterpret_cast<uintptr_t>(d_gbuffer) |
         reinterpret_cast<uintptr_t>(d_out)) & 15)
        return fail(CF_ERROR_INVALID_ARGUMENT, "lights, G-buffer and output must be 16-byte aligned");
    shade_kernel<<<(unsigned)((n + 255) / 256), 256, 0, (cudaStream_t)stream>>>(
        *ubo, make_float3(camera_position[0], camera_position[1], camera_position[2]), *pc, d_gbuffer, width,
        (uint32_t)n, d_cells, d_indices, index_count, d_lights, light_count, reinterpret_cast<float4*>(d_out));
    const cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? CF_SUCCESS : cuda_fail(e, "clustered shading launch");
}

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
