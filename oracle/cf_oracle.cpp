/*
 * cf_oracle.cpp — CPU oracle for the clustered-forward light-culling path.
 *
 * TEST INFRASTRUCTURE ONLY.  Only the tests, the smoke check and the CPU
 * baseline leg of the benchmark load this library, always as the checker of
 * the CUDA path and never as a part of it.
 *
 * A scalar restatement of the two compute shaders of HelloVulkan's clustered
 * forward pass, in the shaders' own operation order:
 *
 *   cfo_generate_aabbs  HelloVulkan/Shaders/ClusteredForward/AABBGenerator.comp:18-89
 *   cfo_cull            HelloVulkan/Shaders/ClusteredForward/LightCulling.comp:26-87
 *   cfo_lookup_clusters HelloVulkan/Shaders/ClusteredForward/Scene.frag:54-78 (the consumer's
 *                       cluster lookup), a check of the culled lists
 *   cfo_shade_clusters  Scene.frag:82-135 + Radiance.glsl:2-57 (direct clustered lighting)
 *   cfo_frustum_cull    HelloVulkan/Shaders/FrustumCulling.comp:14-57
 *
 * with the three implementation-defined parts of GLSL pinned exactly as in
 * include/cf_pinned_math.h (pow, mat4*vec4 summation order, no FMA).  This
 * file restates the mat4*vec4 order and the GLSL min/max with its own code
 * and takes only pow from that header, because pow has no unique value.
 *
 * The reference reserves each cluster's slice of the index list with an
 * atomicAdd on a global counter (LightCulling.comp:79), so its offsets depend
 * on scheduling.  The oracle assigns offsets by an exclusive scan of the
 * per-cluster counts in cluster-index order, which is what the reference
 * produces when its workgroups run one after another in index order.
 *
 * Build: oracle/build.py (g++ -O2 -ffp-contract=off, OpenMP over clusters).
 */
#include <cstdint>
#include <cstring>
#include <vector>
#include <omp.h>

#include "cf_types.h"
#include "cf_pinned_math.h"

namespace {

struct V3 { float x, y, z; };
struct V4 { float x, y, z, w; };

/* GLSL M * v, column-major M, summed left to right (no FMA: -ffp-contract=off). */
inline V4 mat_mul(const float* m, const V4& v)
{
    V4 r;
    r.x = ((m[0] * v.x + m[4] * v.y) + m[8] * v.z) + m[12] * v.w;
    r.y = ((m[1] * v.x + m[5] * v.y) + m[9] * v.z) + m[13] * v.w;
    r.z = ((m[2] * v.x + m[6] * v.y) + m[10] * v.z) + m[14] * v.w;
    r.w = ((m[3] * v.x + m[7] * v.y) + m[11] * v.z) + m[15] * v.w;
    return r;
}

inline float gmin(float x, float y) { return (y < x) ? y : x; }
inline float gmax(float x, float y) { return (x < y) ? y : x; }
inline V3 gmin3(const V3& a, const V3& b) { return {gmin(a.x, b.x), gmin(a.y, b.y), gmin(a.z, b.z)}; }
inline V3 gmax3(const V3& a, const V3& b) { return {gmax(a.x, b.x), gmax(a.y, b.y), gmax(a.z, b.z)}; }

/* AABBGenerator.comp:18-32 */
inline V4 screen_to_view(const CfClusterForwardUBO& u, const V4& screen)
{
    const V4 clip = {screen.x * 2.0f - 1.0f, screen.y * 2.0f - 1.0f, screen.z, screen.w};
    V4 view = mat_mul(u.cameraInverseProjection, clip);
    const float w = view.w;
    view.x = view.x / w;
    view.y = view.y / w;
    view.z = view.z / w;
    view.w = view.w / w;
    return view;
}

/* AABBGenerator.comp:34-37: (incident * zOffset) / incident.z */
inline V3 ray_intersect_z_plane(const V3& incident, float z_offset)
{
    return {(incident.x * z_offset) / incident.z,
            (incident.y * z_offset) / incident.z,
            (incident.z * z_offset) / incident.z};
}

/* AABBGenerator.comp:39-89 for workgroup (i, j, k). */
inline void aabb_one(const CfClusterForwardUBO& u, uint32_t i, uint32_t j, uint32_t k, CfAABB* out)
{
    const float npx = 1.0f / float(u.sliceCountX);
    const float npy = 1.0f / float(u.sliceCountY);
    const V4 max_ss = {(float(i) + 1.0f) * npx, (float(j) + 1.0f) * npy, 0.0f, 1.0f};
    const V4 min_ss = {float(i) * npx, float(j) * npy, 0.0f, 1.0f};
    const V4 mx = screen_to_view(u, max_ss);
    const V4 mn = screen_to_view(u, min_ss);
    const V3 max_vs = {mx.x, mx.y, mx.z};
    const V3 min_vs = {mn.x, mn.y, mn.z};
    const float ratio = u.cameraFar / u.cameraNear;
    const float tile_near = -u.cameraNear * cf_pow_pinned(ratio, float(k) / float(u.sliceCountZ));
    const float tile_far = -u.cameraNear * cf_pow_pinned(ratio, float(k + 1u) / float(u.sliceCountZ));
    const V3 min_near = ray_intersect_z_plane(min_vs, tile_near);
    const V3 min_far = ray_intersect_z_plane(min_vs, tile_far);
    const V3 max_near = ray_intersect_z_plane(max_vs, tile_near);
    const V3 max_far = ray_intersect_z_plane(max_vs, tile_far);
    const V3 lo = gmin3(gmin3(min_near, min_far), gmin3(max_near, max_far));
    const V3 hi = gmax3(gmax3(min_near, min_far), gmax3(max_near, max_far));
    out->minPoint[0] = lo.x; out->minPoint[1] = lo.y; out->minPoint[2] = lo.z; out->minPoint[3] = 0.0f;
    out->maxPoint[0] = hi.x; out->maxPoint[1] = hi.y; out->maxPoint[2] = hi.z; out->maxPoint[3] = 0.0f;
}

/* LightCulling.comp:26-47 */
inline float sq_dist_point_aabb(const float p[3], const CfAABB& cell)
{
    float sq = 0.0f;
    for (int a = 0; a < 3; ++a) {
        const float v = p[a];
        if (v < cell.minPoint[a]) {
            const float d = cell.minPoint[a] - v;
            sq += d * d;
        } else if (v > cell.maxPoint[a]) {
            const float d = cell.maxPoint[a] - v;
            sq += d * d;
        }
    }
    return sq;
}

}  // namespace

extern "C" {

int cfo_generate_aabbs(const CfClusterForwardUBO* ubo, CfAABB* out, int threads)
{
    if (!ubo || !out) return 1;
    const uint32_t X = ubo->sliceCountX, Y = ubo->sliceCountY, Z = ubo->sliceCountZ;
    const int64_t C = int64_t(X) * Y * Z;
    if (threads <= 0) threads = omp_get_max_threads();
#pragma omp parallel for num_threads(threads) schedule(static)
    for (int64_t c = 0; c < C; ++c) {
        const uint32_t i = uint32_t(c % X), j = uint32_t((c / X) % Y), k = uint32_t(c / (int64_t(X) * Y));
        aabb_one(*ubo, i, j, k, out + c);
    }
    return 0;
}

/*
 * LightCulling.comp:59-87 for every cluster.  Writes cells[C] and the packed
 * index list; *total_out = number of indices written.  *executed_tests_out =
 * sum over clusters of the number of TestSphereAABB calls the reference loop
 * makes (it stops after the cap-th hit).  Returns 0, 1 (bad argument) or
 * 2 (index_capacity too small).
 */
int cfo_cull(const CfClusterForwardUBO* ubo, const CfAABB* aabbs, const CfLightData* lights,
             uint32_t light_count, uint32_t cap, CfLightCell* cells, uint32_t* indices,
             uint64_t index_capacity, uint64_t* total_out, uint64_t* executed_tests_out,
             int threads)
{
    if (!ubo || !aabbs || !cells || cap == 0 || (light_count && !lights)) return 1;
    const int64_t C = int64_t(ubo->sliceCountX) * ubo->sliceCountY * ubo->sliceCountZ;
    if (threads <= 0) threads = omp_get_max_threads();
    std::vector<uint32_t> stage(static_cast<size_t>(C) * cap);
    std::vector<uint32_t> count(static_cast<size_t>(C));
    uint64_t executed = 0;
    const float* V = ubo->cameraView;
#pragma omp parallel for num_threads(threads) schedule(dynamic, 8) reduction(+ : executed)
    for (int64_t c = 0; c < C; ++c) {
        const CfAABB cell = aabbs[c];
        uint32_t* mine = stage.data() + size_t(c) * cap;
        uint32_t n = 0;
        uint32_t i = 0;
        for (; i < light_count && n < cap; ++i) {
            const CfLightData& L = lights[i];
            const V4 pw = {L.position[0], L.position[1], L.position[2], L.position[3]};
            const V4 pv = mat_mul(V, pw);
            const float p[3] = {pv.x, pv.y, pv.z};
            const float sq = sq_dist_point_aabb(p, cell);
            if (sq < L.radius * L.radius) mine[n++] = i;
        }
        executed += i;
        count[size_t(c)] = n;
    }
    uint64_t off = 0;
    for (int64_t c = 0; c < C; ++c) {
        cells[c].offset = uint32_t(off);
        cells[c].count = count[size_t(c)];
        off += count[size_t(c)];
    }
    if (total_out) *total_out = off;
    if (executed_tests_out) *executed_tests_out = executed;
    if (off > index_capacity) return 2;
    if (off && !indices) return 1;
#pragma omp parallel for num_threads(threads) schedule(static)
    for (int64_t c = 0; c < C; ++c) {
        if (cells[c].count)
            memcpy(indices + cells[c].offset, stage.data() + size_t(c) * cap, sizeof(uint32_t) * cells[c].count);
    }
    return 0;
}

/*
 * Scene.frag:54-78's cluster lookup for every pixel of a depth buffer
 * (row-major from the top row, fragment at the pixel centre), with log2
 * pinned like the kernel (cf_log2_pinned), the fragment unprojected like
 * AABBGenerator.comp:18-32's ScreenToView, and the containment test
 * |fragment - light|^2 < r^2 summed x, y, z.  Same outputs as
 * cf_lookup_clusters (include/cfcull.h).  Returns 0 or 1 (bad argument).
 */
int cfo_lookup_clusters(const CfClusterForwardUBO* ubo, const float* depth, uint32_t width, uint32_t height,
                        const CfLightCell* cells, const uint32_t* indices, uint64_t index_count,
                        const CfLightData* lights, uint32_t light_count, uint32_t cap, const CfAABB* aabbs,
                        int check_all, CfFragmentSample* out, int threads)
{
    if (!ubo || !depth || !cells || !out) return 1;
    const CfClusterForwardUBO& u = *ubo;
    const uint32_t X = u.sliceCountX, Y = u.sliceCountY, Z = u.sliceCountZ;
    if (cap == 0) cap = 0xFFFFFFFFu;
    if (threads <= 0) threads = omp_get_max_threads();
    const int64_t n = int64_t(width) * height;
    const float* V = u.cameraView;
#pragma omp parallel for num_threads(threads) schedule(dynamic, 256)
    for (int64_t pix = 0; pix < n; ++pix) {
        const float x = float(uint32_t(pix % width)) + 0.5f, y = float(uint32_t(pix / width)) + 0.5f;
        const float zd = depth[pix];
        const float near_ = u.cameraNear, far_ = u.cameraFar;
        const float lin = near_ * far_ / (far_ + zd * (near_ - far_));
        const float zi = gmax(cf_log2_pinned(lin) * u.sliceScaling + u.sliceBias, 0.0f);
        const float tile_x = u.screenSize[0] / float(X), tile_y = u.screenSize[1] / float(Y);
        const float xi = x / tile_x, yi = y / tile_y;
        const V4 screen = {x / u.screenSize[0], y / u.screenSize[1], zd, 1.0f};
        const V4 clip = {screen.x * 2.0f - 1.0f, screen.y * 2.0f - 1.0f, screen.z, screen.w};
        const V4 vv = mat_mul(u.cameraInverseProjection, clip);
        const float fp[3] = {vv.x / vv.w, vv.y / vv.w, vv.z / vv.w};
        CfFragmentSample r{};
        r.view_z = fp[2];
        r.linear_depth = lin;
        uint32_t first = 0, count = 0;
        const bool inside = zi < float(Z) && xi < float(X) && yi < float(Y);
        if (inside) {
            const uint32_t c = uint32_t(xi) + uint32_t(yi) * X + uint32_t(zi) * X * Y;
            r.cluster = c;
            first = cells[c].offset;
            count = cells[c].count;
            if (uint64_t(first) + count > index_count) {
                r.flags |= CF_FRAGMENT_BAD_CELL;
                count = 0;
            }
            if (count >= cap) r.flags |= CF_FRAGMENT_CAPPED;
            if (aabbs) {
                const CfAABB& b = aabbs[c];
                bool out_box = false;
                for (int a = 0; a < 3; ++a) out_box |= fp[a] < b.minPoint[a] || fp[a] > b.maxPoint[a];
                if (out_box) r.flags |= CF_FRAGMENT_OUTSIDE_AABB;
            }
        } else {
            r.cluster = 0xFFFFFFFFu;
            r.flags |= CF_FRAGMENT_OUTSIDE_GRID;
        }
        auto covers = [&](uint32_t li) {
            const CfLightData& L = lights[li];
            const V4 pv = mat_mul(V, V4{L.position[0], L.position[1], L.position[2], L.position[3]});
            const float dx = fp[0] - pv.x, dy = fp[1] - pv.y, dz = fp[2] - pv.z;
            return (dx * dx + dy * dy) + dz * dz < L.radius * L.radius;
        };
        std::vector<char> listed(check_all ? light_count : 0, 0);
        for (uint32_t j = 0; j < count; ++j) {
            const uint32_t li = indices[first + j];
            if (li >= light_count) {
                r.flags |= CF_FRAGMENT_BAD_CELL;
                continue;
            }
            if (check_all) listed[li] = 1;
            r.covering += covers(li) ? 1u : 0u;
        }
        r.offset = first;
        r.count = (r.flags & CF_FRAGMENT_BAD_CELL) ? 0u : count;
        if (check_all)
            for (uint32_t i = 0; i < light_count; ++i)
                if (!listed[i] && covers(i)) r.missing++;
        out[pix] = r;
    }
    return 0;
}

/*
 * Scene.frag:82-135's direct clustered lighting per G-buffer texel (the
 * lookup as in cfo_lookup_clusters), Radiance.glsl:2-57 and the PBRHeader.glsl
 * helpers in their operation order, with normalize(v) = v / sqrt(dot(v, v)),
 * length = sqrt(dot), pow = cf_pow_pinned (the pins cf_shade_clusters states).
 * out: width x height x 4 floats.  Returns 0 or 1 (bad argument).
 */
int cfo_shade_clusters(const CfClusterForwardUBO* ubo, const float* cam, const CfPBRPushConstant* pc,
                       const CfGBufferTexel* gbuf, uint32_t width, uint32_t height, const CfLightCell* cells,
                       const uint32_t* indices, uint64_t index_count, const CfLightData* lights, uint32_t light_count,
                       float* out, int threads)
{
    if (!ubo || !cam || !pc || !gbuf || !cells || !out) return 1;
    const CfClusterForwardUBO& u = *ubo;
    const uint32_t X = u.sliceCountX, Y = u.sliceCountY, Z = u.sliceCountZ;
    const float pi = 3.14159265358979323846f;
    if (threads <= 0) threads = omp_get_max_threads();
    const int64_t n = int64_t(width) * height;
    auto dot3 = [](const float a[3], const float b[3]) { return (a[0] * b[0] + a[1] * b[1]) + a[2] * b[2]; };
    auto normalize3 = [&](const float v[3], float r[3]) {
        const float l = cf_fsqrt(dot3(v, v));
        for (int c = 0; c < 3; ++c) r[c] = v[c] / l;
    };
#pragma omp parallel for num_threads(threads) schedule(dynamic, 256)
    for (int64_t pix = 0; pix < n; ++pix) {
        const CfGBufferTexel& t = gbuf[pix];
        const float P[3] = {t.position[0], t.position[1], t.position[2]};
        const float N[3] = {t.normal[0], t.normal[1], t.normal[2]};
        const float A[3] = {t.albedo[0], t.albedo[1], t.albedo[2]};
        const float metallic = t.normal[3], roughness = t.albedo[3];
        const float cp[3] = {cam[0] - P[0], cam[1] - P[1], cam[2] - P[2]};
        float V[3];
        normalize3(cp, V);
        const float NoV = gmax(dot3(N, V), 0.0f);
        float F0[3], lo[3];
        for (int c = 0; c < 3; ++c) {
            F0[c] = pc->baseReflectivity * (1.0f - metallic) + A[c] * metallic;  // mix(x, y, a)
            lo[c] = A[c] * pc->albedoMultipler;
        }
        const float alpha_r = ((roughness + 1.0f) * (roughness + 1.0f)) / 8.0f;
        float alpha = 0.0f;
        // the cluster lookup
        const float near_ = u.cameraNear, far_ = u.cameraFar, zd = t.position[3];
        const float lin = near_ * far_ / (far_ + zd * (near_ - far_));
        const float zi = gmax(cf_log2_pinned(lin) * u.sliceScaling + u.sliceBias, 0.0f);
        const float x = float(uint32_t(pix % width)) + 0.5f, y = float(uint32_t(pix / width)) + 0.5f;
        const float xi = x / (u.screenSize[0] / float(X)), yi = y / (u.screenSize[1] / float(Y));
        if (zi < float(Z) && xi < float(X) && yi < float(Y)) {
            const CfLightCell cell = cells[uint32_t(xi) + uint32_t(yi) * X + uint32_t(zi) * X * Y];
            if (uint64_t(cell.offset) + cell.count <= index_count) {
                alpha = 1.0f;
                for (uint32_t j = 0; j < cell.count; ++j) {
                    const uint32_t li = indices[cell.offset + j];
                    if (li >= light_count) {
                        alpha = 0.0f;
                        continue;
                    }
                    const CfLightData& L = lights[li];
                    const float d[3] = {L.position[0] - P[0], L.position[1] - P[1], L.position[2] - P[2]};
                    float Lv[3], h0[3], H[3];
                    normalize3(d, Lv);
                    for (int c = 0; c < 3; ++c) h0[c] = V[c] + Lv[c];
                    normalize3(h0, H);
                    const float NoH = gmax(dot3(N, H), 0.0f);
                    const float NoL = gmax(dot3(N, Lv), 0.0f);
                    const float HoV = gmax(dot3(H, V), 0.0f);
                    const float dist = cf_fsqrt(dot3(d, d));
                    const float att = gmax(1.0f - dist / L.radius, 0.0f) / cf_pow_pinned(dist, pc->lightFalloff);
                    const float a = roughness * roughness, a2 = a * a;
                    float den = (NoH * NoH) * (a2 - 1.0f) + 1.0f;
                    den = pi * den * den;
                    const float D = a2 / den;
                    const float G = (NoL / (NoL * (1.0f - alpha_r) + alpha_r)) * (NoV / (NoV * (1.0f - alpha_r) + alpha_r));
                    const float p5 = cf_pow_pinned(gmin(gmax(1.0f - HoV, 0.0f), 1.0f), 5.0f);
                    const float denom = 4.0f * NoV * NoL + 0.0001f;
                    for (int c = 0; c < 3; ++c) {
                        const float F = F0[c] + (1.0f - F0[c]) * p5;
                        const float spec = D * G * F / denom;
                        const float kd = (1.0f - F) * (1.0f - metallic);
                        const float diff = kd * A[c] / pi;
                        const float rad = L.color[c] * att * pc->lightIntensity;
                        // Radiance returns its own Lo, vec3(0.0) plus the term
                        // (Radiance.glsl:13,55): 0 + (-0) is +0
                        lo[c] = lo[c] + (0.0f + (diff + spec) * rad * NoL);
                    }
                }
            }
        }
        out[4 * pix + 0] = lo[0];
        out[4 * pix + 1] = lo[1];
        out[4 * pix + 2] = lo[2];
        out[4 * pix + 3] = alpha;
    }
    return 0;
}

/*
 * FrustumCulling.comp:14-57 for n boxes: instance[i] = 1 when box i may meet
 * the frustum, else 0; dot(plane, (x, y, z, 1)) summed x, y, z, w in order.
 */
int cfo_frustum_cull(const CfFrustum* f, const CfAABB* boxes, uint32_t n, uint32_t* instance, int threads)
{
    if (!f || (n && (!boxes || !instance))) return 1;
    if (threads <= 0) threads = omp_get_max_threads();
    auto pd = [](const float* p, float x, float y, float z) { return ((p[0] * x + p[1] * y) + p[2] * z) + p[3] * 1.0f; };
#pragma omp parallel for num_threads(threads) schedule(static)
    for (int64_t i = 0; i < int64_t(n); ++i) {
        const CfAABB& b = boxes[i];
        const float* mn = b.minPoint;
        const float* mx = b.maxPoint;
        bool in = true;
        for (int k = 0; k < 6 && in; ++k) {
            const float* p = f->planes[k];
            int r = 0;
            r += pd(p, mn[0], mn[1], mn[2]) < 0.0f;
            r += pd(p, mx[0], mn[1], mn[2]) < 0.0f;
            r += pd(p, mn[0], mx[1], mn[2]) < 0.0f;
            r += pd(p, mx[0], mx[1], mn[2]) < 0.0f;
            r += pd(p, mn[0], mn[1], mx[2]) < 0.0f;
            r += pd(p, mx[0], mn[1], mx[2]) < 0.0f;
            r += pd(p, mn[0], mx[1], mx[2]) < 0.0f;
            r += pd(p, mx[0], mx[1], mx[2]) < 0.0f;
            if (r == 8) in = false;
        }
        for (int a = 0; a < 3 && in; ++a) {
            int above = 0, below = 0;
            for (int c = 0; c < 8; ++c) {
                above += f->corners[c][a] > mx[a];
                below += f->corners[c][a] < mn[a];
            }
            if (above == 8 || below == 8) in = false;
        }
        instance[i] = in ? 1u : 0u;
    }
    return 0;
}

float cfo_pow(float x, float y) { return cf_pow_pinned(x, y); }
float cfo_log2(float x) { return cf_log2_pinned(x); }
float cfo_exp2(float x) { return cf_exp2_pinned(x); }

/* 1 when a*b+c is evaluated with two roundings (no contraction), else 0. */
int cfo_fp_contract_probe(void)
{
    /* (1 + 2^-12)^2 = 1 + 2^-11 + 2^-24 rounds (tie to even) to 1 + 2^-11, so
     * the unfused sum is 0 and a fused one keeps 2^-24. */
    volatile float va = 1.0f + 0x1p-12f, vc = -(1.0f + 0x1p-11f);
    const float a = va, b = va, c = vc;
    const float r = a * b + c;
    if (r == 0.0f) return 1;
    if (r == 0x1p-24f) return 0;
    return -1;
}

int cfo_max_threads(void) { return omp_get_max_threads(); }

}  // extern "C"
