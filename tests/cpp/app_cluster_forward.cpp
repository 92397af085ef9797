// A C++ host driving the culling path through include/cfcull.h the way
// AppPBRClusterForward drives PipelineAABBGenerator and PipelineLightCulling
// (Source/Apps/AppPBRClusterForward.cpp:45-136): create the resources and the
// two pipelines once, then per frame set the UBO, reset the global index and
// fill both pipelines; move a light with UpdateLightPosition; resize the
// window.  Every frame's LightCells and index list are checked against the
// oracle library (oracle/cf_oracle.cpp), bit for bit.  Exit status 0 and
// "ok" on success.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <vector>

#include "cfcull.h"

extern "C" {  // oracle/cf_oracle.cpp (test infrastructure)
int cfo_generate_aabbs(const CfClusterForwardUBO* ubo, CfAABB* out, int threads);
int cfo_cull(const CfClusterForwardUBO* ubo, const CfAABB* aabbs, const CfLightData* lights, uint32_t light_count,
             uint32_t cap, CfLightCell* cells, uint32_t* indices, uint64_t index_capacity, uint64_t* total_out,
             uint64_t* executed_tests_out, int threads);
}

namespace {

constexpr uint32_t kX = 16, kY = 9, kZ = 24, kCap = 150;

#define CHECK(call)                                                                                  \
    do {                                                                                             \
        const int s_ = (call);                                                                       \
        if (s_ != CF_SUCCESS) {                                                                      \
            std::fprintf(stderr, "%s: %s (%s)\n", #call, cf_status_string(s_), cf_last_error_message()); \
            return 1;                                                                                \
        }                                                                                            \
    } while (0)

// Camera::GetClusterForwardUBO for a camera at the origin looking down -z:
// a right-handed perspective with depth in [0, 1] and the Vulkan y flip, its
// closed-form inverse, and the log2 slice scale and bias.
CfClusterForwardUBO make_ubo(float fovy, float width, float height, float n, float f)
{
    CfClusterForwardUBO u{};
    const float t = std::tan(fovy / 2.0f);
    const float p00 = 1.0f / ((width / height) * t), p11 = -1.0f / t;
    const float p22 = f / (n - f), p32 = -(f * n) / (f - n);
    float* inv = u.cameraInverseProjection;  // column-major
    inv[0] = 1.0f / p00;
    inv[5] = 1.0f / p11;
    inv[11] = 1.0f / p32;
    inv[14] = -1.0f;
    inv[15] = p22 / p32;
    for (int i = 0; i < 4; ++i) u.cameraView[5 * i] = 1.0f;
    u.screenSize[0] = width;
    u.screenSize[1] = height;
    u.sliceScaling = float(kZ) / std::log2(f / n);
    u.sliceBias = -float(kZ) * std::log2(n) / std::log2(f / n);
    u.cameraNear = n;
    u.cameraFar = f;
    u.sliceCountX = kX;
    u.sliceCountY = kY;
    u.sliceCountZ = kZ;
    return u;
}

struct Rng {  // splitmix64
    uint64_t s;
    float uniform(float lo, float hi)
    {
        uint64_t z = (s += 0x9E3779B97F4A7C15ull);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        z ^= z >> 31;
        return lo + (hi - lo) * float(z >> 40) * 0x1p-24f;
    }
};

int check_frame(CfResourcesClusterForward* res, const CfClusterForwardUBO& ubo, const std::vector<CfLightData>& lights,
                int frame)
{
    const uint32_t C = kX * kY * kZ;
    std::vector<CfLightCell> cells(C), ref_cells(C);
    std::vector<uint32_t> indices(size_t(C) * kCap), ref_indices(size_t(C) * kCap);
    uint32_t total = 0;
    CHECK(cf_resources_cluster_forward_read_outputs(res, cells.data(), indices.data(), indices.size(), &total,
                                                    nullptr));
    std::vector<CfAABB> aabbs(C);
    uint64_t ref_total = 0;
    if (cfo_generate_aabbs(&ubo, aabbs.data(), 0) != 0 ||
        cfo_cull(&ubo, aabbs.data(), lights.data(), uint32_t(lights.size()), kCap, ref_cells.data(),
                 ref_indices.data(), ref_indices.size(), &ref_total, nullptr, 0) != 0) {
        std::fprintf(stderr, "frame %d: oracle failed\n", frame);
        return 1;
    }
    if (total != ref_total || std::memcmp(cells.data(), ref_cells.data(), C * sizeof(CfLightCell)) != 0 ||
        std::memcmp(indices.data(), ref_indices.data(), total * sizeof(uint32_t)) != 0) {
        std::fprintf(stderr, "frame %d: outputs differ from the oracle (%u vs %llu indices)\n", frame, total,
                     (unsigned long long)ref_total);
        return 1;
    }
    std::printf("frame %d: %u indices, bit-exact\n", frame, total);
    return 0;
}

}  // namespace

int main()
{
    // Init (once)
    std::vector<CfLightData> lights(1024);
    Rng rng{7};
    for (CfLightData& L : lights) {
        L = CfLightData{};
        L.position[0] = rng.uniform(-20.0f, 20.0f);
        L.position[1] = rng.uniform(0.0f, 15.0f);
        L.position[2] = rng.uniform(-40.0f, 10.0f);
        L.position[3] = 1.0f;
        for (int c = 0; c < 3; ++c) L.color[c] = rng.uniform(0.0f, 1.0f);
        L.color[3] = 1.0f;
        L.radius = rng.uniform(1.0f, 5.0f);
    }
    CfContext* cf = nullptr;
    CHECK(cf_context_create(0, &cf));
    CfResourcesLight* res_light = nullptr;
    CHECK(cf_resources_light_create(cf, &res_light));
    CHECK(cf_resources_light_add_lights(res_light, lights.data(), uint32_t(lights.size())));
    CfResourcesClusterForward* res_cf = nullptr;
    CHECK(cf_resources_cluster_forward_create(cf, &res_cf));
    CHECK(cf_resources_cluster_forward_create_buffers(res_cf, kX, kY, kZ, kCap));
    CfPipelineAABBGenerator* aabb = nullptr;
    CHECK(cf_pipeline_aabb_generator_create(cf, res_cf, &aabb));
    CfPipelineLightCulling* cull = nullptr;
    CHECK(cf_pipeline_light_culling_create(cf, res_light, res_cf, &cull));

    float width = 1920.0f, height = 1080.0f;
    const float fovy = 45.0f * 3.14159265358979f / 180.0f;
    for (int frame = 0; frame < 4; ++frame) {
        if (frame == 2) {  // OnWindowResized: a new aspect ratio, so new cluster AABBs
            width = 1280.0f;
            height = 1024.0f;
            CHECK(cf_pipeline_aabb_generator_on_window_resized(aabb));
        }
        // UpdateUBOs + FillCommandBuffer (every frame)
        const CfClusterForwardUBO ubo = make_ubo(fovy, width, height, 0.1f, 1000.0f);
        CHECK(cf_pipeline_aabb_generator_set_cluster_forward_ubo(aabb, &ubo));
        CHECK(cf_pipeline_light_culling_reset_global_index(cull));
        CHECK(cf_pipeline_light_culling_set_cluster_forward_ubo(cull, &ubo));
        CHECK(cf_pipeline_aabb_generator_fill_command_buffer(aabb, nullptr));
        CHECK(cf_pipeline_light_culling_fill_command_buffer(cull, nullptr));
        if (check_frame(res_cf, ubo, lights, frame)) return 1;
        // ResourcesLight::UpdateLightPosition on one light between frames
        const uint32_t moved = uint32_t(37 * frame + 5);
        const float pos[3] = {rng.uniform(-5.0f, 5.0f), rng.uniform(0.0f, 5.0f), rng.uniform(-20.0f, -2.0f)};
        CHECK(cf_resources_light_update_light_position(res_light, moved, pos));
        std::memcpy(lights[moved].position, pos, sizeof(pos));
    }
    uint32_t device_error = 0;
    CHECK(cf_context_check_device_error(cf, &device_error));
    if (device_error) {
        std::fprintf(stderr, "device error word %u\n", device_error);
        return 1;
    }
    cf_pipeline_light_culling_destroy(cull);
    cf_pipeline_aabb_generator_destroy(aabb);
    cf_resources_cluster_forward_destroy(res_cf);
    cf_resources_light_destroy(res_light);
    cf_context_destroy(cf);
    std::printf("ok\n");
    return 0;
}
