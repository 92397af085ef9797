// sanitize_main.cpp — host code of the library and the oracle under
// AddressSanitizer and UndefinedBehaviorSanitizer (tests/test_sanitizers.py
// builds and runs it; no GPU is needed or touched).
//
//   argv[1]  a file of views: per view the 176-byte ClusterForwardUBO, the
//            cap and the light count (uint32 each), then the LightData records
//
// It runs, for each view: the oracle's AABB generation and culling (checking
// that offsets are the exclusive scan of the counts, counts are capped and
// every list ascends), its cluster lookup and shading over a synthetic depth
// buffer / G-buffer, and frustum culling of the view's own boxes;
// cf_cull_workspace_size through the C ABI.  Then a randomised sequence of
// the server arena's allocations and releases, checked against a shadow map,
// and the C ABI's argument checks (null handles, bad grids, unknown modes),
// which must fail cleanly without a device.  Any sanitizer report or failed
// check exits non-zero.
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <random>
#include <vector>

#include "cf_arena.h"
#include "cf_types.h"
#include "cfcull.h"
#include "cfcull_testing.h"

extern "C" {
int cfo_generate_aabbs(const CfClusterForwardUBO* ubo, CfAABB* out, int threads);
int cfo_cull(const CfClusterForwardUBO* ubo, const CfAABB* aabbs, const CfLightData* lights, uint32_t light_count,
             uint32_t cap, CfLightCell* cells, uint32_t* indices, uint64_t index_capacity, uint64_t* total,
             uint64_t* executed, int threads);
int cfo_lookup_clusters(const CfClusterForwardUBO* ubo, const float* depth, uint32_t width, uint32_t height,
                        const CfLightCell* cells, const uint32_t* indices, uint64_t index_count,
                        const CfLightData* lights, uint32_t light_count, uint32_t cap, const CfAABB* aabbs,
                        int check_all, CfFragmentSample* out, int threads);
int cfo_shade_clusters(const CfClusterForwardUBO* ubo, const float* cam, const CfPBRPushConstant* pc,
                       const CfGBufferTexel* gbuf, uint32_t width, uint32_t height, const CfLightCell* cells,
                       const uint32_t* indices, uint64_t index_count, const CfLightData* lights, uint32_t light_count,
                       float* out, int threads);
int cfo_frustum_cull(const CfFrustum* f, const CfAABB* boxes, uint32_t n, uint32_t* instance, int threads);
}

static int g_failures = 0;
#define CHECK(c)                                                          \
    do {                                                                  \
        if (!(c)) {                                                       \
            std::fprintf(stderr, "check failed: %s (line %d)\n", #c, __LINE__); \
            ++g_failures;                                                 \
        }                                                                 \
    } while (0)

static void run_view(const CfClusterForwardUBO& u, uint32_t cap, const std::vector<CfLightData>& lights)
{
    const uint32_t C = u.sliceCountX * u.sliceCountY * u.sliceCountZ;
    const uint32_t L = (uint32_t)lights.size();
    std::vector<CfAABB> aabbs(C);
    CHECK(cfo_generate_aabbs(&u, aabbs.data(), 2) == 0);
    std::vector<CfLightCell> cells(C);
    std::vector<uint32_t> idx((size_t)C * cap + 1);
    uint64_t total = 0, executed = 0;
    CHECK(cfo_cull(&u, aabbs.data(), L ? lights.data() : nullptr, L, cap, cells.data(), idx.data(), (uint64_t)C * cap,
                   &total, &executed, 2) == 0);
    uint64_t off = 0;
    for (uint32_t c = 0; c < C; ++c) {
        CHECK(cells[c].offset == off && cells[c].count <= cap);
        for (uint32_t j = 1; j < cells[c].count; ++j) CHECK(idx[off + j - 1] < idx[off + j]);
        for (uint32_t j = 0; j < cells[c].count; ++j) CHECK(idx[off + j] < L);
        off += cells[c].count;
    }
    CHECK(off == total && executed <= (uint64_t)C * L);

    // a small screen of the view's aspect: depth ramps over (0, 1], the last column on the far plane
    const uint32_t W = 32, H = 18;
    CfClusterForwardUBO us = u;
    us.screenSize[0] = (float)W;
    us.screenSize[1] = (float)H;
    std::vector<float> depth((size_t)W * H);
    for (uint32_t i = 0; i < W * H; ++i) depth[i] = (i % W == W - 1) ? 1.0f : (float)(i + 1) / (float)(W * H + 1);
    std::vector<CfFragmentSample> samples((size_t)W * H);
    CHECK(cfo_lookup_clusters(&us, depth.data(), W, H, cells.data(), idx.data(), total, L ? lights.data() : nullptr, L,
                              cap, aabbs.data(), 1, samples.data(), 2) == 0);
    std::vector<CfGBufferTexel> g((size_t)W * H);
    for (uint32_t i = 0; i < W * H; ++i) {
        const CfAABB& b = aabbs[i % C];
        for (int a = 0; a < 3; ++a) g[i].position[a] = 0.5f * (b.minPoint[a] + b.maxPoint[a]);
        g[i].position[3] = depth[i];
        g[i].normal[0] = 0.0f;
        g[i].normal[1] = 0.0f;
        g[i].normal[2] = 1.0f;
        g[i].normal[3] = 0.25f;
        for (int a = 0; a < 3; ++a) g[i].albedo[a] = 0.5f;
        g[i].albedo[3] = 0.5f;
    }
    const float cam[3] = {0.0f, 0.0f, 0.0f};
    const CfPBRPushConstant pc = {1.75f, 0.01f, 0.0f, 0.1f, 0.1f};
    std::vector<float> rgba((size_t)W * H * 4);
    CHECK(cfo_shade_clusters(&us, cam, &pc, g.data(), W, H, cells.data(), idx.data(), total,
                             L ? lights.data() : nullptr, L, rgba.data(), 2) == 0);

    // frustum culling of the view's own boxes against a box-shaped frustum
    CfFrustum f{};
    const float planes[6][4] = {{1, 0, 0, 50}, {-1, 0, 0, 50}, {0, 1, 0, 50}, {0, -1, 0, 50}, {0, 0, 1, 500}, {0, 0, -1, 0}};
    std::memcpy(f.planes, planes, sizeof(planes));
    for (int k = 0; k < 8; ++k) {
        f.corners[k][0] = (k & 1) ? 50.0f : -50.0f;
        f.corners[k][1] = (k & 2) ? 50.0f : -50.0f;
        f.corners[k][2] = (k & 4) ? -500.0f : 0.0f;
        f.corners[k][3] = 1.0f;
    }
    std::vector<uint32_t> inst(C);
    CHECK(cfo_frustum_cull(&f, aabbs.data(), C, inst.data(), 2) == 0);
    for (uint32_t v : inst) CHECK(v <= 1u);

    uint64_t ws = 0;
    const int st = cf_cull_workspace_size(&u, L, cap, &ws);
    CHECK(st == CF_SUCCESS && ws >= 256);
}

static void arena_fuzz()
{
    const size_t size = 64ull << 20;
    unsigned char* base = reinterpret_cast<unsigned char*>(uintptr_t(1) << 40);  // never dereferenced
    cfrt::Arena a;
    a.reset(base, size);
    std::mt19937_64 rng(7);
    std::map<size_t, size_t> live;  // offset -> rounded length
    for (int step = 0; step < 200000; ++step) {
        if (live.empty() || rng() % 3) {
            const size_t want = (size_t)(rng() % (1u << 20)) + 1;
            unsigned char* p = a.alloc(want);
            if (!p) continue;
            const size_t off = (size_t)(p - base), len = (want + 255) & ~(size_t)255;
            CHECK(off % 256 == 0 && off + len <= size);
            auto next = live.lower_bound(off);
            if (next != live.end()) CHECK(off + len <= next->first);
            if (next != live.begin()) {
                auto prev = std::prev(next);
                CHECK(prev->first + prev->second <= off);
            }
            live[off] = len;
        } else {
            auto it = live.begin();
            std::advance(it, (long)(rng() % live.size()));
            a.release(base + it->first);
            live.erase(it);
        }
        size_t used = 0;
        if (step % 997 == 0) {
            for (auto& kv : live) used += kv.second;
            CHECK(used == a.used());
        }
    }
    for (auto& kv : live) a.release(base + kv.first);
    CHECK(a.used() == 0 && a.free_blocks() == 1 && a.largest_free() == size);
}

static void abi_argument_checks()
{
    CHECK(cf_context_create(0, nullptr) == CF_ERROR_INVALID_ARGUMENT);
    CfContext* ctx = nullptr;
    CHECK(cf_context_create(0, &ctx) != CF_SUCCESS && ctx == nullptr);  // no device here
    CHECK(cf_pipeline_light_culling_set_tuning(nullptr, 1, 8, 512, 4, 0) == CF_ERROR_INVALID_ARGUMENT);
    CHECK(cf_pipeline_light_culling_fill_command_buffer(nullptr, nullptr) == CF_ERROR_INVALID_ARGUMENT);
    CHECK(cf_cull_workspace_size(nullptr, 1, 150, nullptr) == CF_ERROR_INVALID_ARGUMENT);
    CfClusterForwardUBO bad{};
    uint64_t ws = 0;
    CHECK(cf_cull_workspace_size(&bad, 10, 150, &ws) == CF_ERROR_INVALID_ARGUMENT);  // zero grid
    bad.sliceCountX = bad.sliceCountY = bad.sliceCountZ = 4096;
    CHECK(cf_cull_workspace_size(&bad, 10, 150, &ws) == CF_ERROR_INVALID_ARGUMENT);  // too many clusters
    CHECK(cf_cull_lights(nullptr, nullptr, nullptr, 0, 150, nullptr, nullptr, 0, nullptr, nullptr, 0, nullptr) ==
          CF_ERROR_INVALID_ARGUMENT);
    CHECK(cf_server_release_many(nullptr, nullptr, 0) == CF_ERROR_INVALID_ARGUMENT);
    CHECK(cf_testing_inject_stall(0x80u) == CF_ERROR_INVALID_ARGUMENT);
    CHECK(cf_testing_fail_allocation_after(-1) == CF_SUCCESS);
    CHECK(std::strlen(cf_last_error_message()) > 0);
    for (int s = 0; s < 10; ++s) CHECK(cf_status_string(s) != nullptr);
}

int main(int argc, char** argv)
{
    if (argc < 2) {
        std::fprintf(stderr, "usage: %s views.bin\n", argv[0]);
        return 2;
    }
    FILE* fp = std::fopen(argv[1], "rb");
    if (!fp) return 2;
    int views = 0;
    for (;;) {
        CfClusterForwardUBO u;
        uint32_t hdr[2];
        if (std::fread(&u, sizeof(u), 1, fp) != 1) break;
        if (std::fread(hdr, sizeof(hdr), 1, fp) != 1) return 2;
        std::vector<CfLightData> lights(hdr[1]);
        if (hdr[1] && std::fread(lights.data(), sizeof(CfLightData), hdr[1], fp) != hdr[1]) return 2;
        run_view(u, hdr[0], lights);
        ++views;
    }
    std::fclose(fp);
    arena_fuzz();
    abi_argument_checks();
    std::printf("views %d, failures %d\n", views, g_failures);
    return g_failures ? 1 : 0;
}
