// cf_runtime.cpp — the C ABI of include/cfcull.h: context, resources, the two
// pipelines and the stateless entry points, over the kernels of cf_kernels.cu.
//
// Object model (mirrors the reference's plugin classes):
//   CfResourcesLight           ResourcesLight           Header/Resources/ResourcesLight.h:42-81
//   CfResourcesClusterForward  ResourcesClusterForward  Header/Resources/ResourcesClusterForward.h:11-31
//   CfPipelineAABBGenerator    PipelineAABBGenerator    Header/Pipelines/PipelineAABBGenerator.h:17-39
//   CfPipelineLightCulling     PipelineLightCulling     Header/Pipelines/PipelineLightCulling.h:18-30
// Pipelines hold non-owning pointers to resources, as in the reference
// (PipelineLightCulling.h:27-28); destroying a resource before a pipeline
// that uses it is the caller's error.
#include <cuda_runtime.h>

#include <atomic>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <new>
#include <string>

#include "cf_batch_internal.h"
#include "cf_kernels.cuh"
#include "cf_runtime_internal.h"
#include "cfcull.h"
#include "cfcull_testing.h"

namespace {

thread_local std::string g_last_error;

}  // namespace

namespace cfrt {

int fail(int status, const char* fmt, ...)
{
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_last_error = buf;
    return status;
}

int cuda_fail(cudaError_t e, const char* what)
{
    if (e == cudaErrorMemoryAllocation) return fail(CF_ERROR_OUT_OF_MEMORY, "%s: %s", what, cudaGetErrorString(e));
    return fail(CF_ERROR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

// True for host memory the current device can address (pinned and mapped);
// *dev receives the device-side address.  Other pointers (pageable, device)
// return false and leave no CUDA error behind.
bool device_addressable(const void* host, void** dev)
{
    cudaPointerAttributes a{};
    if (cudaPointerGetAttributes(&a, host) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    if (a.type != cudaMemoryTypeHost || !a.devicePointer) return false;
    *dev = a.devicePointer;
    return true;
}

bool projection_equal(const CfClusterForwardUBO& a, const CfClusterForwardUBO& b)
{
    return memcmp(a.cameraInverseProjection, b.cameraInverseProjection, sizeof(a.cameraInverseProjection)) == 0 &&
           memcmp(&a.cameraNear, &b.cameraNear, sizeof(float)) == 0 &&
           memcmp(&a.cameraFar, &b.cameraFar, sizeof(float)) == 0 && a.sliceCountX == b.sliceCountX &&
           a.sliceCountY == b.sliceCountY && a.sliceCountZ == b.sliceCountZ;
}

int validate_grid(uint32_t x, uint32_t y, uint32_t z, uint32_t cap, uint32_t* clusters)
{
    if (x == 0 || y == 0 || z == 0) return fail(CF_ERROR_INVALID_ARGUMENT, "cluster grid %ux%ux%u has a zero side", x, y, z);
    const uint64_t c = (uint64_t)x * y * z;
    if (c > kMaxClusters)
        return fail(CF_ERROR_INVALID_ARGUMENT, "cluster grid %ux%ux%u exceeds %u clusters", x, y, z, kMaxClusters);
    if (cap == 0 || cap > kMaxCap)
        return fail(CF_ERROR_INVALID_ARGUMENT, "max_lights_per_cluster %u outside [1, %u]", cap, kMaxCap);
    if (c * cap > 0xffffffffull)
        return fail(CF_ERROR_INVALID_ARGUMENT, "clusters x cap = %llu exceeds 32-bit offsets",
                    (unsigned long long)(c * cap));
    *clusters = (uint32_t)c;
    return CF_SUCCESS;
}

DeviceGuard::DeviceGuard(int device)
{
    cudaGetDevice(&prev_);
    if (prev_ != device) err_ = cudaSetDevice(device);
    else prev_ = -1;
}

DeviceGuard::~DeviceGuard()
{
    if (prev_ >= 0) cudaSetDevice(prev_);
}

namespace {
std::atomic<int32_t> g_fail_allocation_after{-1};  // allocations to let through before one fails; < 0: none
std::atomic<int32_t> g_fail_version_writes{0};     // server version-write launches still to fail
}  // namespace

bool take_injected_version_write_failure()
{
    int32_t n = g_fail_version_writes.load();
    while (n > 0)
        if (g_fail_version_writes.compare_exchange_weak(n, n - 1)) return true;
    return false;
}

cudaError_t device_malloc(void** ptr, size_t bytes)
{
    int32_t n = g_fail_allocation_after.load(std::memory_order_relaxed);
    while (n >= 0 && !g_fail_allocation_after.compare_exchange_weak(n, n - 1, std::memory_order_relaxed)) {
    }
    if (n == 0) {
        *ptr = nullptr;
        return cudaErrorMemoryAllocation;
    }
    return cudaMalloc(ptr, bytes);
}

void set_fail_allocation_after(int32_t n) { g_fail_allocation_after.store(n < 0 ? -1 : n, std::memory_order_relaxed); }

int grow(void** ptr, size_t* capacity, size_t bytes, const char* what)
{
    if (*capacity >= bytes && *ptr) return CF_SUCCESS;
    if (*ptr) {
        cudaError_t e = cudaDeviceSynchronize();
        if (e != cudaSuccess) return cuda_fail(e, what);
        cudaFree(*ptr);
        *ptr = nullptr;
        *capacity = 0;
    }
    if (bytes == 0) return CF_SUCCESS;
    cudaError_t e = device_malloc(ptr, bytes);
    if (e != cudaSuccess) {
        *ptr = nullptr;
        return cuda_fail(e, what);
    }
    e = cudaMemset(*ptr, 0, bytes);
    if (e != cudaSuccess) return cuda_fail(e, what);
    *capacity = bytes;
    return CF_SUCCESS;
}

cfk::CullConfig choose_config(const CfClusterForwardUBO& ubo, uint32_t light_count, const cfk::CullConfig* override_cfg)
{
    if (override_cfg) return *override_cfg;
    const uint32_t C = ubo.sliceCountX * ubo.sliceCountY * ubo.sliceCountZ;
    return cfk::default_cull_config(C, light_count, ubo.sliceCountZ);
}

cfk::WorkspaceLayout layout_for(const CfClusterForwardUBO& ubo, uint32_t light_count, uint32_t cap,
                                const cfk::CullConfig& cfg)
{
    const uint32_t C = ubo.sliceCountX * ubo.sliceCountY * ubo.sliceCountZ;
    const uint32_t groups = cfk::group_count(C, ubo.sliceCountX * ubo.sliceCountY, ubo.sliceCountZ,
                                             cfk::group_width(cfg), cfg.binned);
    return cfk::workspace_layout(C, light_count, cap, ubo.sliceCountZ, cfg.binned, groups);
}

int enqueue_cull(const CfClusterForwardUBO& ubo, const CfAABB* d_aabbs, const CfLightData* d_lights,
                 uint32_t light_count, uint32_t cap, CfLightCell* d_cells, uint32_t* d_indices, uint32_t* d_total,
                 unsigned char* ws, uint32_t* dev_error, const cfk::CullConfig& cfg, cudaStream_t stream,
                 cudaEvent_t* stage_events, unsigned long long* work)
{
    const uint32_t C = ubo.sliceCountX * ubo.sliceCountY * ubo.sliceCountZ;
    const cfk::WorkspaceLayout L = layout_for(ubo, light_count, cap, cfg);
    if (cfg.binned == cfk::kModeOneLaunch) {
        if (light_count > (uint32_t)cfg.tile)
            return fail(CF_ERROR_INVALID_ARGUMENT, "%u lights exceed the %d of this one-launch configuration",
                        light_count, cfg.tile);
        cfk::FusedCull f{};
        f.lights = d_lights;
        f.aabbs = reinterpret_cast<const float4*>(d_aabbs);
        f.cells = d_cells;
        f.indices = d_indices;
        f.total = d_total;
        f.partials = reinterpret_cast<unsigned long long*>(ws + L.partials);
        f.epoch = reinterpret_cast<uint32_t*>(ws + cfk::kEpochWord);
        f.work = work;
        for (int i = 0; i < 16; ++i) f.view[i] = ubo.cameraView[i];
        f.light_count = light_count;
        f.clusters = C;
        f.cap = cap;
        f.per_cta = cfk::group_width(cfg);
        f.ctas = cfk::group_count(C, 0, 0, f.per_cta, cfg.binned);
        cudaError_t e = stage_events ? cudaEventRecord(stage_events[0], stream) : cudaSuccess;
        if (e == cudaSuccess && stage_events) e = cudaEventRecord(stage_events[1], stream);
        if (e == cudaSuccess) e = cfk::launch_one_launch(f, cfg.warps, cfg.tile, dev_error, stream);
        if (e != cudaSuccess) return cuda_fail(e, "one-launch culling");
        if (stage_events) e = cudaEventRecord(stage_events[2], stream);
        if (e == cudaSuccess && stage_events) e = cudaEventRecord(stage_events[3], stream);
        return e == cudaSuccess ? CF_SUCCESS : cuda_fail(e, "stage event");
    }
    cfk::ViewCull v{};
    v.work = work;
    v.vlights = reinterpret_cast<const float4*>(ws + L.vlights);
    v.nonfinite = reinterpret_cast<const uint32_t*>(ws + L.nonfinite);
    v.aabbs = reinterpret_cast<const float4*>(d_aabbs);
    v.counts = reinterpret_cast<uint32_t*>(ws + L.counts);
    v.staging = reinterpret_cast<uint32_t*>(ws + L.staging);
    v.cells = d_cells;
    v.indices = d_indices;
    v.total = d_total;
    v.lpad = cfk::pad_lights(light_count);
    v.clusters = C;
    v.cap = cap;
    v.slice_clusters = ubo.sliceCountX * ubo.sliceCountY;
    v.slices = ubo.sliceCountZ;
    v.binned = cfg.binned ? 1u : 0u;
    v.group_width = cfk::group_width(cfg);
    v.groups = cfk::group_count(C, v.slice_clusters, v.slices, v.group_width, cfg.binned);
    v.group_sums = reinterpret_cast<uint32_t*>(ws + L.group_sums);
    v.group_offsets = reinterpret_cast<uint32_t*>(ws + L.group_offsets);
    if (cfg.binned) {
        v.slice_lights = reinterpret_cast<float4*>(ws + L.slice_lights);
        v.slice_idx = reinterpret_cast<uint32_t*>(ws + L.slice_idx);
        v.slice_count = reinterpret_cast<uint32_t*>(ws + L.slice_count);
        v.slice_nonfinite = reinterpret_cast<uint32_t*>(ws + L.slice_nonfinite);
        v.group_boxes = reinterpret_cast<float4*>(ws + L.group_boxes);
        v.queue = reinterpret_cast<uint32_t*>(ws + cfk::kQueueWord);
    }
    cudaError_t e = stage_events ? cudaEventRecord(stage_events[0], stream) : cudaSuccess;
    if (e == cudaSuccess)
        e = cfk::launch_light_xform(d_lights, light_count, ubo.cameraView,
                                    reinterpret_cast<float4*>(ws + L.vlights),
                                    reinterpret_cast<uint32_t*>(ws + L.nonfinite), stream);
    if (e != cudaSuccess) return cuda_fail(e, "light transform launch");
    if (stage_events) e = cudaEventRecord(stage_events[1], stream);
    if (e == cudaSuccess && cfg.binned) e = cfk::launch_bin(v, stream);
    if (e != cudaSuccess) return cuda_fail(e, "slice binning launch");
    e = cfk::launch_cull(v, cfg, dev_error, stream);
    if (e != cudaSuccess) return cuda_fail(e, "light culling launch");
    if (stage_events) e = cudaEventRecord(stage_events[2], stream);
    if (e == cudaSuccess) e = cfk::launch_finalize(v, stream);
    if (e != cudaSuccess) return cuda_fail(e, "offset scan launch");
    if (stage_events) e = cudaEventRecord(stage_events[3], stream);
    return e == cudaSuccess ? CF_SUCCESS : cuda_fail(e, "stage event");
}

}  // namespace cfrt

using namespace cfrt;

// ---------------------------------------------------------------------------
// Handles.
// ---------------------------------------------------------------------------
struct CfContext {
    int device = 0;
    uint32_t* dev_error = nullptr;  // OR of cfk::kErr* codes from bounded in-kernel waits
};

struct CfResourcesLight {
    CfContext* ctx = nullptr;
    CfLightData* d_lights = nullptr;
    size_t capacity_bytes = 0;
    uint32_t count = 0;
};

struct CfResourcesClusterForward {
    CfContext* ctx = nullptr;
    uint32_t x = 0, y = 0, z = 0, cap = 0, clusters = 0;
    CfAABB* d_aabbs = nullptr;
    CfLightCell* d_cells = nullptr;
    uint32_t* d_indices = nullptr;
    uint32_t* d_total = nullptr;
    unsigned char* d_ws = nullptr;
    size_t ws_capacity = 0;
    uint32_t* h_total = nullptr;  // pinned word the one-launch read-back writes the total into
    bool aabb_dirty = true;
    bool aabb_built = false;
    CfClusterForwardUBO built_from{};
};

struct CfPipelineAABBGenerator {
    CfContext* ctx = nullptr;
    CfResourcesClusterForward* res = nullptr;
    CfClusterForwardUBO ubo{};
    bool has_ubo = false;
};

struct CfPipelineLightCulling {
    CfContext* ctx = nullptr;
    CfResourcesLight* lights = nullptr;
    CfResourcesClusterForward* res = nullptr;
    CfClusterForwardUBO ubo{};
    bool has_ubo = false;
    cfk::CullConfig cfg{};
    bool has_cfg = false;
    cudaEvent_t stage_events[4] = {nullptr, nullptr, nullptr, nullptr};  // stage timing, when enabled
    unsigned long long* d_work = nullptr;                                   // work counters, when enabled
};

namespace cfrt {
int context_device(const CfContext* ctx) { return ctx->device; }
uint32_t* context_error_word(const CfContext* ctx) { return ctx->dev_error; }
}  // namespace cfrt

namespace {

void free_cluster_buffers(CfResourcesClusterForward* r)
{
    cudaFree(r->d_aabbs);
    cudaFree(r->d_cells);
    cudaFree(r->d_indices);
    cudaFree(r->d_total);
    cudaFree(r->d_ws);
    r->d_aabbs = nullptr;
    r->d_cells = nullptr;
    r->d_indices = nullptr;
    r->d_total = nullptr;
    r->d_ws = nullptr;
    r->ws_capacity = 0;
}

}  // namespace

extern "C" {

const char* cf_status_string(int s)
{
    switch (s) {
        case CF_SUCCESS: return "success";
        case CF_ERROR_INVALID_ARGUMENT: return "invalid argument";
        case CF_ERROR_OUT_OF_MEMORY: return "out of memory";
        case CF_ERROR_CUDA: return "CUDA error";
        case CF_ERROR_CAPACITY: return "buffer too small";
        case CF_ERROR_NOT_READY: return "not ready";
        case CF_ERROR_DEVICE_TIMEOUT: return "device wait timed out";
        case CF_ERROR_BUDGET: return "device-memory budget exceeded";
        case CF_ERROR_UNSUPPORTED: return "unsupported device";
        default: return "unknown status";
    }
}

const char* cf_last_error_message(void) { return g_last_error.c_str(); }

int cf_version(void) { return 10000; }

// --- context ---------------------------------------------------------------
int cf_context_create(int device, CfContext** out)
{
    if (!out) return fail(CF_ERROR_INVALID_ARGUMENT, "cf_context_create: null out");
    *out = nullptr;
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess || device < 0 || device >= n)
        return fail(CF_ERROR_UNSUPPORTED, "no CUDA device %d (%d visible)", device, n);
    cudaDeviceProp prop;
    e = cudaGetDeviceProperties(&prop, device);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetDeviceProperties");
    if (prop.major * 10 + prop.minor != 103)
        return fail(CF_ERROR_UNSUPPORTED, "device %d is sm_%d%d; this library is built for sm_103a", device,
                    prop.major, prop.minor);
    DeviceGuard g(device);
    if (g.err()) return cuda_fail(g.err(), "cudaSetDevice");
    CfContext* c = new (std::nothrow) CfContext();
    if (!c) return fail(CF_ERROR_OUT_OF_MEMORY, "host allocation");
    c->device = device;
    e = device_malloc(reinterpret_cast<void**>(&c->dev_error), sizeof(uint32_t));
    if (e != cudaSuccess) {
        delete c;
        return cuda_fail(e, "device error word");
    }
    cudaMemset(c->dev_error, 0, sizeof(uint32_t));
    *out = c;
    return CF_SUCCESS;
}

int cf_context_destroy(CfContext* ctx)
{
    if (!ctx) return CF_SUCCESS;
    DeviceGuard g(ctx->device);
    cudaFree(ctx->dev_error);
    delete ctx;
    return CF_SUCCESS;
}

int cf_context_check_device_error(CfContext* ctx, uint32_t* device_error)
{
    if (!ctx || !device_error) return fail(CF_ERROR_INVALID_ARGUMENT, "cf_context_check_device_error: null argument");
    DeviceGuard g(ctx->device);
    cudaError_t e = cudaDeviceSynchronize();
    if (e != cudaSuccess) return cuda_fail(e, "cudaDeviceSynchronize");
    uint32_t v = 0;
    e = cudaMemcpy(&v, ctx->dev_error, sizeof(v), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_fail(e, "read device error word");
    cudaMemset(ctx->dev_error, 0, sizeof(uint32_t));
    *device_error = v;
    return v ? fail(CF_ERROR_DEVICE_TIMEOUT, "device error word 0x%x", v) : CF_SUCCESS;
}

// --- ResourcesLight --------------------------------------------------------
int cf_resources_light_create(CfContext* ctx, CfResourcesLight** out)
{
    if (!ctx || !out) return fail(CF_ERROR_INVALID_ARGUMENT, "cf_resources_light_create: null argument");
    CfResourcesLight* r = new (std::nothrow) CfResourcesLight();
    if (!r) return fail(CF_ERROR_OUT_OF_MEMORY, "host allocation");
    r->ctx = ctx;
    *out = r;
    return CF_SUCCESS;
}

int cf_resources_light_destroy(CfResourcesLight* r)
{
    if (!r) return CF_SUCCESS;
    DeviceGuard g(r->ctx->device);
    cudaFree(r->d_lights);
    delete r;
    return CF_SUCCESS;
}

int cf_resources_light_upload_async(CfResourcesLight* r, const CfLightData* lights, uint32_t count, void* stream)
{
    if (!r || (count && !lights)) return fail(CF_ERROR_INVALID_ARGUMENT, "cf_resources_light_upload: null argument");
    if (count > kMaxLights) return fail(CF_ERROR_INVALID_ARGUMENT, "%u lights exceed %u", count, kMaxLights);
    DeviceGuard g(r->ctx->device);
    if (g.err()) return cuda_fail(g.err(), "cudaSetDevice");
    const size_t bytes = (size_t)count * sizeof(CfLightData);
    int s = grow(reinterpret_cast<void**>(&r->d_lights), &r->capacity_bytes, bytes, "light buffer");
    if (s) return s;
    if (bytes) {
        cudaError_t e = cudaMemcpyAsync(r->d_lights, lights, bytes, cudaMemcpyHostToDevice, (cudaStream_t)stream);
        if (e != cudaSuccess) return cuda_fail(e, "light upload");
    }
    r->count = count;
    return CF_SUCCESS;
}

int cf_resources_light_add_lights(CfResourcesLight* r, const CfLightData* lights, uint32_t count)
{
    int s = cf_resources_light_upload_async(r, lights, count, nullptr);
    if (s) return s;
    DeviceGuard g(r->ctx->device);
    cudaError_t e = cudaStreamSynchronize(nullptr);
    return e == cudaSuccess ? CF_SUCCESS : cuda_fail(e, "light upload");
}

int cf_resources_light_update_light_position(CfResourcesLight* r, uint32_t index, const float position[3])
{
    if (!r || !position) return fail(CF_ERROR_INVALID_ARGUMENT, "cf_resources_light_update_light_position: null argument");
    if (index >= r->count) return CF_SUCCESS;  // ignored, as ResourcesLight.cpp:22-25
    DeviceGuard g(r->ctx->device);
    const float p[4] = {position[0], position[1], position[2], 1.0f};
    cudaError_t e = cudaMemcpy(reinterpret_cast<float*>(r->d_lights + index), p, sizeof(p), cudaMemcpyHostToDevice);
    return e == cudaSuccess ? CF_SUCCESS : cuda_fail(e, "light position update");
}

int cf_resources_light_get_light_count(const CfResourcesLight* r, uint32_t* count)
{
    if (!r || !count) return fail(CF_ERROR_INVALID_ARGUMENT, "null argument");
    *count = r->count;
    return CF_SUCCESS;
}

int cf_resources_light_get_device_buffer(const CfResourcesLight* r, const CfLightData** device_lights)
{
    if (!r || !device_lights) return fail(CF_ERROR_INVALID_ARGUMENT, "null argument");
    *device_lights = r->d_lights;
    return CF_SUCCESS;
}

// --- ResourcesClusterForward -----------------------------------------------
int cf_resources_cluster_forward_create(CfContext* ctx, CfResourcesClusterForward** out)
{
    if (!ctx || !out) return fail(CF_ERROR_INVALID_ARGUMENT, "cf_resources_cluster_forward_create: null argument");
    CfResourcesClusterForward* r = new (std::nothrow) CfResourcesClusterForward();
    if (!r) return fail(CF_ERROR_OUT_OF_MEMORY, "host allocation");
    r->ctx = ctx;
    *out = r;
    return CF_SUCCESS;
}

int cf_resources_cluster_forward_destroy(CfResourcesClusterForward* r)
{
    if (!r) return CF_SUCCESS;
    DeviceGuard g(r->ctx->device);
    free_cluster_buffers(r);
    if (r->h_total) cudaFreeHost(r->h_total);
    delete r;
    return CF_SUCCESS;
}

int cf_resources_cluster_forward_create_buffers(CfResourcesClusterForward* r, uint32_t x, uint32_t y, uint32_t z,
                                                uint32_t cap)
{
    if (!r) return fail(CF_ERROR_INVALID_ARGUMENT, "null resources");
    uint32_t C = 0;
    int s = validate_grid(x, y, z, cap, &C);
    if (s) return s;
    DeviceGuard g(r->ctx->device);
    if (g.err()) return cuda_fail(g.err(), "cudaSetDevice");
    cudaError_t e = cudaDeviceSynchronize();
    if (e != cudaSuccess) return cuda_fail(e, "cudaDeviceSynchronize");
    free_cluster_buffers(r);
    e = device_malloc(reinterpret_cast<void**>(&r->d_aabbs), (size_t)C * sizeof(CfAABB));
    if (e == cudaSuccess) e = device_malloc(reinterpret_cast<void**>(&r->d_cells), (size_t)C * sizeof(CfLightCell));
    if (e == cudaSuccess) e = device_malloc(reinterpret_cast<void**>(&r->d_indices), (size_t)C * cap * sizeof(uint32_t));
    if (e == cudaSuccess) e = device_malloc(reinterpret_cast<void**>(&r->d_total), sizeof(uint32_t));
    if (e == cudaSuccess) e = cudaMemset(r->d_cells, 0, (size_t)C * sizeof(CfLightCell));
    if (e == cudaSuccess) e = cudaMemset(r->d_total, 0, sizeof(uint32_t));
    if (e != cudaSuccess) {
        free_cluster_buffers(r);
        return cuda_fail(e, "cluster buffers");
    }
    r->x = x;
    r->y = y;
    r->z = z;
    r->cap = cap;
    r->clusters = C;
    r->aabb_dirty = true;
    r->aabb_built = false;
    return CF_SUCCESS;
}

int cf_resources_cluster_forward_get_buffers(const CfResourcesClusterForward* r, CfClusterForwardBuffers* out)
{
    if (!r || !out) return fail(CF_ERROR_INVALID_ARGUMENT, "null argument");
    out->aabbs = r->d_aabbs;
    out->light_cells = r->d_cells;
    out->light_indices = r->d_indices;
    out->total_indices = r->d_total;
    out->cluster_count = r->clusters;
    out->max_lights_per_cluster = r->cap;
    out->index_capacity = (uint64_t)r->clusters * r->cap;
    return CF_SUCCESS;
}

int cf_resources_cluster_forward_is_aabb_dirty(const CfResourcesClusterForward* r, int* dirty)
{
    if (!r || !dirty) return fail(CF_ERROR_INVALID_ARGUMENT, "null argument");
    *dirty = r->aabb_dirty ? 1 : 0;
    return CF_SUCCESS;
}

int cf_resources_cluster_forward_read_outputs(CfResourcesClusterForward* r, CfLightCell* host_cells,
                                              uint32_t* host_indices, uint64_t host_index_capacity, uint32_t* total,
                                              void* stream)
{
    if (!r || !total) return fail(CF_ERROR_INVALID_ARGUMENT, "null argument");
    if (!r->d_cells) return fail(CF_ERROR_NOT_READY, "buffers were never created");
    DeviceGuard g(r->ctx->device);
    cudaStream_t st = (cudaStream_t)stream;
    // Host buffers the device can address (pinned, mapped): one read-back
    // launch writes the total, the cells and the indices, then one wait.
    void* dev_cells = nullptr;
    void* dev_indices = nullptr;
    if ((!host_cells || device_addressable(host_cells, &dev_cells)) &&
        (!host_indices || device_addressable(host_indices, &dev_indices)) &&
        (r->h_total || cudaHostAlloc(reinterpret_cast<void**>(&r->h_total), sizeof(uint32_t), cudaHostAllocMapped) ==
                           cudaSuccess)) {
        void* dev_total = nullptr;
        cudaError_t e = cudaHostGetDevicePointer(&dev_total, r->h_total, 0);
        if (e == cudaSuccess)
            e = cfk::launch_readback(r->d_cells, r->clusters, r->d_indices, r->d_total, host_indices ? host_index_capacity : 0,
                                     static_cast<CfLightCell*>(dev_cells), static_cast<uint32_t*>(dev_indices),
                                     static_cast<uint32_t*>(dev_total), st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) return cuda_fail(e, "read outputs");
        *total = *reinterpret_cast<volatile uint32_t*>(r->h_total);
        return CF_SUCCESS;
    }
    cudaGetLastError();  // a failed pinned-word allocation leaves no sticky error
    uint32_t t = 0;
    cudaError_t e = cudaMemcpyAsync(&t, r->d_total, sizeof(t), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess && host_cells)
        e = cudaMemcpyAsync(host_cells, r->d_cells, (size_t)r->clusters * sizeof(CfLightCell), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cuda_fail(e, "read outputs");
    const uint64_t n = t < host_index_capacity ? t : host_index_capacity;
    if (n && host_indices) {
        e = cudaMemcpyAsync(host_indices, r->d_indices, n * sizeof(uint32_t), cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) return cuda_fail(e, "read indices");
    }
    *total = t;
    return CF_SUCCESS;
}

// --- PipelineAABBGenerator -------------------------------------------------
int cf_pipeline_aabb_generator_create(CfContext* ctx, CfResourcesClusterForward* res, CfPipelineAABBGenerator** out)
{
    if (!ctx || !res || !out) return fail(CF_ERROR_INVALID_ARGUMENT, "cf_pipeline_aabb_generator_create: null argument");
    CfPipelineAABBGenerator* p = new (std::nothrow) CfPipelineAABBGenerator();
    if (!p) return fail(CF_ERROR_OUT_OF_MEMORY, "host allocation");
    p->ctx = ctx;
    p->res = res;
    *out = p;
    return CF_SUCCESS;
}

int cf_pipeline_aabb_generator_destroy(CfPipelineAABBGenerator* p)
{
    delete p;
    return CF_SUCCESS;
}

int cf_pipeline_aabb_generator_set_cluster_forward_ubo(CfPipelineAABBGenerator* p, const CfClusterForwardUBO* ubo)
{
    if (!p || !ubo) return fail(CF_ERROR_INVALID_ARGUMENT, "null argument");
    p->ubo = *ubo;
    p->has_ubo = true;
    if (!p->res->aabb_built || !projection_equal(p->res->built_from, *ubo)) p->res->aabb_dirty = true;
    return CF_SUCCESS;
}

int cf_pipeline_aabb_generator_on_window_resized(CfPipelineAABBGenerator* p)
{
    if (!p) return fail(CF_ERROR_INVALID_ARGUMENT, "null pipeline");
    p->res->aabb_dirty = true;
    return CF_SUCCESS;
}

int cf_pipeline_aabb_generator_fill_command_buffer(CfPipelineAABBGenerator* p, void* stream)
{
    TraceRange trace("AABB_Generator");
    if (!p) return fail(CF_ERROR_INVALID_ARGUMENT, "null pipeline");
    if (!p->has_ubo) return fail(CF_ERROR_NOT_READY, "SetClusterForwardUBO was never called");
    CfResourcesClusterForward* r = p->res;
    if (!r->d_aabbs) return fail(CF_ERROR_NOT_READY, "CreateBuffers was never called");
    if (p->ubo.sliceCountX != r->x || p->ubo.sliceCountY != r->y || p->ubo.sliceCountZ != r->z)
        return fail(CF_ERROR_INVALID_ARGUMENT, "UBO grid %ux%ux%u differs from the buffers' %ux%ux%u", p->ubo.sliceCountX,
                    p->ubo.sliceCountY, p->ubo.sliceCountZ, r->x, r->y, r->z);
    if (!r->aabb_dirty) return CF_SUCCESS;
    DeviceGuard g(p->ctx->device);
    cudaError_t e = cfk::launch_aabb(p->ubo, r->d_aabbs, (cudaStream_t)stream);
    if (e != cudaSuccess) return cuda_fail(e, "AABB generator launch");
    r->aabb_dirty = false;
    r->aabb_built = true;
    r->built_from = p->ubo;
    return CF_SUCCESS;
}

// --- PipelineLightCulling --------------------------------------------------
int cf_pipeline_light_culling_create(CfContext* ctx, CfResourcesLight* lights, CfResourcesClusterForward* res,
                                     CfPipelineLightCulling** out)
{
    if (!ctx || !lights || !res || !out)
        return fail(CF_ERROR_INVALID_ARGUMENT, "cf_pipeline_light_culling_create: null argument");
    CfPipelineLightCulling* p = new (std::nothrow) CfPipelineLightCulling();
    if (!p) return fail(CF_ERROR_OUT_OF_MEMORY, "host allocation");
    p->ctx = ctx;
    p->lights = lights;
    p->res = res;
    *out = p;
    return CF_SUCCESS;
}

int cf_pipeline_light_culling_destroy(CfPipelineLightCulling* p)
{
    if (!p) return CF_SUCCESS;
    DeviceGuard g(p->ctx->device);
    for (cudaEvent_t& e : p->stage_events)
        if (e) cudaEventDestroy(e);
    cudaFree(p->d_work);
    delete p;
    return CF_SUCCESS;
}

int cf_pipeline_light_culling_enable_work_counters(CfPipelineLightCulling* p, int enable)
{
    if (!p) return fail(CF_ERROR_INVALID_ARGUMENT, "null pipeline");
    DeviceGuard g(p->ctx->device);
    if (!enable) {
        if (p->d_work) cudaDeviceSynchronize();  // a queued cull may still count into it
        cudaFree(p->d_work);
        p->d_work = nullptr;
        return CF_SUCCESS;
    }
    if (p->d_work) return CF_SUCCESS;
    cudaError_t e = device_malloc(reinterpret_cast<void**>(&p->d_work), 2 * sizeof(unsigned long long));
    if (e == cudaSuccess) e = cudaMemset(p->d_work, 0, 2 * sizeof(unsigned long long));
    return e == cudaSuccess ? CF_SUCCESS : cuda_fail(e, "work counters");
}

int cf_pipeline_light_culling_read_work_counters(CfPipelineLightCulling* p, uint64_t counters[2])
{
    if (!p || !counters) return fail(CF_ERROR_INVALID_ARGUMENT, "null argument");
    if (!p->d_work) return fail(CF_ERROR_NOT_READY, "work counters are not enabled");
    DeviceGuard g(p->ctx->device);
    unsigned long long h[2] = {0, 0};
    cudaError_t e = cudaDeviceSynchronize();
    if (e == cudaSuccess) e = cudaMemcpy(h, p->d_work, sizeof(h), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemset(p->d_work, 0, sizeof(h));
    if (e != cudaSuccess) return cuda_fail(e, "read work counters");
    counters[0] = h[0];
    counters[1] = h[1];
    return CF_SUCCESS;
}

int cf_pipeline_light_culling_enable_stage_timing(CfPipelineLightCulling* p, int enable)
{
    if (!p) return fail(CF_ERROR_INVALID_ARGUMENT, "null pipeline");
    DeviceGuard g(p->ctx->device);
    if (!enable) {
        for (cudaEvent_t& e : p->stage_events) {
            if (e) cudaEventDestroy(e);
            e = nullptr;
        }
        return CF_SUCCESS;
    }
    for (cudaEvent_t& e : p->stage_events) {
        if (e) continue;
        cudaError_t err = cudaEventCreate(&e);
        if (err != cudaSuccess) return cuda_fail(err, "cudaEventCreate");
    }
    return CF_SUCCESS;
}

int cf_pipeline_light_culling_get_stage_times(CfPipelineLightCulling* p, float* ms)
{
    if (!p || !ms) return fail(CF_ERROR_INVALID_ARGUMENT, "null argument");
    if (!p->stage_events[0]) return fail(CF_ERROR_NOT_READY, "stage timing is not enabled");
    DeviceGuard g(p->ctx->device);
    cudaError_t e = cudaEventSynchronize(p->stage_events[3]);
    for (int i = 0; i < 3 && e == cudaSuccess; ++i) e = cudaEventElapsedTime(&ms[i], p->stage_events[i], p->stage_events[i + 1]);
    return e == cudaSuccess ? CF_SUCCESS : cuda_fail(e, "stage times");
}

int cf_pipeline_light_culling_reset_global_index(CfPipelineLightCulling* p)
{
    return p ? CF_SUCCESS : fail(CF_ERROR_INVALID_ARGUMENT, "null pipeline");
}

int cf_pipeline_light_culling_set_cluster_forward_ubo(CfPipelineLightCulling* p, const CfClusterForwardUBO* ubo)
{
    if (!p || !ubo) return fail(CF_ERROR_INVALID_ARGUMENT, "null argument");
    p->ubo = *ubo;
    p->has_ubo = true;
    return CF_SUCCESS;
}

int cf_pipeline_light_culling_fill_command_buffer(CfPipelineLightCulling* p, void* stream)
{
    TraceRange trace("Light_Culling");
    if (!p) return fail(CF_ERROR_INVALID_ARGUMENT, "null pipeline");
    if (!p->has_ubo) return fail(CF_ERROR_NOT_READY, "SetClusterForwardUBO was never called");
    CfResourcesClusterForward* r = p->res;
    if (!r->d_aabbs) return fail(CF_ERROR_NOT_READY, "CreateBuffers was never called");
    if (!r->aabb_built) return fail(CF_ERROR_NOT_READY, "the AABB generator has not run on these buffers");
    if (p->ubo.sliceCountX != r->x || p->ubo.sliceCountY != r->y || p->ubo.sliceCountZ != r->z)
        return fail(CF_ERROR_INVALID_ARGUMENT, "UBO grid %ux%ux%u differs from the buffers' %ux%ux%u", p->ubo.sliceCountX,
                    p->ubo.sliceCountY, p->ubo.sliceCountZ, r->x, r->y, r->z);
    if (p->lights->count && !p->lights->d_lights) return fail(CF_ERROR_NOT_READY, "no lights uploaded");
    DeviceGuard g(p->ctx->device);
    if (g.err()) return cuda_fail(g.err(), "cudaSetDevice");
    const cfk::CullConfig cfg = choose_config(p->ubo, p->lights->count, p->has_cfg ? &p->cfg : nullptr);
    const cfk::WorkspaceLayout L = layout_for(p->ubo, p->lights->count, r->cap, cfg);
    int s = grow(reinterpret_cast<void**>(&r->d_ws), &r->ws_capacity, L.bytes, "culling workspace");
    if (s) return s;
    return enqueue_cull(p->ubo, r->d_aabbs, p->lights->d_lights, p->lights->count, r->cap, r->d_cells, r->d_indices,
                        r->d_total, r->d_ws, p->ctx->dev_error, cfg, (cudaStream_t)stream,
                        p->stage_events[0] ? p->stage_events : nullptr, p->d_work);
}

int cf_pipeline_light_culling_set_tuning(CfPipelineLightCulling* p, int clusters_per_warp, int warps, int tile,
                                         int stages, int binned)
{
    if (!p) return fail(CF_ERROR_INVALID_ARGUMENT, "null pipeline");
    if (clusters_per_warp == 0) {
        p->has_cfg = false;
        return CF_SUCCESS;
    }
    if (binned < cfk::kModeBruteForce || binned > cfk::kModeOneLaunch)
        return fail(CF_ERROR_INVALID_ARGUMENT, "culling mode %d (0 brute force, 1 binned, 2 one launch)", binned);
    const cfk::CullConfig c{clusters_per_warp, warps, tile, stages, binned};
    if (!cfk::cull_config_supported(c))
        return fail(CF_ERROR_INVALID_ARGUMENT, "no culling kernel for K=%d warps=%d tile=%d stages=%d binned=%d",
                    clusters_per_warp, warps, tile, stages, binned);
    p->cfg = c;
    p->has_cfg = true;
    return CF_SUCCESS;
}

int cf_pipeline_light_culling_get_tuning(const CfPipelineLightCulling* p, int config[5])
{
    if (!p || !config) return fail(CF_ERROR_INVALID_ARGUMENT, "null argument");
    if (!p->has_ubo || !p->lights) return fail(CF_ERROR_NOT_READY, "no cluster-forward UBO set yet");
    const cfk::CullConfig c = choose_config(p->ubo, p->lights->count, p->has_cfg ? &p->cfg : nullptr);
    config[0] = c.clusters_per_warp;
    config[1] = c.warps;
    config[2] = c.tile;
    config[3] = c.stages;
    config[4] = c.binned;
    return CF_SUCCESS;
}

// --- stateless -------------------------------------------------------------
int cf_cull_workspace_device_error(void* d_workspace, uint32_t* device_error)
{
    if (!d_workspace || !device_error) return fail(CF_ERROR_INVALID_ARGUMENT, "null argument");
    cudaError_t e = cudaDeviceSynchronize();
    uint32_t v = 0;
    if (e == cudaSuccess) e = cudaMemcpy(&v, d_workspace, sizeof(v), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemset(d_workspace, 0, sizeof(v));
    if (e != cudaSuccess) return cuda_fail(e, "read workspace error word");
    *device_error = v;
    return v ? fail(CF_ERROR_DEVICE_TIMEOUT, "device error word 0x%x", v) : CF_SUCCESS;
}

int cf_cull_workspace_size(const CfClusterForwardUBO* ubo, uint32_t light_count, uint32_t cap, uint64_t* bytes)
{
    if (!ubo || !bytes) return fail(CF_ERROR_INVALID_ARGUMENT, "cf_cull_workspace_size: null argument");
    uint32_t C = 0;
    int s = validate_grid(ubo->sliceCountX, ubo->sliceCountY, ubo->sliceCountZ, cap, &C);
    if (s) return s;
    *bytes = layout_for(*ubo, light_count, cap, choose_config(*ubo, light_count, nullptr)).bytes;
    return CF_SUCCESS;
}

int cf_generate_aabbs(const CfClusterForwardUBO* ubo, CfAABB* d_aabbs, void* stream)
{
    if (!ubo || !d_aabbs) return fail(CF_ERROR_INVALID_ARGUMENT, "cf_generate_aabbs: null argument");
    uint32_t C = 0;
    int s = validate_grid(ubo->sliceCountX, ubo->sliceCountY, ubo->sliceCountZ, 1, &C);
    if (s) return s;
    cudaError_t e = cfk::launch_aabb(*ubo, d_aabbs, (cudaStream_t)stream);
    return e == cudaSuccess ? CF_SUCCESS : cuda_fail(e, "AABB generator launch");
}

int cf_animate_light_orbits(CfLightData* d_lights, CfLightOrbit* d_orbits, uint64_t count, uint32_t frames,
                            void* stream)
{
    if (count && (!d_lights || !d_orbits)) return fail(CF_ERROR_INVALID_ARGUMENT, "cf_animate_light_orbits: null argument");
    if ((reinterpret_cast<uintptr_t>(d_lights) | reinterpret_cast<uintptr_t>(d_orbits)) & 15)
        return fail(CF_ERROR_INVALID_ARGUMENT, "cf_animate_light_orbits: buffers must be 16-byte aligned");
    const cudaError_t e = cfk::launch_orbits(d_lights, d_orbits, count, frames, (cudaStream_t)stream);
    return e == cudaSuccess ? CF_SUCCESS : cuda_fail(e, "light orbit launch");
}

int cf_cull_lights(const CfClusterForwardUBO* ubo, const CfAABB* d_aabbs, const CfLightData* d_lights,
                   uint32_t light_count, uint32_t cap, CfLightCell* d_cells, uint32_t* d_indices,
                   uint64_t index_capacity, uint32_t* d_total, void* d_workspace, uint64_t workspace_bytes,
                   void* stream)
{
    TraceRange trace("Light_Culling");
    if (!ubo || !d_aabbs || !d_cells || !d_indices || !d_workspace || (light_count && !d_lights))
        return fail(CF_ERROR_INVALID_ARGUMENT, "cf_cull_lights: null argument");
    if (light_count > kMaxLights) return fail(CF_ERROR_INVALID_ARGUMENT, "%u lights exceed %u", light_count, kMaxLights);
    if (reinterpret_cast<uintptr_t>(d_workspace) % 256)
        return fail(CF_ERROR_INVALID_ARGUMENT, "workspace must be 256-byte aligned");
    uint32_t C = 0;
    int s = validate_grid(ubo->sliceCountX, ubo->sliceCountY, ubo->sliceCountZ, cap, &C);
    if (s) return s;
    if (index_capacity < (uint64_t)C * cap)
        return fail(CF_ERROR_CAPACITY, "index capacity %llu < clusters x cap = %llu", (unsigned long long)index_capacity,
                    (unsigned long long)C * cap);
    const cfk::CullConfig cfg = choose_config(*ubo, light_count, nullptr);
    const cfk::WorkspaceLayout L = layout_for(*ubo, light_count, cap, cfg);
    if (workspace_bytes < L.bytes)
        return fail(CF_ERROR_CAPACITY, "workspace %llu bytes < %llu needed", (unsigned long long)workspace_bytes,
                    (unsigned long long)L.bytes);
    unsigned char* ws = static_cast<unsigned char*>(d_workspace);
    return enqueue_cull(*ubo, d_aabbs, d_lights, light_count, cap, d_cells, d_indices, d_total, ws,
                        reinterpret_cast<uint32_t*>(ws), cfg, (cudaStream_t)stream, nullptr);
}


// --- test hooks (include/cfcull_testing.h) ---------------------------------
namespace {
std::mutex g_knob_mutex;
uint64_t g_knob_wait_ns = 0;  // 0: the kernels' default
uint32_t g_knob_inject = 0;

int apply_test_knobs()
{
    const uint64_t limit = g_knob_wait_ns ? g_knob_wait_ns : 2000000000ull;
    cudaError_t e = cfk::set_test_knobs_kernels(limit, g_knob_inject);
    if (e == cudaSuccess) e = cfk::set_test_knobs_one_launch(limit, g_knob_inject);
    return e == cudaSuccess ? CF_SUCCESS : cuda_fail(e, "set test knobs");
}
}  // namespace

int cf_testing_set_wait_limit_ns(uint64_t limit_ns)
{
    std::lock_guard<std::mutex> lock(g_knob_mutex);
    g_knob_wait_ns = limit_ns;
    return apply_test_knobs();
}

int cf_testing_inject_stall(uint32_t mode)
{
    if (mode & ~(CF_TESTING_STALL_ONE_LAUNCH | CF_TESTING_STALL_BRUTE_FORCE))
        return fail(CF_ERROR_INVALID_ARGUMENT, "unknown stall injection bits 0x%x", mode);
    std::lock_guard<std::mutex> lock(g_knob_mutex);
    g_knob_inject = mode;
    return apply_test_knobs();
}

int cf_testing_fail_allocation_after(int32_t n)
{
    set_fail_allocation_after(n);
    return CF_SUCCESS;
}

int cf_testing_fail_version_writes(int32_t n)
{
    g_fail_version_writes.store(n > 0 ? n : 0);
    return CF_SUCCESS;
}

}  // extern "C"
