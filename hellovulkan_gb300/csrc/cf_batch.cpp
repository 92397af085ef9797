// cf_batch.cpp — many views culled together (the batched form of the path).
//
// A batch holds N views, each with its own UBO, light set, AABBs and output
// buffers (caller-owned device memory).  One culling pass of the batch is
//   batch_xform   every view's lights to view space            (1 launch)
//   batch_bin     every view's depth-slice candidate lists      (1 launch)
//   cull_batch    a persistent kernel taking (view, cluster group) items
//                 from a device queue (1 launch per run of shape buckets
//                 with the same configuration, largest grids first)
//   batch_scan    every view's group offsets                    (1 launch)
//   batch_copy    every view's LightCells and index list        (1 launch)
// and can be captured once into a CUDA graph and replayed while the views'
// shapes and buffers stay the same (light positions and view matrices may
// change in place between replays).
//
// A shape bucket is the set of views with the same clusters per depth slice
// (X * Y): they share a cluster-group layout, and the autotuner picks the
// culling configuration (clusters per warp, warps per CTA, lights per
// shared-memory stage) of each bucket by timing the candidates on the batch.
//
// There is no counterpart of a batch in the reference, which culls one view
// per frame (PipelineLightCulling::FillCommandBuffer).
#include <cuda_runtime.h>

#include <algorithm>
#include <map>
#include <new>
#include <numeric>
#include <vector>

#include "cf_batch_internal.h"
#include "cf_kernels.cuh"
#include "cf_runtime_internal.h"
#include "cfcull.h"

using namespace cfrt;

namespace {

const cfk::CullConfig kBatchCandidates[] = {
    {1, 4, 256, 4, 1}, {2, 4, 256, 4, 1}, {4, 4, 256, 4, 1}, {1, 8, 256, 4, 1}, {2, 8, 256, 4, 1}, {4, 8, 256, 4, 1},
    {2, 4, 512, 2, 1}, {4, 4, 512, 2, 1}, {2, 8, 512, 2, 1}, {4, 8, 512, 2, 1}, {2, 8, 1024, 2, 1}, {4, 8, 1024, 2, 1},
};
const cfk::CullConfig kBatchDefault = {2, 8, 1024, 2, 1};

size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

}  // namespace

struct CfBatch {
    CfContext* ctx = nullptr;
    int device = 0;
    uint32_t* dev_error = nullptr;
    std::vector<CfBatchView> views;
    std::map<uint32_t, cfk::CullConfig> tuned;  // bucket key (X*Y) -> configuration
    // derived, rebuilt by rebuild()
    struct Bucket {
        uint32_t key;
        cfk::CullConfig cfg;
        uint32_t item_begin, item_count;
        int ctas;
    };
    std::vector<Bucket> buckets;
    // culling launches: consecutive buckets with the same configuration share
    // one persistent launch over their (contiguous) items, so the batch pays
    // one launch tail per configuration instead of one per grid
    struct Launch {
        cfk::CullConfig cfg;
        uint32_t item_begin, item_count;
        int ctas;
    };
    std::vector<Launch> launches;
    std::vector<cfk::ViewJob> jobs;
    uint32_t xform_blocks = 0, bin_blocks = 0, copy_blocks_total = 0, n_items = 0;
    size_t ws_bytes = 0;
    // device
    cfk::ViewJob* d_jobs = nullptr;
    size_t jobs_cap = 0;
    uint32_t* d_prefix = nullptr;  // 4 x n: xform, bin (in bin order), copy, bin order
    size_t prefix_cap = 0;
    uint2* d_items = nullptr;
    size_t items_cap = 0;
    uint32_t* d_queues = nullptr;
    unsigned char* d_ws = nullptr;
    size_t ws_cap = 0;
    cfk::AabbJob* d_aabb_jobs = nullptr;  // one AABB-generator record per view
    size_t aabb_jobs_cap = 0;
    uint32_t* d_aabb_prefix = nullptr;    // first block of each view in the AABB launch
    size_t aabb_prefix_cap = 0;
    uint32_t aabb_blocks = 0;
    // graph
    bool use_graph = true;
    cudaGraphExec_t exec = nullptr;
    cudaStream_t graph_stream = nullptr;
    // Recorded after the last pass or AABB generation enqueued outside a
    // stream capture: the device tables, the workspace and the graph are not
    // changed until it has completed.
    cudaEvent_t last_use = nullptr;
    bool used = false;
};

namespace {

// Waits until no work this batch enqueued can still read its tables.
int wait_idle(CfBatch* b)
{
    if (!b->used) return CF_SUCCESS;
    const cudaError_t e = cudaEventSynchronize(b->last_use);
    if (e != cudaSuccess) return cuda_fail(e, "waiting for the batch's last pass");
    b->used = false;
    return CF_SUCCESS;
}

// Notes work enqueued on st that reads the batch's tables.
int mark_used(CfBatch* b, cudaStream_t st)
{
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    cudaError_t e = cudaStreamIsCapturing(st, &cs);
    if (e == cudaSuccess && cs == cudaStreamCaptureStatusNone) {
        e = cudaEventRecord(b->last_use, st);
        if (e == cudaSuccess) b->used = true;
    }
    return e == cudaSuccess ? CF_SUCCESS : cuda_fail(e, "batch completion event");
}

void drop_graph(CfBatch* b)
{
    if (b->exec) cudaGraphExecDestroy(b->exec);
    b->exec = nullptr;
    b->graph_stream = nullptr;
}

cfk::CullConfig config_for(const CfBatch* b, uint32_t key)
{
    auto it = b->tuned.find(key);
    return it == b->tuned.end() ? kBatchDefault : it->second;
}

bool same_config(const cfk::CullConfig& a, const cfk::CullConfig& c)
{
    return a.clusters_per_warp == c.clusters_per_warp && a.warps == c.warps && a.tile == c.tile &&
           a.stages == c.stages && a.binned == c.binned;
}

int validate_view(const CfBatchView& v, uint32_t i, uint32_t* clusters)
{
    int s = validate_grid(v.ubo.sliceCountX, v.ubo.sliceCountY, v.ubo.sliceCountZ, v.max_lights_per_cluster, clusters);
    if (s) return fail(s, "batch view %u: %s", i, cf_last_error_message());
    if (!v.d_aabbs || !v.d_cells || !v.d_indices || (v.light_count && !v.d_lights))
        return fail(CF_ERROR_INVALID_ARGUMENT, "batch view %u: null device pointer", i);
    if (v.light_count > kMaxLights) return fail(CF_ERROR_INVALID_ARGUMENT, "batch view %u: too many lights", i);
    if (v.index_capacity < (uint64_t)*clusters * v.max_lights_per_cluster)
        return fail(CF_ERROR_CAPACITY, "batch view %u: index capacity %llu < clusters x cap", i,
                    (unsigned long long)v.index_capacity);
    return CF_SUCCESS;
}

// Recomputes every derived table from b->views and b->tuned and uploads it.
int rebuild(CfBatch* b)
{
    const int w = wait_idle(b);  // passes still queued read the tables rewritten below
    if (w) return w;
    drop_graph(b);
    const uint32_t n = (uint32_t)b->views.size();
    b->jobs.assign(n, cfk::ViewJob{});
    std::vector<size_t> ws_off(n);
    std::vector<cfk::WorkspaceLayout> lay(n);
    std::vector<uint32_t> prefix(4 * (size_t)n), aabb_prefix(n);
    std::vector<cfk::AabbJob> aabb_jobs(n);
    uint32_t ab = 0;
    size_t ws = 0;
    uint32_t xb = 0, bb = 0, cb = 0;
    for (uint32_t i = 0; i < n; ++i) {
        const CfBatchView& bv = b->views[i];
        uint32_t C = 0;
        int s = validate_view(bv, i, &C);
        if (s) return s;
        const uint32_t xy = bv.ubo.sliceCountX * bv.ubo.sliceCountY, Z = bv.ubo.sliceCountZ;
        const cfk::CullConfig cfg = config_for(b, xy);
        const uint32_t gw = (uint32_t)(cfg.warps * cfg.clusters_per_warp);
        const uint32_t groups = cfk::group_count(C, xy, Z, gw, true);
        lay[i] = cfk::workspace_layout(C, bv.light_count, bv.max_lights_per_cluster, Z, true, groups);
        ws_off[i] = ws;
        ws += align256(lay[i].bytes);
        cfk::ViewJob& j = b->jobs[i];
        j.v.aabbs = reinterpret_cast<const float4*>(bv.d_aabbs);
        j.v.cells = bv.d_cells;
        j.v.indices = bv.d_indices;
        j.v.total = bv.d_total;
        j.v.lpad = cfk::pad_lights(bv.light_count);
        j.v.clusters = C;
        j.v.cap = bv.max_lights_per_cluster;
        j.v.slice_clusters = xy;
        j.v.slices = Z;
        j.v.group_width = gw;
        j.v.groups = groups;
        j.v.binned = 1;
        j.lights = bv.d_lights;
        j.light_count = bv.light_count;
        for (int q = 0; q < 16; ++q) j.view[q] = bv.ubo.cameraView[q];
        prefix[i] = xb;
        prefix[2 * (size_t)n + i] = cb;
        aabb_jobs[i] = cfk::AabbJob{bv.ubo, bv.d_aabbs, 0};
        aabb_prefix[i] = ab;
        ab += (C + 255) / 256;
        xb += cfk::granules(j.v.lpad);
        cb += cfk::copy_blocks(groups);
    }
    // binning blocks: the views with the most lights first (a block reads all
    // of its view's lights, so those blocks run longest)
    uint32_t* const order = prefix.data() + 3 * (size_t)n;
    for (uint32_t i = 0; i < n; ++i) order[i] = i;
    std::stable_sort(order, order + n, [&](uint32_t a, uint32_t c) { return b->jobs[a].light_count > b->jobs[c].light_count; });
    for (uint32_t r = 0; r < n; ++r) {
        prefix[n + r] = bb;
        bb += cfk::bin_blocks(b->jobs[order[r]].v.slices);
    }
    b->xform_blocks = xb;
    b->bin_blocks = bb;
    b->copy_blocks_total = cb;
    b->aabb_blocks = ab;
    b->ws_bytes = ws;
    DeviceGuard g(b->device);
    int s = grow(reinterpret_cast<void**>(&b->d_ws), &b->ws_cap, std::max<size_t>(ws, 256), "batch workspace");
    if (s) return s;
    for (uint32_t i = 0; i < n; ++i) {
        cfk::ViewJob& j = b->jobs[i];
        unsigned char* w = b->d_ws + ws_off[i];
        const cfk::WorkspaceLayout& L = lay[i];
        j.v.vlights = reinterpret_cast<const float4*>(w + L.vlights);
        j.v.nonfinite = reinterpret_cast<const uint32_t*>(w + L.nonfinite);
        j.v.counts = reinterpret_cast<uint32_t*>(w + L.counts);
        j.v.staging = reinterpret_cast<uint32_t*>(w + L.staging);
        j.v.group_sums = reinterpret_cast<uint32_t*>(w + L.group_sums);
        j.v.group_offsets = reinterpret_cast<uint32_t*>(w + L.group_offsets);
        j.v.slice_lights = reinterpret_cast<float4*>(w + L.slice_lights);
        j.v.slice_idx = reinterpret_cast<uint32_t*>(w + L.slice_idx);
        j.v.slice_count = reinterpret_cast<uint32_t*>(w + L.slice_count);
        j.v.slice_nonfinite = reinterpret_cast<uint32_t*>(w + L.slice_nonfinite);
        j.v.group_boxes = reinterpret_cast<float4*>(w + L.group_boxes);
    }
    // buckets and items: views by decreasing light count, groups in order
    std::map<uint32_t, std::vector<uint32_t>> by_key;
    for (uint32_t i = 0; i < n; ++i) by_key[b->jobs[i].v.slice_clusters].push_back(i);
    if (by_key.size() > cfk::kMaxBatchQueues)
        return fail(CF_ERROR_INVALID_ARGUMENT, "%zu distinct grids exceed %u per batch", by_key.size(),
                    cfk::kMaxBatchQueues);
    // largest grids first: their items are the longest, so within a launch
    // shared with smaller grids they start in the first wave
    std::vector<uint2> items;
    b->buckets.clear();
    b->launches.clear();
    for (auto it = by_key.rbegin(); it != by_key.rend(); ++it) {
        std::vector<uint32_t>& vs = it->second;
        std::stable_sort(vs.begin(), vs.end(),
                         [&](uint32_t x, uint32_t y) { return b->jobs[x].light_count > b->jobs[y].light_count; });
        CfBatch::Bucket bk{it->first, config_for(b, it->first), (uint32_t)items.size(), 0, 0};
        for (uint32_t vi : vs)
            for (uint32_t gi = 0; gi < b->jobs[vi].v.groups; ++gi) items.push_back(make_uint2(vi, gi));
        bk.item_count = (uint32_t)items.size() - bk.item_begin;
        int resident = 0;
        cudaError_t e = cfk::batch_cull_resident_ctas(bk.cfg, &resident);
        if (e != cudaSuccess) return cuda_fail(e, "occupancy query");
        bk.ctas = std::min<int>(resident, (int)std::max<uint32_t>(bk.item_count, 1));
        b->buckets.push_back(bk);
        if (!b->launches.empty() && same_config(b->launches.back().cfg, bk.cfg)) {
            CfBatch::Launch& l = b->launches.back();
            l.item_count += bk.item_count;
            l.ctas = std::min<int>(resident, (int)std::max<uint32_t>(l.item_count, 1));
        } else {
            b->launches.push_back(CfBatch::Launch{bk.cfg, bk.item_begin, bk.item_count, bk.ctas});
        }
    }
    b->n_items = (uint32_t)items.size();
    s = grow(reinterpret_cast<void**>(&b->d_jobs), &b->jobs_cap, std::max<size_t>(n, 1) * sizeof(cfk::ViewJob), "batch jobs");
    if (!s) s = grow(reinterpret_cast<void**>(&b->d_prefix), &b->prefix_cap, std::max<size_t>(4 * (size_t)n, 1) * 4, "batch prefix");
    if (!s) s = grow(reinterpret_cast<void**>(&b->d_items), &b->items_cap, std::max<size_t>(items.size(), 1) * sizeof(uint2), "batch items");
    if (!s) s = grow(reinterpret_cast<void**>(&b->d_aabb_jobs), &b->aabb_jobs_cap, std::max<size_t>(n, 1) * sizeof(cfk::AabbJob), "batch AABB jobs");
    if (!s) s = grow(reinterpret_cast<void**>(&b->d_aabb_prefix), &b->aabb_prefix_cap, std::max<size_t>(n, 1) * 4, "batch AABB prefix");
    if (s) return s;
    cudaError_t e = cudaSuccess;
    if (n) e = cudaMemcpy(b->d_jobs, b->jobs.data(), n * sizeof(cfk::ViewJob), cudaMemcpyHostToDevice);
    if (e == cudaSuccess && n) e = cudaMemcpy(b->d_prefix, prefix.data(), prefix.size() * 4, cudaMemcpyHostToDevice);
    if (e == cudaSuccess && !items.empty())
        e = cudaMemcpy(b->d_items, items.data(), items.size() * sizeof(uint2), cudaMemcpyHostToDevice);
    if (e == cudaSuccess && n) e = cudaMemcpy(b->d_aabb_jobs, aabb_jobs.data(), n * sizeof(cfk::AabbJob), cudaMemcpyHostToDevice);
    if (e == cudaSuccess && n) e = cudaMemcpy(b->d_aabb_prefix, aabb_prefix.data(), n * 4, cudaMemcpyHostToDevice);
    return e == cudaSuccess ? CF_SUCCESS : cuda_fail(e, "batch tables upload");
}

int enqueue_batch(CfBatch* b, cudaStream_t st)
{
    const uint32_t n = (uint32_t)b->views.size();
    if (n == 0) return CF_SUCCESS;
    const uint32_t* px = b->d_prefix;
    const uint32_t* pb = b->d_prefix + n;
    cudaError_t e = cfk::launch_batch_xform(b->d_jobs, px, n, b->xform_blocks, b->d_queues,
                                            (uint32_t)b->launches.size(), st);
    if (e == cudaSuccess) e = cfk::launch_batch_bin(b->d_jobs, pb, b->d_prefix + 3 * (size_t)n, n, b->bin_blocks, st);
    for (size_t q = 0; q < b->launches.size() && e == cudaSuccess; ++q) {
        const CfBatch::Launch& l = b->launches[q];
        cfk::BatchCull bc{b->d_jobs, b->d_items + l.item_begin, l.item_count, b->d_queues + q};
        e = cfk::launch_batch_cull(bc, l.cfg, l.ctas, b->dev_error, st);
    }
    if (e == cudaSuccess) e = cfk::launch_batch_scan(b->d_jobs, n, st);
    if (e == cudaSuccess) e = cfk::launch_batch_copy(b->d_jobs, b->d_prefix + 2 * (size_t)n, n, b->copy_blocks_total, st);
    return e == cudaSuccess ? CF_SUCCESS : cuda_fail(e, "batch launch");
}

}  // namespace

namespace cfrt {

int batch_cull(CfBatch* b, cudaStream_t st)
{
    DeviceGuard g(b->device);
    if (!b->use_graph || st == nullptr) {
        const int s = enqueue_batch(b, st);
        return s ? s : mark_used(b, st);
    }
    if (!b->exec || b->graph_stream != st) {
        if (b->exec) {  // the graph may still run on its former stream
            const int w = wait_idle(b);
            if (w) return w;
        }
        drop_graph(b);
        cudaGraph_t graph = nullptr;
        cudaError_t e = cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal);
        if (e != cudaSuccess) return cuda_fail(e, "cudaStreamBeginCapture");
        const int s = enqueue_batch(b, st);
        e = cudaStreamEndCapture(st, &graph);
        if (s) {
            if (graph) cudaGraphDestroy(graph);
            return s;
        }
        if (e != cudaSuccess) return cuda_fail(e, "cudaStreamEndCapture");
        e = cudaGraphInstantiate(&b->exec, graph, 0);
        cudaGraphDestroy(graph);
        if (e != cudaSuccess) {
            b->exec = nullptr;
            return cuda_fail(e, "cudaGraphInstantiate");
        }
        b->graph_stream = st;
    }
    const cudaError_t e = cudaGraphLaunch(b->exec, st);
    return e == cudaSuccess ? mark_used(b, st) : cuda_fail(e, "cudaGraphLaunch");
}

}  // namespace cfrt

extern "C" {

int cf_batch_create(CfContext* ctx, CfBatch** out)
{
    if (!ctx || !out) return fail(CF_ERROR_INVALID_ARGUMENT, "cf_batch_create: null argument");
    CfBatch* b = new (std::nothrow) CfBatch();
    if (!b) return fail(CF_ERROR_OUT_OF_MEMORY, "host allocation");
    b->ctx = ctx;
    b->device = context_device(ctx);
    b->dev_error = context_error_word(ctx);
    DeviceGuard g(b->device);
    cudaError_t e = device_malloc(reinterpret_cast<void**>(&b->d_queues), cfk::kMaxBatchQueues * sizeof(uint32_t));
    if (e == cudaSuccess) e = cudaMemset(b->d_queues, 0, cfk::kMaxBatchQueues * sizeof(uint32_t));
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->last_use, cudaEventDisableTiming);
    if (e != cudaSuccess) {
        cudaFree(b->d_queues);
        delete b;
        return cuda_fail(e, "batch queues");
    }
    *out = b;
    return CF_SUCCESS;
}

int cf_batch_destroy(CfBatch* b)
{
    if (!b) return CF_SUCCESS;
    DeviceGuard g(b->device);
    wait_idle(b);
    drop_graph(b);
    if (b->last_use) cudaEventDestroy(b->last_use);
    cudaFree(b->d_jobs);
    cudaFree(b->d_prefix);
    cudaFree(b->d_items);
    cudaFree(b->d_queues);
    cudaFree(b->d_ws);
    cudaFree(b->d_aabb_jobs);
    cudaFree(b->d_aabb_prefix);
    delete b;
    return CF_SUCCESS;
}

int cf_batch_set_views(CfBatch* b, const CfBatchView* views, uint32_t n)
{
    if (!b || (n && !views)) return fail(CF_ERROR_INVALID_ARGUMENT, "cf_batch_set_views: null argument");
    b->views.assign(views, views + n);
    return rebuild(b);
}

int cf_batch_update_view_matrices(CfBatch* b, const CfClusterForwardUBO* ubos, uint32_t n, void* stream)
{
    if (!b || (n && !ubos)) return fail(CF_ERROR_INVALID_ARGUMENT, "null argument");
    if (n != b->views.size()) return fail(CF_ERROR_INVALID_ARGUMENT, "%u UBOs for %zu views", n, b->views.size());
    DeviceGuard g(b->device);
    const int w = wait_idle(b);  // a pass queued on another stream may still read the table
    if (w) return w;
    for (uint32_t i = 0; i < n; ++i) {
        for (int q = 0; q < 16; ++q) b->jobs[i].view[q] = ubos[i].cameraView[q];
        b->views[i].ubo = ubos[i];
    }
    // synchronous for a pageable source; the graph reads the table at replay
    cudaError_t e = cudaMemcpyAsync(b->d_jobs, b->jobs.data(), n * sizeof(cfk::ViewJob), cudaMemcpyHostToDevice,
                                    (cudaStream_t)stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize((cudaStream_t)stream);
    return e == cudaSuccess ? CF_SUCCESS : cuda_fail(e, "view matrix upload");
}

int cf_batch_generate_aabbs(CfBatch* b, void* stream)
{
    if (!b) return fail(CF_ERROR_INVALID_ARGUMENT, "null batch");
    DeviceGuard g(b->device);
    const cudaError_t e = cfk::launch_batch_aabb(b->d_aabb_jobs, b->d_aabb_prefix, (uint32_t)b->views.size(),
                                                 b->aabb_blocks, (cudaStream_t)stream);
    return e == cudaSuccess ? mark_used(b, (cudaStream_t)stream) : cuda_fail(e, "AABB generator launch");
}

int cf_batch_cull(CfBatch* b, void* stream)
{
    TraceRange trace("Batch_Light_Culling");
    if (!b) return fail(CF_ERROR_INVALID_ARGUMENT, "null batch");
    return batch_cull(b, (cudaStream_t)stream);
}

int cf_batch_set_graph(CfBatch* b, int enable)
{
    if (!b) return fail(CF_ERROR_INVALID_ARGUMENT, "null batch");
    const int w = wait_idle(b);
    if (w) return w;
    b->use_graph = enable != 0;
    drop_graph(b);
    return CF_SUCCESS;
}

int cf_batch_set_tuning(CfBatch* b, uint32_t slice_clusters, int clusters_per_warp, int warps, int tile, int stages)
{
    if (!b) return fail(CF_ERROR_INVALID_ARGUMENT, "null batch");
    if (clusters_per_warp == 0) {
        b->tuned.erase(slice_clusters);
    } else {
        const cfk::CullConfig c{clusters_per_warp, warps, tile, stages, 1};
        if (!cfk::cull_config_supported(c))
            return fail(CF_ERROR_INVALID_ARGUMENT, "no batched culling kernel for K=%d warps=%d tile=%d stages=%d",
                        clusters_per_warp, warps, tile, stages);
        b->tuned[slice_clusters] = c;
    }
    return rebuild(b);
}

int cf_batch_autotune(CfBatch* b, int repeats, void* stream)
{
    if (!b) return fail(CF_ERROR_INVALID_ARGUMENT, "null batch");
    if (repeats <= 0) repeats = 3;
    DeviceGuard g(b->device);
    cudaStream_t st = (cudaStream_t)stream;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    const bool graph = b->use_graph;
    b->use_graph = false;
    std::vector<uint32_t> keys;
    for (const CfBatchView& v : b->views) keys.push_back(v.ubo.sliceCountX * v.ubo.sliceCountY);
    std::sort(keys.begin(), keys.end());
    keys.erase(std::unique(keys.begin(), keys.end()), keys.end());
    int status = CF_SUCCESS;
    for (uint32_t key : keys) {
        float best = 1e30f;
        cfk::CullConfig best_cfg = config_for(b, key);
        for (const cfk::CullConfig& c : kBatchCandidates) {
            b->tuned[key] = c;
            if ((status = rebuild(b))) break;
            if ((status = enqueue_batch(b, st))) break;  // warm
            float total = 0.f;
            for (int r = 0; r < repeats && !status; ++r) {
                cudaEventRecord(e0, st);
                status = enqueue_batch(b, st);
                cudaEventRecord(e1, st);
                cudaEventSynchronize(e1);
                float ms = 0.f;
                cudaEventElapsedTime(&ms, e0, e1);
                total += ms;
            }
            if (status) break;
            if (total < best) {
                best = total;
                best_cfg = c;
            }
        }
        if (status) break;
        b->tuned[key] = best_cfg;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    b->use_graph = graph;
    const int s2 = rebuild(b);
    return status ? status : s2;
}

int cf_batch_get_info(const CfBatch* b, CfBatchInfo* info)
{
    if (!b || !info) return fail(CF_ERROR_INVALID_ARGUMENT, "null argument");
    info->views = (uint32_t)b->views.size();
    info->items = b->n_items;
    info->buckets = (uint32_t)b->buckets.size();
    info->workspace_bytes = b->ws_bytes;
    for (uint32_t q = 0; q < 8; ++q) {
        if (q < b->buckets.size()) {
            const CfBatch::Bucket& bk = b->buckets[q];
            info->bucket_slice_clusters[q] = bk.key;
            info->bucket_config[q][0] = bk.cfg.clusters_per_warp;
            info->bucket_config[q][1] = bk.cfg.warps;
            info->bucket_config[q][2] = bk.cfg.tile;
            info->bucket_config[q][3] = bk.cfg.stages;
            info->bucket_ctas[q] = bk.ctas;
        } else {
            info->bucket_slice_clusters[q] = 0;
            for (int a = 0; a < 4; ++a) info->bucket_config[q][a] = 0;
            info->bucket_ctas[q] = 0;
        }
    }
    return CF_SUCCESS;
}

}  // extern "C"
