// cf_kernels.cuh — launch interface of the clustered-forward CUDA kernels.
//
// Data layout in device memory for one view (all 256-byte aligned):
//   aabbs     C x CfAABB (32 B)            written by the AABB generator, reused
//                                          while the projection is unchanged
//   vlights   lpad x float4 (16 B)         view-space light (x, y, z, r^2); lpad is
//                                          the light count rounded up to 32 and
//                                          the pad entries are (0, 0, 0, -inf),
//                                          which fail every test
//   nonfinite ceil(lpad / 256) x uint32    1 where a 256-light granule holds a
//                                          light whose view-space position is not
//                                          finite (those granules take the exact
//                                          branchy test)
//   counts    C x uint32                   capped hit count per cluster (plain path)
//   staging   C x cap x uint32             each cluster's hits in ascending order
//   cells     C x CfLightCell              output
//   indices   >= sum(counts) x uint32      output, packed in cluster order
// and, on the binned path, per depth slice a candidate list (slice_*).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "cf_types.h"

namespace cfk {

constexpr uint32_t kLightPad = 32;       // view-space light arrays are padded to this
constexpr uint32_t kFlagGranule = 256;   // lights per non-finite flag word


// Device error codes (OR-ed into the context's error word).
constexpr uint32_t kErrFullWaitTimeout = 1u << 0;   // a consumer waited too long for a light tile
constexpr uint32_t kErrEmptyWaitTimeout = 1u << 1;  // the producer waited too long for a free stage
constexpr uint32_t kErrLookbackTimeout = 1u << 2;   // a one-launch CTA waited too long for an earlier CTA's total

// Culling modes (CullConfig::binned).
constexpr int kModeBruteForce = 0;  // transform, every light against every cluster, copy
constexpr int kModeBinned = 1;      // transform, slice binning, persistent culling of the candidates, copy
constexpr int kModeOneLaunch = 2;   // everything in one launch (cf_fused.cu), views of up to kOneLaunchMaxLights

inline uint32_t pad_lights(uint32_t n) { return (n + kLightPad - 1) / kLightPad * kLightPad; }
inline uint32_t granules(uint32_t lpad) { return (lpad + kFlagGranule - 1) / kFlagGranule; }
// Start of a slice list's second segment (see ViewCull): half the padded
// lights, rounded up to a multiple of 32.
__host__ __device__ inline uint32_t list_split(uint32_t lpad) { return (lpad / 32 + 1) / 2 * 32; }

struct ViewCull {
    const float4* vlights;
    const uint32_t* nonfinite;
    const float4* aabbs;
    uint32_t* counts;
    uint32_t* staging;
    CfLightCell* cells;
    uint32_t* indices;
    uint32_t* total;  // may be null
    // binned path: per depth slice, a candidate list of lpad entries
    float4* slice_lights;
    uint32_t* slice_idx;
    // A slice's list is two segments, each in ascending light order and
    // padded to a multiple of 32: the candidates among lights [0, S) at the
    // list's start, those among [S, lpad) from entry S (S = list_split(lpad));
    // the list is the first followed by the second.  A single view bins the
    // two with separate CTAs; a batch writes everything to the first.
    uint32_t* slice_count;      // [2k + h]: padded length of segment h of slice k
    uint32_t* slice_nonfinite;  // [2k + h]: 1 when segment h lists a light with a non-finite coordinate
    float4* group_boxes;        // per cluster group, the union of its AABBs (lo, hi; NaN bound: infinite)
    // optional work counters (profiling only, null otherwise): [0] sphere-box
    // tests against slice slabs and warp union boxes, [1] sphere-box tests
    // against cluster boxes
    unsigned long long* work;
    // cluster groups: the clusters one culling CTA owns.  Plain: group b is
    // [b*gw, min((b+1)*gw, C)); binned: group b is slice b / gps, clusters
    // [k*XY + (b % gps)*gw, min(.. + gw, (k+1)*XY)).
    uint32_t* group_sums;     // capped hit count of each group (plain path)
    uint32_t* group_offsets;  // exclusive scan of group_sums (plain path)
    uint32_t* queue;          // single-view binned launch: item counter, zeroed by the binning launch
    uint32_t lpad;
    uint32_t clusters;
    uint32_t cap;
    uint32_t slice_clusters;  // X * Y
    uint32_t slices;          // Z
    uint32_t group_width;     // gw = warps * clusters per warp (<= 32)
    uint32_t groups;
    uint32_t binned;
};

// One view of a batch: its culling state plus the inputs of the per-view
// stages, and where its blocks start in each batched launch.
struct ViewJob {
    ViewCull v;
    const CfLightData* lights;
    uint32_t light_count;
    uint32_t pad_[3];
    float view[16];  // cameraView, column-major
};

// First cluster and end of group b (see ViewCull).
__host__ __device__ inline void group_range(const ViewCull& v, uint32_t b, uint32_t* first, uint32_t* end)
{
    if (v.binned) {
        const uint32_t gps = (v.slice_clusters + v.group_width - 1) / v.group_width;
        const uint32_t k = b / gps;
        *first = k * v.slice_clusters + (b % gps) * v.group_width;
        const uint32_t e = *first + v.group_width, se = (k + 1) * v.slice_clusters;
        *end = e < se ? e : se;
    } else {
        *first = b * v.group_width;
        const uint32_t e = *first + v.group_width;
        *end = e < v.clusters ? e : v.clusters;
    }
}

inline uint32_t group_count(uint32_t clusters, uint32_t slice_clusters, uint32_t slices, uint32_t gw, int mode)
{
    return mode == kModeBinned ? slices * ((slice_clusters + gw - 1) / gw) : (clusters + gw - 1) / gw;
}

// One culling configuration: clusters per warp, consumer warps per CTA,
// lights per shared-memory stage, number of stages, mode.  A one-launch
// configuration reads them as clusters per CTA, warps per CTA, the most
// lights it takes (32 per warp and chunk), and 1.
struct CullConfig {
    int clusters_per_warp;
    int warps;
    int tile;
    int stages;
    int binned;  // kModeBruteForce, kModeBinned or kModeOneLaunch
};

// Clusters one culling CTA owns (a cluster group).
inline uint32_t group_width(const CullConfig& c)
{
    return c.binned == kModeOneLaunch ? (uint32_t)c.clusters_per_warp : (uint32_t)(c.warps * c.clusters_per_warp);
}

// Workspace carve-up for one view (cf_cull_lights).  A one-launch view needs
// only the status block and one 8-byte word per CTA (`partials`).
struct WorkspaceLayout {
    size_t vlights, nonfinite, counts, staging, group_sums, group_offsets, slice_lights, slice_idx, slice_count,
        slice_nonfinite, group_boxes, partials, bytes;
};
constexpr size_t kQueueWord = 64;   // byte offset, in a workspace's status block, of the single-view item counter
constexpr size_t kEpochWord = 128;  // byte offset of the one-launch kernel's epoch (see FusedCull)
// Scratch of one view; `groups` = group_count(...) of the configuration used.
WorkspaceLayout workspace_layout(uint32_t clusters, uint32_t lights, uint32_t cap, uint32_t slices, int mode,
                                 uint32_t groups);

// One-launch culling of a small view (cf_fused.cu): light transform,
// LightCulling.comp's test for every (cluster, light) pair, the capped
// ordered lists, the cluster-order offsets and the packed output, all in one
// cooperative launch.  CTA b owns clusters [b*per_cta, (b+1)*per_cta); its
// warps transform their share of the lights into registers and test them
// against the CTA's clusters; each test's 32 results are one ballot mask.
// The CTA's capped hit total goes to partials[b] as (tag << 32) | total, and
// each CTA sums the totals of the CTAs before it: that is its output offset.
// The tag is *epoch + 1, read at kernel start; the last CTA stores it back
// into *epoch once every CTA has published (so each CTA has read the old
// value), and words from earlier launches never carry the current tag.  The
// workspace must be zero-filled once after allocation.
struct FusedCull {
    const CfLightData* lights;
    const float4* aabbs;
    CfLightCell* cells;
    uint32_t* indices;
    uint32_t* total;                // may be null
    unsigned long long* partials;   // ctas words
    uint32_t* epoch;
    unsigned long long* work;       // optional work counters (see ViewCull)
    float view[16];                 // cameraView, column-major
    uint32_t light_count;
    uint32_t clusters;
    uint32_t cap;
    uint32_t per_cta;               // clusters per CTA, <= kOneLaunchMaxClustersPerCta
    uint32_t ctas;
};
constexpr uint32_t kOneLaunchMaxLights = 2048;
constexpr uint32_t kOneLaunchMaxClustersPerCta = 32;
constexpr uint32_t kOneLaunchMaxCtas = 256;
// The compiled one-launch shapes: (warps per CTA, most lights) = (32, 1024), (16, 2048), (16, 1024).
bool one_launch_shape_supported(int warps, int max_lights);
// CTAs of that shape that can be resident at once on the current device.
cudaError_t one_launch_resident_ctas(int warps, int max_lights, int* ctas);
// The one-launch configuration for a view, if one fits (false otherwise).
bool one_launch_config(uint32_t clusters, uint32_t lights, CullConfig* cfg);
cudaError_t launch_one_launch(const FusedCull& f, int warps, int max_lights, uint32_t* dev_error, cudaStream_t stream);

bool cull_config_supported(const CullConfig& c);
CullConfig default_cull_config(uint32_t clusters, uint32_t lights, uint32_t slices);

// Test knobs of the culling kernels on the current device (cf_device.cuh):
// the bounded-wait limit and the injected stall bits, per translation unit.
cudaError_t set_test_knobs_kernels(uint64_t wait_limit_ns, uint32_t inject);
cudaError_t set_test_knobs_one_launch(uint64_t wait_limit_ns, uint32_t inject);

cudaError_t launch_aabb(const CfClusterForwardUBO& ubo, CfAABB* aabbs, cudaStream_t stream);
cudaError_t launch_light_xform(const CfLightData* lights, uint32_t count, const float view[16], float4* vlights,
                               uint32_t* nonfinite, cudaStream_t stream);
cudaError_t launch_bin(const ViewCull& v, cudaStream_t stream);
cudaError_t launch_cull(const ViewCull& v, const CullConfig& cfg, uint32_t* dev_error, cudaStream_t stream);
cudaError_t launch_finalize(const ViewCull& v, cudaStream_t stream);
// total, cells and min(total, capacity) indices of one view into device-addressable host memory
cudaError_t launch_readback(const CfLightCell* cells, uint32_t clusters, const uint32_t* indices,
                            const uint32_t* d_total, uint64_t capacity, CfLightCell* h_cells, uint32_t* h_indices,
                            uint32_t* h_total, cudaStream_t stream);
// Jitters of many light sets in as few launches as possible (one per run of
// tasks none of which reads another's output), in task order: each task's
// dst = src with positions moved by sigma * (Irwin-Hall variate) from (seed,
// light, axis).
struct JitterTask {
    const CfLightData* src;
    CfLightData* dst;
    uint64_t seed;
    uint32_t n;
    float sigma;
};
constexpr uint32_t kMaxJitterTasks = 32;  // tasks per launch (passed by value)
cudaError_t launch_jitter_tasks(const JitterTask* tasks, uint32_t n, cudaStream_t stream);
// Copies of many buffers from device-mapped pinned host memory (16-byte
// aligned, whole 16-byte words) in as few launches as possible.
struct UploadTask {
    const uint4* src;  // the host buffer's device-side address
    uint4* dst;
    uint32_t words;    // 16-byte words
};
constexpr uint32_t kMaxUploadTasks = 48;  // tasks per launch (passed by value)
cudaError_t launch_upload_tasks(const UploadTask* tasks, uint32_t n, cudaStream_t stream);
// Every light `frames` steps along its orbit, in place (CfLightOrbit).
cudaError_t launch_orbits(CfLightData* lights, CfLightOrbit* orbits, uint64_t n, uint32_t frames, cudaStream_t stream);

// AABBs of many views in one launch: view v owns blocks [prefix[v], prefix[v+1])
// of 256 clusters each.
struct AabbJob {
    CfClusterForwardUBO ubo;
    CfAABB* out;
    uint64_t _pad;
};
cudaError_t launch_batch_aabb(const AabbJob* jobs, const uint32_t* prefix, uint32_t n_views, uint32_t blocks,
                              cudaStream_t stream);

// Batches: every stage of many views in one launch (the culling stage once per
// shape bucket).  `prefix` arrays hold, per view, the first block of that view
// in the launch; `blocks` is the launch's total.
struct BatchCull {
    const ViewJob* jobs;
    const uint2* items;  // (view, group) in the order the queue hands them out
    uint32_t n_items;
    uint32_t* queue;     // reset to 0 by launch_batch_xform
};
constexpr uint32_t kMaxBatchQueues = 256;  // queues a batch_xform launch resets (<= its block size)
cudaError_t launch_batch_xform(const ViewJob* jobs, const uint32_t* prefix, uint32_t n_views, uint32_t blocks,
                               uint32_t* queues, uint32_t n_queues, cudaStream_t stream);
// order (optional): view index per block range, prefix then follows that order
cudaError_t launch_batch_bin(const ViewJob* jobs, const uint32_t* prefix, const uint32_t* order, uint32_t n_views,
                             uint32_t blocks, cudaStream_t stream);
cudaError_t launch_batch_cull(const BatchCull& b, const CullConfig& cfg, int ctas, uint32_t* dev_error,
                              cudaStream_t stream);
cudaError_t batch_cull_resident_ctas(const CullConfig& cfg, int* ctas);
cudaError_t launch_batch_scan(const ViewJob* jobs, uint32_t n_views, cudaStream_t stream);
cudaError_t launch_batch_copy(const ViewJob* jobs, const uint32_t* prefix, uint32_t n_views, uint32_t blocks,
                              cudaStream_t stream);
uint32_t copy_blocks(uint32_t groups);  // blocks of the copy launch for a view of `groups` cluster groups
uint32_t bin_blocks(uint32_t slices);   // blocks of a batched binning launch for a view of `slices` depth slices

}  // namespace cfk
