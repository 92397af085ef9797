/*
 * cfcull.h — C ABI of the GB300 clustered-forward light-culling library.
 *
 * The library replaces the two compute passes of HelloVulkan's clustered
 * forward renderer — the cluster AABB generator and the light culling pass —
 * with CUDA kernels for sm_103a.  Its objects mirror the reference's plugin
 * classes one to one, so a host that drove
 *
 *     ResourcesLight, ResourcesClusterForward,
 *     PipelineAABBGenerator, PipelineLightCulling
 *
 * drives the same calls here (each declaration cites the member it
 * replaces).  Buffers keep the reference layouts (cf_types.h), so the
 * LightCell list and the light-index list feed the unchanged cluster-forward
 * fragment shader (Shaders/ClusteredForward/Scene.frag:64-78,119-134).
 *
 * Conventions
 *  - Every function returns a CfStatus (0 = success) and never throws.
 *    cf_last_error_message() gives a human-readable detail of the last failure
 *    on the calling thread.
 *  - `stream` arguments are cudaStream_t passed as void* (NULL = the legacy
 *    default stream).  Work is enqueued asynchronously unless stated.
 *  - Handles are not thread-safe; use one per thread or serialise.
 *  - The caller owns host memory; the library owns the device memory of its
 *    objects.  Device pointers returned by *_get_* stay valid until the
 *    object is destroyed or its buffers are re-created.
 *  - Light indices are 32-bit and view-local; the index list is packed in
 *    cluster order: cell c's indices start at the exclusive prefix sum of the
 *    counts of clusters 0..c-1.  The reference reserves the same slices with
 *    a global atomicAdd (LightCulling.comp:79), which gives the same cells
 *    and list when its workgroups run in index order and a permutation of the
 *    slices otherwise; each cluster's own list is identical in both cases:
 *    the first max_lights_per_cluster hits in ascending light order.
 */
#ifndef CFCULL_H
#define CFCULL_H

#include <stddef.h>
#include <stdint.h>

#include "cf_types.h"

#if defined(__GNUC__)
#define CFCULL_API __attribute__((visibility("default")))
#else
#define CFCULL_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

typedef enum CfStatus {
    CF_SUCCESS = 0,
    CF_ERROR_INVALID_ARGUMENT = 1, /* null handle/pointer, zero or oversized grid, cap 0, ... */
    CF_ERROR_OUT_OF_MEMORY = 2,    /* a device or pinned allocation failed                  */
    CF_ERROR_CUDA = 3,             /* a CUDA runtime call failed (see the message)          */
    CF_ERROR_CAPACITY = 4,         /* an output or workspace buffer is too small            */
    CF_ERROR_NOT_READY = 5,        /* a required input (UBO, lights, buffers) was never set */
    CF_ERROR_DEVICE_TIMEOUT = 6,   /* a bounded wait inside a kernel gave up                */
    CF_ERROR_BUDGET = 7,           /* an admission would exceed the device-memory budget    */
    CF_ERROR_UNSUPPORTED = 8,      /* no usable sm_103 device                              */
} CfStatus;

CFCULL_API const char* cf_status_string(int status);
/* Detail of the most recent failing call on this thread ("" if none). */
CFCULL_API const char* cf_last_error_message(void);
/* Library version as 10000*major + 100*minor + patch. */
CFCULL_API int cf_version(void);

/* ------------------------------------------------------------------------ */
/* Context: one CUDA device (stands in for VulkanContext).                  */
/* ------------------------------------------------------------------------ */
typedef struct CfContext CfContext;

CFCULL_API int cf_context_create(int device, CfContext** out);
CFCULL_API int cf_context_destroy(CfContext* ctx);
/* Reads and clears the device-side error word that bounded in-kernel waits
 * set on timeout (0 = none).  Synchronises the device. */
CFCULL_API int cf_context_check_device_error(CfContext* ctx, uint32_t* device_error);

/* ------------------------------------------------------------------------ */
/* ResourcesLight — Header/Resources/ResourcesLight.h:42-81                  */
/* ------------------------------------------------------------------------ */
typedef struct CfResourcesLight CfResourcesLight;

CFCULL_API int cf_resources_light_create(CfContext* ctx, CfResourcesLight** out);
CFCULL_API int cf_resources_light_destroy(CfResourcesLight* res);
/* ResourcesLight::AddLights (Source/Resources/ResourcesLight.cpp:8-18):
 * replaces the light set with `count` records and uploads them.  Synchronous. */
CFCULL_API int cf_resources_light_add_lights(CfResourcesLight* res, const CfLightData* lights, uint32_t count);
/* Asynchronous upload into the existing device buffer (grown if needed,
 * which synchronises).  `lights` should be pinned for a truly async copy. */
CFCULL_API int cf_resources_light_upload_async(CfResourcesLight* res, const CfLightData* lights, uint32_t count,
                                               void* stream);
/* ResourcesLight::UpdateLightPosition (Source/Resources/ResourcesLight.cpp:20-29):
 * sets light `index` to (x, y, z, 1).  Out-of-range indices are ignored, as
 * in the reference.  Synchronous. */
CFCULL_API int cf_resources_light_update_light_position(CfResourcesLight* res, uint32_t index, const float position[3]);
/* ResourcesLight::GetLightCount */
CFCULL_API int cf_resources_light_get_light_count(const CfResourcesLight* res, uint32_t* count);
/* ResourcesLight::GetVulkanBufferPtr: device pointer to the CfLightData array. */
CFCULL_API int cf_resources_light_get_device_buffer(const CfResourcesLight* res, const CfLightData** device_lights);

/* ------------------------------------------------------------------------ */
/* ResourcesClusterForward — Header/Resources/ResourcesClusterForward.h:11-31 */
/* ------------------------------------------------------------------------ */
typedef struct CfResourcesClusterForward CfResourcesClusterForward;

typedef struct CfClusterForwardBuffers {
    CfAABB* aabbs;            /* aabbBuffer_:         cluster_count records       */
    CfLightCell* light_cells; /* lightCellsBuffer_:   cluster_count records       */
    uint32_t* light_indices;  /* lightIndicesBuffer_: index_capacity entries      */
    uint32_t* total_indices;  /* one uint32: indices written by the last culling  */
    uint32_t cluster_count;
    uint32_t max_lights_per_cluster;
    uint64_t index_capacity;  /* = cluster_count * max_lights_per_cluster         */
} CfClusterForwardBuffers;

CFCULL_API int cf_resources_cluster_forward_create(CfContext* ctx, CfResourcesClusterForward** out);
CFCULL_API int cf_resources_cluster_forward_destroy(CfResourcesClusterForward* res);
/* ResourcesClusterForward::CreateBuffers (Source/Resources/ResourcesClusterForward.cpp:5-34)
 * with the grid and cap as arguments instead of compile-time constants
 * (the reference uses 16 x 9 x 24 and 150).  Marks the AABBs dirty. */
CFCULL_API int cf_resources_cluster_forward_create_buffers(CfResourcesClusterForward* res, uint32_t slice_count_x,
                                                           uint32_t slice_count_y, uint32_t slice_count_z,
                                                           uint32_t max_lights_per_cluster);
CFCULL_API int cf_resources_cluster_forward_get_buffers(const CfResourcesClusterForward* res,
                                                        CfClusterForwardBuffers* out);
/* ResourcesClusterForward::aabbDirty_ */
CFCULL_API int cf_resources_cluster_forward_is_aabb_dirty(const CfResourcesClusterForward* res, int* dirty);
/* Copies the cells and the first min(total, host_index_capacity) indices to
 * host memory and returns the total; synchronises `stream`.  When both host
 * buffers are pinned memory the device can address (cudaHostAlloc /
 * cudaHostRegister, e.g. torch's pin_memory), one kernel writes total, cells
 * and indices straight into them and the call waits once; other buffers go
 * through two copies and two waits (the total first, then the indices). */
CFCULL_API int cf_resources_cluster_forward_read_outputs(CfResourcesClusterForward* res, CfLightCell* host_cells,
                                                         uint32_t* host_indices, uint64_t host_index_capacity,
                                                         uint32_t* total, void* stream);

/* ------------------------------------------------------------------------ */
/* PipelineAABBGenerator — Header/Pipelines/PipelineAABBGenerator.h:17-39    */
/* ------------------------------------------------------------------------ */
typedef struct CfPipelineAABBGenerator CfPipelineAABBGenerator;

CFCULL_API int cf_pipeline_aabb_generator_create(CfContext* ctx, CfResourcesClusterForward* res_cf,
                                                 CfPipelineAABBGenerator** out);
CFCULL_API int cf_pipeline_aabb_generator_destroy(CfPipelineAABBGenerator* pipe);
/* PipelineAABBGenerator::SetClusterForwardUBO.  A UBO whose projection part
 * (inverse projection, near, far, grid) differs from the one the AABBs were
 * built from marks the AABBs dirty, so zoom changes also regenerate them. */
CFCULL_API int cf_pipeline_aabb_generator_set_cluster_forward_ubo(CfPipelineAABBGenerator* pipe,
                                                                  const CfClusterForwardUBO* ubo);
/* PipelineAABBGenerator::OnWindowResized (PipelineAABBGenerator.cpp:31-34) */
CFCULL_API int cf_pipeline_aabb_generator_on_window_resized(CfPipelineAABBGenerator* pipe);
/* PipelineAABBGenerator::FillCommandBuffer (PipelineAABBGenerator.cpp:36-47):
 * enqueues the generator on `stream` when the AABBs are dirty, else nothing. */
CFCULL_API int cf_pipeline_aabb_generator_fill_command_buffer(CfPipelineAABBGenerator* pipe, void* stream);

/* ------------------------------------------------------------------------ */
/* PipelineLightCulling — Header/Pipelines/PipelineLightCulling.h:18-30      */
/* ------------------------------------------------------------------------ */
typedef struct CfPipelineLightCulling CfPipelineLightCulling;

CFCULL_API int cf_pipeline_light_culling_create(CfContext* ctx, CfResourcesLight* res_light,
                                                CfResourcesClusterForward* res_cf, CfPipelineLightCulling** out);
CFCULL_API int cf_pipeline_light_culling_destroy(CfPipelineLightCulling* pipe);
/* PipelineLightCulling::ResetGlobalIndex (PipelineLightCulling.cpp:38-43).
 * Kept for call compatibility; offsets come from a prefix scan, so there is
 * no counter to reset and this does nothing. */
CFCULL_API int cf_pipeline_light_culling_reset_global_index(CfPipelineLightCulling* pipe);
/* PipelineLightCulling::SetClusterForwardUBO (PipelineLightCulling.cpp:45-49) */
CFCULL_API int cf_pipeline_light_culling_set_cluster_forward_ubo(CfPipelineLightCulling* pipe,
                                                                 const CfClusterForwardUBO* ubo);
/* PipelineLightCulling::FillCommandBuffer (PipelineLightCulling.cpp:51-119):
 * enqueues light transform, culling and the offset scan on `stream` — for a
 * small view (at most 2048 lights, clusters spread at most 32 per SM) all
 * three in one kernel launch. */
CFCULL_API int cf_pipeline_light_culling_fill_command_buffer(CfPipelineLightCulling* pipe, void* stream);

/* Tuning: selects the culling kernel configuration (clusters per warp,
 * consumer warps per CTA, lights per shared-memory stage, stages, and the
 * mode: binned = 0 every light against every cluster, 1 the depth-slice
 * candidate lists first, 2 the whole step in one launch, for which the
 * arguments are clusters per CTA (1..32), warps per CTA, the most lights the
 * launch takes and 1 — (M, 32, 1024, 1, 2), (M, 16, 2048, 1, 2) or
 * (M, 16, 1024, 1, 2); a view with more lights than that is rejected when
 * culled); clusters_per_warp = 0 restores the automatic choice.  Unsupported
 * combinations are rejected.  Every configuration gives the same output. */
CFCULL_API int cf_pipeline_light_culling_set_tuning(CfPipelineLightCulling* pipe, int clusters_per_warp, int warps,
                                                    int tile, int stages, int binned);
/* The configuration the next fill_command_buffer uses (the override, or the
 * automatic choice for the current UBO and light count): clusters per warp,
 * warps, tile, stages, binned. */
CFCULL_API int cf_pipeline_light_culling_get_tuning(const CfPipelineLightCulling* p, int config[5]);
/* Stage timing, the counterpart of the reference's Tracy GPU zone
 * "Light_Culling" (PipelineLightCulling.cpp:53): when enabled, each
 * fill_command_buffer records CUDA events around its three kernels, and
 * get_stage_times returns the last call's light-transform, culling and
 * offset-scan durations in milliseconds (waits for them). */
CFCULL_API int cf_pipeline_light_culling_enable_stage_timing(CfPipelineLightCulling* pipe, int enable);
CFCULL_API int cf_pipeline_light_culling_get_stage_times(CfPipelineLightCulling* pipe, float ms[3]);
/* Work counters for profiling: when enabled, the kernels add up the
 * sphere-box tests they execute — counters[0] against depth-slice slabs and
 * per-warp union boxes, counters[1] against cluster boxes.  read returns the
 * sums since the last read and clears them (synchronises the device). */
CFCULL_API int cf_pipeline_light_culling_enable_work_counters(CfPipelineLightCulling* pipe, int enable);
CFCULL_API int cf_pipeline_light_culling_read_work_counters(CfPipelineLightCulling* pipe, uint64_t counters[2]);

/* ------------------------------------------------------------------------ */
/* Batches: many views culled together.  No counterpart in the reference,     */
/* which culls one view per frame; each view's outputs are the ones           */
/* PipelineLightCulling would produce for it.                                 */
/* ------------------------------------------------------------------------ */
typedef struct CfBatch CfBatch;

/* One view of a batch; every pointer is caller-owned device memory that must
 * stay valid while the batch uses it. */
typedef struct CfBatchView {
    CfClusterForwardUBO ubo;        /* grid, projection and view of this view     */
    const CfLightData* d_lights;    /* light_count records                        */
    CfAABB* d_aabbs;                /* X*Y*Z boxes (written by generate_aabbs)    */
    CfLightCell* d_cells;           /* X*Y*Z cells (output)                       */
    uint32_t* d_indices;            /* index list (output)                        */
    uint32_t* d_total;              /* optional: indices written (output)         */
    uint64_t index_capacity;        /* >= X*Y*Z * max_lights_per_cluster          */
    uint32_t light_count;
    uint32_t max_lights_per_cluster;
    uint32_t _pad[2];
} CfBatchView;

typedef struct CfBatchInfo {
    uint32_t views, items, buckets, _pad;
    uint64_t workspace_bytes;
    uint32_t bucket_slice_clusters[8]; /* first 8 buckets: X*Y of their views      */
    int32_t bucket_config[8][4];       /* clusters/warp, warps, tile, stages        */
    int32_t bucket_ctas[8];            /* persistent CTAs of their culling launch   */
} CfBatchInfo;

CFCULL_API int cf_batch_create(CfContext* ctx, CfBatch** out);
CFCULL_API int cf_batch_destroy(CfBatch* batch);
/* Replaces the batch's views (copied); allocates its workspace and builds its
 * work-item tables.  Synchronous: it first waits for every pass and AABB
 * generation the batch enqueued (outside a stream capture) to finish, since
 * those read the tables it rewrites.  cf_batch_set_tuning,
 * cf_batch_update_view_matrices and cf_batch_set_graph wait the same way. */
CFCULL_API int cf_batch_set_views(CfBatch* batch, const CfBatchView* views, uint32_t count);
/* Updates the view matrices (cameraView of each UBO; the projection part must
 * not change) for the next cf_batch_cull.  Synchronises `stream`. */
CFCULL_API int cf_batch_update_view_matrices(CfBatch* batch, const CfClusterForwardUBO* ubos, uint32_t count,
                                             void* stream);
/* AABBGenerator.comp for every view into its d_aabbs. */
CFCULL_API int cf_batch_generate_aabbs(CfBatch* batch, void* stream);
/* One culling pass over every view.  With graphs enabled (the default) and a
 * non-null stream, the first call captures the pass into a CUDA graph and
 * later calls replay it. */
CFCULL_API int cf_batch_cull(CfBatch* batch, void* stream);
CFCULL_API int cf_batch_set_graph(CfBatch* batch, int enable);
/* Fixes the culling configuration of the views whose grid has slice_clusters
 * = X*Y clusters per depth slice (clusters_per_warp 0 = default). */
CFCULL_API int cf_batch_set_tuning(CfBatch* batch, uint32_t slice_clusters, int clusters_per_warp, int warps,
                                   int tile, int stages);
/* Times every candidate configuration on the current views, `repeats` passes
 * each, and keeps the fastest per shape bucket (views sharing X*Y). */
CFCULL_API int cf_batch_autotune(CfBatch* batch, int repeats, void* stream);
CFCULL_API int cf_batch_get_info(const CfBatch* batch, CfBatchInfo* info);

/* ------------------------------------------------------------------------ */
/* Server: culling requests admitted as they arrive (continuous batching).    */
/* No counterpart in the reference.  A request names a view (UBO) and a light */
/* set resident on the device; the server keeps light sets and the AABBs of   */
/* each projection resident, admits requests in arrival order within a fixed  */
/* device-memory budget, and launches every admissible pending request as one */
/* batch whenever one of its streams is free, so batches overlap on the GPU.  */
/* ------------------------------------------------------------------------ */
typedef struct CfServer CfServer;

typedef struct CfServerConfig {
    uint64_t hbm_budget_bytes;     /* device memory for light sets, AABBs, scratch and outputs (default 8 GiB) */
    uint32_t max_batch_views;      /* views per launch (default 64)                                         */
    uint32_t streams;              /* batches in flight at once (default 4)                                  */
    uint32_t max_pending;          /* submissions waiting for admission (default 4096; past it CF_ERROR_BUDGET) */
    uint32_t max_groups_per_view;  /* largest view, in cluster groups (default 16384)                        */
} CfServerConfig;

typedef struct CfServerRequest {
    CfClusterForwardUBO ubo;
    uint64_t light_set;              /* id from cf_server_register_light_set            */
    uint64_t user_tag;               /* returned in the completion                      */
    uint32_t max_lights_per_cluster; /* 0 = 150                                         */
    uint32_t _pad[3];
} CfServerRequest;

typedef struct CfServerCompletion {
    uint64_t request_id, user_tag;
    int32_t status;                  /* CF_SUCCESS, CF_ERROR_NOT_READY (light set not resident), CF_ERROR_BUDGET ... */
    uint32_t clusters;
    double t_submit, t_launch, t_complete; /* seconds since the server was created (host steady clock) */
    const CfLightCell* d_cells;      /* device results, valid until cf_server_release   */
    const uint32_t* d_indices;
    const uint32_t* d_total;
} CfServerCompletion;

typedef struct CfServerStats {
    uint64_t submitted, completed, batches, views_launched, max_pending, evictions;
    uint64_t arena_bytes, arena_used_bytes, arena_peak_bytes, pending, resident_light_sets, resident_projections;
    uint32_t max_batch_views, max_held_outputs; /* most completed requests at once whose outputs were not released */
} CfServerStats;

CFCULL_API int cf_server_create(CfContext* ctx, const CfServerConfig* config, CfServer** out);
/* Finishes every submitted request, then frees everything. */
CFCULL_API int cf_server_destroy(CfServer* server);
/* Uploads a light set (device memory from the budget; CF_ERROR_BUDGET if it
 * cannot fit).  Sets no submitted request uses are evicted least recently
 * used when admission needs room; submitting against an evicted set returns
 * CF_ERROR_NOT_READY (register it again).  The copy follows cudaMemcpyAsync's
 * rule: from pageable memory `lights` is copied before the call returns and
 * is then free to reuse; from pinned (page-locked, 16-byte aligned) memory
 * the call makes no copy: the server's worker reads `lights` from the device,
 * together with the other queued uploads and jitters, before the next batch
 * (or within a few ms when idle), so `lights` must stay allocated and
 * unchanged until the first request that uses the set has completed, and at
 * least until cf_server_destroy if none does (cf_server_update_light_set
 * likewise). */
CFCULL_API int cf_server_register_light_set(CfServer* server, const CfLightData* lights, uint32_t count, uint64_t* id);
/* Declares host memory [host, host + bytes) pinned for the server's lifetime:
 * the caller keeps it allocated and page-locked until cf_server_destroy.
 * Registers and updates whose lights lie inside a declared range then make no
 * CUDA call at all (an undeclared pointer costs one cudaPointerGetAttributes).
 * Every page is checked once here: CF_ERROR_INVALID_ARGUMENT if any is not
 * pinned and mapped for the device, the mapping is not linear, or the range
 * overlaps another declared range (declaring the same range again is a
 * no-op).  A client with a pool of pinned staging buffers declares the pool. */
CFCULL_API int cf_server_declare_pinned_host(CfServer* server, const void* host, size_t bytes);
/* Replaces a set's lights for requests submitted from now on (copy on write:
 * a request binds the set's version current when it is submitted). */
CFCULL_API int cf_server_update_light_set(CfServer* server, uint64_t id, const CfLightData* lights, uint32_t count);
/* Moves every light of a set on the device, copy on write like an update:
 * position += sigma * (s - 6), s the sum of 12 uniforms in [0, 1) drawn from
 * a splitmix64 hash of (seed + light * 0x9E3779B97F4A7C15 + (axis * 12 + term)
 * * 0xD1B54A32D192ED03), u = (hash >> 40) * 2^-24, every operation rounded
 * to nearest in that order, so a host can reproduce the result bit for bit.
 * The call makes no CUDA call: the server's worker launches every queued
 * jitter (up to 32 sets per launch) on the upload stream ahead of the next
 * batch's upload fence, or alone when no batch is ready, so every request that
 * binds the new version reads it after it is written. */
CFCULL_API int cf_server_jitter_light_set(CfServer* server, uint64_t id, uint64_t seed, float sigma);
CFCULL_API int cf_server_release_light_set(CfServer* server, uint64_t id);
CFCULL_API int cf_server_is_light_set_resident(CfServer* server, uint64_t id, int* resident);
/* Thread-safe. */
CFCULL_API int cf_server_submit(CfServer* server, const CfServerRequest* request, uint64_t* request_id);
/* Up to `max` completions, waiting up to wait_ms for the first one. */
CFCULL_API int cf_server_poll(CfServer* server, CfServerCompletion* out, uint32_t max, uint32_t* count, int wait_ms);
/* Returns a completed request's device results to the budget. */
CFCULL_API int cf_server_release(CfServer* server, uint64_t request_id);
/* cf_server_release for n requests under one acquisition of the server's
 * lock (a poller releasing what one cf_server_poll returned).  Ids that hold
 * no outputs are skipped; the call then returns CF_ERROR_INVALID_ARGUMENT
 * after releasing every other one. */
CFCULL_API int cf_server_release_many(CfServer* server, const uint64_t* request_ids, uint32_t n);
CFCULL_API int cf_server_set_tuning(CfServer* server, uint32_t slice_clusters, int clusters_per_warp, int warps,
                                    int tile, int stages);
CFCULL_API int cf_server_get_stats(CfServer* server, CfServerStats* stats);

/* A served stream replayed in real time against a server (load driver for
 * measurement): Poisson arrivals at rate_per_s for duration_s; each request
 * takes one of the projections (its cameraView is replaced by a look-at from
 * an eye uniform in [eye_lo, eye_hi] to a target uniform in
 * [target_lo, target_hi]) and, with probability p_reuse, one of its
 * submitting thread's recent light sets moved by cf_server_jitter_light_set
 * (sigma jitter_sigma), else a new set copied from base_sets.  recent_sets
 * is split across submit_threads; sets leaving a window are released.  Base
 * sets in pinned memory are declared to the server first
 * (cf_server_declare_pinned_host), so they must stay allocated until
 * cf_server_destroy; pageable ones are copied at each register. */
typedef struct CfServeLoad {
    double rate_per_s, duration_s, p_reuse;
    uint64_t seed;
    float jitter_sigma;
    uint32_t recent_sets, submit_threads, max_lights_per_cluster;
    uint32_t n_projections, n_base_sets;
    const CfClusterForwardUBO* projections;
    const CfLightData* const* base_sets;
    const uint32_t* base_counts;
    float eye_lo[3], eye_hi[3], target_lo[3], target_hi[3];
} CfServeLoad;

typedef struct CfServeReport {
    uint64_t scheduled, submitted, completed, failed, new_sets, reused_sets, tests_brute_force;
    double wall_s, offered_rate, achieved_rate;
    double latency_p50_ms, latency_p90_ms, latency_p99_ms, latency_p999_ms, latency_max_ms; /* arrival -> done */
    double queue_p50_ms, queue_p99_ms;                                                     /* arrival -> launch */
    double submit_lag_p99_ms;                                                              /* arrival -> submit */
    double exec_p50_ms, exec_p99_ms;                                                       /* launch -> done    */
    double register_call_p50_us, register_call_p99_us;  /* time inside cf_server_register_light_set */
    double jitter_call_p50_us, jitter_call_p99_us;      /* time inside cf_server_jitter_light_set   */
    double submit_call_p50_us, submit_call_p99_us;      /* time inside cf_server_submit             */
    double register_call_max_us, jitter_call_max_us, submit_call_max_us;
    double worst_lag_arrival_s;                         /* scheduled arrival of the most delayed submit */
} CfServeReport;

CFCULL_API int cf_serve_run_load(CfServer* server, const CfServeLoad* load, CfServeReport* report);

/* ------------------------------------------------------------------------ */
/* Stateless entry points on caller-owned device memory.                     */
/* ------------------------------------------------------------------------ */

/* Bytes of device workspace cf_cull_lights needs for a view of this grid
 * (ubo: host pointer) and light count. */
CFCULL_API int cf_cull_workspace_size(const CfClusterForwardUBO* ubo, uint32_t light_count,
                                      uint32_t max_lights_per_cluster, uint64_t* bytes);
/* AABBGenerator.comp over the grid of `ubo` (host pointer) into
 * d_aabbs[X*Y*Z] (device). */
CFCULL_API int cf_generate_aabbs(const CfClusterForwardUBO* ubo, CfAABB* d_aabbs, void* stream);
/* Moves d_lights[0..count) `frames` steps along their orbits d_orbits[0..count)
 * in place (CfLightOrbit, include/cf_types.h); both device buffers, 16-byte
 * aligned; stream-ordered, so a cull enqueued after it on the same stream sees
 * the new positions.  The device-side counterpart of
 * ResourcesLight::UpdateLightPosition (Source/Resources/ResourcesLight.cpp:20-29)
 * for every light at once. */
CFCULL_API int cf_animate_light_orbits(CfLightData* d_lights, CfLightOrbit* d_orbits, uint64_t count, uint32_t frames,
                                       void* stream);
/* Scene.frag's cluster lookup (Shaders/ClusteredForward/Scene.frag:54-78)
 * for every pixel of a depth buffer, as a check that the (offset, count)
 * cells drop into the reference's fragment pass: d_depth is width x height
 * window-space depths (0..1, ZO), row-major from the top row, width and
 * height equal to ubo->screenSize; fragment (x, y) is at the pixel centre.
 * LinearDepth, log2 and the tile division follow the shader with log2
 * pinned (cf_log2_pinned).  For each pixel d_out receives the cluster, its
 * cell, the number of its listed lights whose sphere contains the fragment's
 * view-space position, and flags; with check_all_lights != 0 also the number
 * of lights outside the list that contain it (every light is tested), which
 * is 0 unless the fragment lies outside its cluster's AABB or the list is
 * capped.  d_aabbs (optional) enables CF_FRAGMENT_OUTSIDE_AABB.  Light lists
 * must be in ascending light order, as this library writes them; index_count
 * bounds the index list (a cell reaching beyond it, or an index >= light_count,
 * is flagged CF_FRAGMENT_BAD_CELL and nothing is read through it). */
CFCULL_API int cf_lookup_clusters(const CfClusterForwardUBO* ubo, const float* d_depth, uint32_t width,
                                  uint32_t height, const CfLightCell* d_cells, const uint32_t* d_indices,
                                  uint64_t index_count, const CfLightData* d_lights, uint32_t light_count,
                                  uint32_t max_lights_per_cluster, const CfAABB* d_aabbs, int check_all_lights,
                                  CfFragmentSample* d_out, void* stream);
/* Scene.frag's direct clustered lighting for every texel of a G-buffer:
 * the cluster lookup of cf_lookup_clusters on the texel's depth and pixel,
 * then Lo = albedo * albedoMultipler + the sum of Radiance(...)
 * (Shaders/ClusteredForward/Radiance.glsl:2-57, Scene.frag:82-135) over the
 * cluster's listed lights, with V = normalize(camera_position - world
 * position) and F0 = mix(baseReflectivity, albedo, metallic).  The shader's
 * implementation-defined parts are pinned: normalize(v) = v / sqrt(dot(v, v))
 * and length = sqrt(dot) with the correctly rounded sqrt, dot summed x, y, z,
 * pow = cf_pow_pinned, every operation rounded to nearest in the shader's
 * order.  The ambient (IBL) and emissive terms, which need the engine's
 * textures, are not part of this pass.  d_out receives width x height float4
 * (Lo, 1); texels whose lookup leaves the grid or meets a bad cell get
 * (albedo * albedoMultipler, 0).  d_gbuffer and d_lights 16-byte aligned. */
CFCULL_API int cf_shade_clusters(const CfClusterForwardUBO* ubo, const float camera_position[3],
                                 const CfPBRPushConstant* pc, const CfGBufferTexel* d_gbuffer, uint32_t width,
                                 uint32_t height, const CfLightCell* d_cells, const uint32_t* d_indices,
                                 uint64_t index_count, const CfLightData* d_lights, uint32_t light_count,
                                 float* d_out, void* stream);
/* FrustumCulling.comp (Shaders/FrustumCulling.comp:14-57) for count boxes:
 * d_commands[i].instanceCount = 1 when box i may intersect the frustum (host
 * pointer; no plane has all 8 box corners behind it and no box face has all
 * 8 frustum corners beyond it), else 0; the other fields of the commands are
 * left as they are.  dot(plane, corner) is summed x, y, z, w in order.
 * d_visible (optional, device, zeroed by the caller) receives the number of
 * boxes kept.  The counterpart of PipelineFrustumCulling::FillCommandBuffer
 * (Source/Pipelines/PipelineFrustumCulling.cpp). */
CFCULL_API int cf_frustum_cull(const CfFrustum* frustum, const CfAABB* d_boxes, uint32_t count,
                               CfDrawIndirectCommand* d_commands, uint32_t* d_visible, void* stream);
/* LightCulling.comp: d_cells[C] and d_indices (capacity >= C * cap) from
 * d_aabbs[C] and d_lights[light_count]; d_total (optional, device) receives
 * the number of indices.  d_workspace: >= cf_cull_workspace_size bytes,
 * 256-byte aligned, zero-filled once after allocation (its first word is the
 * device error word that bounded in-kernel waits set on timeout). */
CFCULL_API int cf_cull_lights(const CfClusterForwardUBO* ubo, const CfAABB* d_aabbs, const CfLightData* d_lights,
                              uint32_t light_count, uint32_t max_lights_per_cluster, CfLightCell* d_cells,
                              uint32_t* d_indices, uint64_t index_capacity, uint32_t* d_total, void* d_workspace,
                              uint64_t workspace_bytes, void* stream);

/* Reads and clears the device error word of a cf_cull_lights workspace
 * (0 = none; CF_ERROR_DEVICE_TIMEOUT otherwise).  Synchronises the device. */
CFCULL_API int cf_cull_workspace_device_error(void* d_workspace, uint32_t* device_error);

/* No counterpart in the reference (its Vulkan buffers are all created up
 * front).  cf_cull_lights for callers that cannot allocate device memory when
 * they cull — a frame recorded inside a host allocator's critical section, a
 * plugin whose device memory its host reserves, a real-time loop that cannot
 * afford cudaMalloc/cudaFree.  Same inputs and outputs as cf_cull_lights, but
 * the scratch comes from a fixed 32 MiB device array that every GPU loading
 * this library holds until the process exits.  A view whose usual kernels
 * need more scratch than that (a 27 648-cluster grid with more than about
 * 17 500 lights at a cap of 150) is culled by the brute-force kernels, which
 * need less but run several times slower on such views; one that fits
 * neither way is rejected with CF_ERROR_CAPACITY.  The first call on a device
 * (and the first after its context was reset) looks up that array's address
 * and should come before any stream capture.  All calls on a device share the
 * array: calls that overlap on the GPU race and must be serialised.
 * d_device_error (optional, device) receives the bounded-wait error bits;
 * without it a timeout cannot be observed (the bits go to the array's own
 * word, which each call clears). */
CFCULL_API int cf_cull_lights_static_scratch(const CfClusterForwardUBO* ubo, const CfAABB* d_aabbs,
                                             const CfLightData* d_lights, uint32_t light_count,
                                             uint32_t max_lights_per_cluster, CfLightCell* d_cells,
                                             uint32_t* d_indices, uint64_t index_capacity, uint32_t* d_total,
                                             uint32_t* d_device_error, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* CFCULL_H */
