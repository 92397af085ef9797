// cf_runtime_internal.h — helpers shared by the host-side translation units.
#pragma once

#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>  // header-only NVTX v3: a no-op unless a profiler is attached
#include <stdint.h>

#include "cf_kernels.cuh"
#include "cf_types.h"

namespace cfrt {

constexpr uint32_t kMaxClusters = 1u << 22;  // 4 M clusters per view
constexpr uint32_t kMaxCap = 4096;           // per-cluster light cap
constexpr uint32_t kMaxLights = 1u << 26;    // 64 M lights per set

// Records a formatted message for cf_last_error_message() and returns status.
int fail(int status, const char* fmt, ...) __attribute__((format(printf, 2, 3)));
int cuda_fail(cudaError_t e, const char* what);

bool projection_equal(const CfClusterForwardUBO& a, const CfClusterForwardUBO& b);
bool device_addressable(const void* host, void** dev);
int validate_grid(uint32_t x, uint32_t y, uint32_t z, uint32_t cap, uint32_t* clusters);

// A named NVTX range on the calling host thread for the guard's lifetime, so
// that the enqueueing of each pass shows in a timeline profiler (nsys, ncu
// ranges): the counterpart of the reference's Tracy zones ("Light_Culling",
// PipelineLightCulling.cpp:53; "RecordCommandBuffer", AppBase.cpp:133).
class TraceRange {
public:
    explicit TraceRange(const char* name) { nvtxRangePushA(name); }
    ~TraceRange() { nvtxRangePop(); }
    TraceRange(const TraceRange&) = delete;
    TraceRange& operator=(const TraceRange&) = delete;
};

// Makes `device` current for the guard's lifetime.
class DeviceGuard {
public:
    explicit DeviceGuard(int device);
    ~DeviceGuard();
    cudaError_t err() const { return err_; }

private:
    int prev_ = -1;
    cudaError_t err_ = cudaSuccess;
};

// cudaMalloc, except that a test may make it fail (cf_testing_fail_allocation_after).
cudaError_t device_malloc(void** ptr, size_t bytes);

// True (and one fewer left) when a test asked the server's next launch of
// queued light-set uploads and jitters to fail (cf_testing_fail_version_writes).
bool take_injected_version_write_failure();

// Ensures *ptr holds at least `bytes` of zero-filled device memory.
int grow(void** ptr, size_t* capacity, size_t bytes, const char* what);

// The culling configuration for a view: the override, else the automatic choice.
cfk::CullConfig choose_config(const CfClusterForwardUBO& ubo, uint32_t light_count,
                              const cfk::CullConfig* override_cfg);
cfk::WorkspaceLayout layout_for(const CfClusterForwardUBO& ubo, uint32_t light_count, uint32_t cap,
                                const cfk::CullConfig& cfg);

// Light transform (+ slice binning) + culling + offset scan of one view on `stream`.
int enqueue_cull(const CfClusterForwardUBO& ubo, const CfAABB* d_aabbs, const CfLightData* d_lights,
                 uint32_t light_count, uint32_t cap, CfLightCell* d_cells, uint32_t* d_indices, uint32_t* d_total,
                 unsigned char* ws, uint32_t* dev_error, const cfk::CullConfig& cfg, cudaStream_t stream,
                 cudaEvent_t* stage_events, unsigned long long* work = nullptr);

}  // namespace cfrt
