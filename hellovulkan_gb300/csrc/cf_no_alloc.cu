// cf_no_alloc.cu — light culling for callers that cannot allocate device memory.
//
// Some hosts cannot call cudaMalloc at the point where they cull: a renderer
// recording its frame from inside a custom allocator's critical section, a
// plugin sandbox whose memory is reserved up front by its host, or a
// real-time loop where an allocation (and the device synchronisation that
// cudaFree implies) would blow the frame budget.  cf_cull_lights asks such a
// caller for a workspace it cannot provide.  cf_cull_lights_static_scratch
// runs the same three kernels, but takes their scratch (view-space lights,
// non-finite flags, per-cluster counts and the staging lists) from the fixed
// array below, which the CUDA runtime reserves when it loads this library on
// a device.
//
// Limits and rules:
//  - The array holds kStaticScratchBytes (32 MiB) on every GPU that loads the
//    library, for as long as the process runs.  The kernels the automatic
//    choice picks are used when their scratch fits: a 2560x1600 view of
//    27 648 clusters with 16 384 lights and a cap of 150 takes the binned
//    kernels' 31.2 MiB.  Past 32 MiB (that grid with more than about 17 500
//    lights) the call falls back to the brute-force kernels, whose scratch is
//    smaller (about 17 MB there) but which run several times slower on such
//    views (0.36 instead of 0.042 ms at 16 384 lights on a GB300).  A view
//    whose scratch fits neither way is rejected with CF_ERROR_CAPACITY.
//  - The first call on a device (and the first after that device's context
//    was reset) looks up the array's device address with
//    cudaGetSymbolAddress while that device is current; make that first call
//    before any stream capture that the call may be part of.
//  - Every call on a device shares the one array and it keeps the last call's
//    contents; calls whose kernels overlap on the GPU (different streams, or
//    threads) race on it and must be serialised by the caller.
//  - A bounded in-kernel wait that runs out is reported through the caller's
//    d_device_error word.  Without one the bits go to the array's own word,
//    which each call clears and nothing reads: pass a word to observe them.
//  - Nothing here allocates: no cudaMalloc, cudaFree or allocating library
//    call; the error word is cleared with cudaMemsetAsync.
#include <cuda.h>  // driver API types only: cuCtxGetId is looked up through the runtime
#include <cuda_runtime.h>

#include <mutex>

#include "cf_kernels.cuh"
#include "cf_runtime_internal.h"
#include "cfcull.h"

namespace {

constexpr size_t kStaticScratchBytes = 32u << 20;
constexpr int kMaxDevices = 64;

static __device__ __align__(256) unsigned char g_static_scratch[kStaticScratchBytes];

std::mutex g_scratch_mutex;
struct ScratchAddress {
    unsigned long long context_id = 0;  // the context the address belongs to (0: none yet)
    unsigned char* ptr = nullptr;
};
ScratchAddress g_scratch[kMaxDevices];

// Unique ID of the current context (cuCtxGetId, looked up through the
// runtime so that the driver library need not be linked); 0 if unavailable.
unsigned long long current_context_id()
{
    typedef CUresult (*GetCurrent)(CUcontext*);
    typedef CUresult (*GetId)(CUcontext, unsigned long long*);
    static GetCurrent get_current = nullptr;
    static GetId get_id = nullptr;
    static bool looked_up = false;
    if (!looked_up) {  // under g_scratch_mutex
        cudaDriverEntryPointQueryResult q1, q2;
        void* f1 = nullptr;
        void* f2 = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f1, 12000, cudaEnableDefault, &q1) == cudaSuccess &&
            q1 == cudaDriverEntryPointSuccess &&
            cudaGetDriverEntryPointByVersion("cuCtxGetId", &f2, 12000, cudaEnableDefault, &q2) == cudaSuccess &&
            q2 == cudaDriverEntryPointSuccess) {
            get_current = reinterpret_cast<GetCurrent>(f1);
            get_id = reinterpret_cast<GetId>(f2);
        }
        looked_up = true;
    }
    CUcontext ctx = nullptr;
    unsigned long long id = 0;
    if (!get_current || !get_id || get_current(&ctx) != CUDA_SUCCESS || !ctx || get_id(ctx, &id) != CUDA_SUCCESS)
        return 0;
    return id;
}

// Device address of g_static_scratch on the current device.  Looked up once
// per device and context: a context reset (cudaDeviceReset) reloads the
// module, so a new context ID triggers a new lookup; where no ID can be had
// the address is looked up on every call.
int scratch_address(unsigned char** out)
{
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return cfrt::cuda_fail(e, "cudaGetDevice");
    if (dev < 0 || dev >= kMaxDevices) return cfrt::fail(CF_ERROR_UNSUPPORTED, "device ordinal %d out of range", dev);
    std::lock_guard<std::mutex> lock(g_scratch_mutex);
    const unsigned long long id = current_context_id();  // 0 before the device's context exists
    ScratchAddress& c = g_scratch[dev];
    if (!c.ptr || id == 0 || c.context_id != id) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_static_scratch);  // also makes the device's context current
        if (e != cudaSuccess) return cfrt::cuda_fail(e, "cudaGetSymbolAddress(static scratch)");
        c.ptr = static_cast<unsigned char*>(p);
        c.context_id = current_context_id();
    }
    *out = c.ptr;
    return CF_SUCCESS;
}

}  // namespace

extern "C" int cf_cull_lights_static_scratch(const CfClusterForwardUBO* ubo, const CfAABB* d_aabbs,
                                             const CfLightData* d_lights, uint32_t light_count, uint32_t cap,
                                             CfLightCell* d_cells, uint32_t* d_indices, uint64_t index_capacity,
                                             uint32_t* d_total, uint32_t* d_device_error, void* stream)
{
    using namespace cfrt;
    if (!ubo || !d_aabbs || !d_cells || !d_indices || (light_count && !d_lights))
        return fail(CF_ERROR_INVALID_ARGUMENT, "cf_cull_lights_static_scratch: null argument");
    if (light_count > kMaxLights) return fail(CF_ERROR_INVALID_ARGUMENT, "%u lights exceed %u", light_count, kMaxLights);
    uint32_t C = 0;
    int s = validate_grid(ubo->sliceCountX, ubo->sliceCountY, ubo->sliceCountZ, cap, &C);
    if (s) return s;
    if (index_capacity < (uint64_t)C * cap)
        return fail(CF_ERROR_CAPACITY, "index capacity %llu < clusters x cap = %llu", (unsigned long long)index_capacity,
                    (unsigned long long)C * cap);
    // the automatic kernel choice when its scratch fits, else the brute-force
    // kernels, which need less (both give the same result)
    cfk::CullConfig cfg = choose_config(*ubo, light_count, nullptr);
    cfk::WorkspaceLayout L = layout_for(*ubo, light_count, cap, cfg);
    if (L.bytes > kStaticScratchBytes && cfg.binned) {
        cfg = cfk::default_cull_config(C, light_count, 1);
        L = layout_for(*ubo, light_count, cap, cfg);
    }
    if (L.bytes > kStaticScratchBytes)
        return fail(CF_ERROR_CAPACITY,
                    "this view needs %llu bytes of scratch (%u clusters, %u lights, cap %u); the static scratch of "
                    "cf_cull_lights_static_scratch holds %llu bytes — use cf_cull_lights with a workspace instead",
                    (unsigned long long)L.bytes, C, light_count, cap, (unsigned long long)kStaticScratchBytes);
    unsigned char* ws = nullptr;
    s = scratch_address(&ws);
    if (s) return s;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    uint32_t* err_word = d_device_error;
    if (!err_word) {
        // no caller word: use the array's own status word, cleared so that an
        // earlier call's code does not linger
        err_word = reinterpret_cast<uint32_t*>(ws);
        cudaError_t e = cudaMemsetAsync(err_word, 0, sizeof(uint32_t), st);
        if (e != cudaSuccess) return cuda_fail(e, "clear the static scratch error word");
    }
    return enqueue_cull(*ubo, d_aabbs, d_lights, light_count, cap, d_cells, d_indices, d_total, ws, err_word, cfg, st,
                        nullptr);
}
