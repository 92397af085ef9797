// cf_kernels.cu — sm_103a kernels of the clustered-forward light-culling path.
//
//   aabb_kernel         HelloVulkan/Shaders/ClusteredForward/AABBGenerator.comp:39-89,
//   batch_aabb_kernel   one thread per cluster, float4 stores (one view / many)
//   light_xform_kernel  the `ubo.cameraView * posWorld` and `radius * radius` of
//   batch_xform_kernel  LightCulling.comp:51-56, hoisted to once per light
//   bin_slices_kernel   per depth slice, the lights whose sphere can reach the
//   batch_bin_kernel    slice's z slab, in light order (the candidate lists; a
//                       single view's in two segments, one CTA per half of the
//                       lights)
//   cull_kernel         LightCulling.comp:59-77 brute force: a producer warp
//                       streams tiles of view-space lights into shared memory
//                       with bulk async copies (cp.async.bulk + mbarrier); each
//                       consumer warp owns K clusters, its 32 lanes test 32
//                       consecutive lights, and __ballot_sync/__popc compact
//                       the hits in ascending light order up to the cap
//   cull_pipe_kernel    the same test over the slice candidate lists, persistent:
//                       CTAs take (view, cluster group) items from a queue, a
//                       producer warp runs one item ahead (descriptor, AABBs and
//                       tiles by bulk copy), the consumer warps filter each tile
//                       against the group's union box, compact the survivors and
//                       test them against their clusters
//   scan_kernel         LightCulling.comp:79-87 with the global atomicAdd replaced
//   copy_kernel         by an exclusive scan of the group totals in cluster order,
//   batch_*             then the packed copy of each cluster's hits
//   jitter_tasks_kernel the served light sets' device jitters, many sets per launch
//   upload_tasks_kernel the served light sets' copies from pinned host memory, many per launch
//   orbit_kernel        the animated workload's in-place light motion
//
// Floating point follows include/cf_pinned_math.h: every product and sum is an
// explicit round-to-nearest intrinsic, so nothing is contracted into an FMA.
#include "cf_kernels.cuh"
#include "cf_device.cuh"

#include <algorithm>
#include <atomic>
#include <utility>

#include "cf_pinned_math.h"

namespace cfk {
namespace {

// ---------------------------------------------------------------------------
// PTX helpers: mbarrier and bulk async copy.
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t smem_u32(const void* p)
{
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}


__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_init_fence()
{
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive(uint32_t bar)
{
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint32_t bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t parity)
{
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n}"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    return ok != 0;
}

// Waits for the phase of `parity` to complete; gives up after g_wait_limit_ns
// (kWaitLimitNs unless a test shortens it) or kWaitLimitIters polls and
// returns false.
__device__ __noinline__ bool mbar_wait_bounded(uint32_t bar, uint32_t parity)
{
    if (mbar_try_wait(bar, parity)) return true;
    const uint64_t t0 = global_timer_ns();
    for (uint32_t it = 0; it < kWaitLimitIters; ++it) {
        if (mbar_try_wait(bar, parity)) return true;
        if (global_timer_ns() - t0 > g_wait_limit_ns) break;
    }
    return false;
}

// As mbar_wait_bounded, but also gives up (returning false) once *abort is set.
__device__ __noinline__ bool mbar_wait_or_abort(uint32_t bar, uint32_t parity, const volatile uint32_t* abort)
{
    if (mbar_try_wait(bar, parity)) return true;
    const uint64_t t0 = global_timer_ns();
    for (uint32_t it = 0; it < kWaitLimitIters; ++it) {
        if (mbar_try_wait(bar, parity)) return true;
        if (*abort || global_timer_ns() - t0 > g_wait_limit_ns) break;
    }
    return false;
}

__device__ __forceinline__ void bulk_copy_g2s(uint32_t dst, const void* src, uint32_t bytes, uint32_t bar)
{
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
        "l"(src), "r"(bytes), "r"(bar)
        : "memory");
}

// Per-thread asynchronous 16-byte global-to-shared copies (cp.async): a thread
// waits only for its own copies, so no flag or barrier is involved.
__device__ __forceinline__ void cp_async16(uint32_t dst, const void* src)
{
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(dst), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory"); }


// Named barrier 1 over the first N threads of the CTA (the consumer warps;
// the producer warp never takes part).
template <int N>
__device__ __forceinline__ void consumer_sync()
{
    asm volatile("bar.sync 1, %0;" ::"n"(N) : "memory");
}


// ---------------------------------------------------------------------------
// AABB generator: AABBGenerator.comp:39-89, one thread per cluster.
// ---------------------------------------------------------------------------
struct ViewPoint {
    float x, y, z;
};

// ScreenToView (AABBGenerator.comp:18-32) for screen = (sx, sy, 0, 1); the
// shader divides all four lanes by w, of which only xyz are used.
__device__ __forceinline__ ViewPoint screen_to_view(const float* inv_proj, float sx, float sy)
{
    const float cx = cf_fsub(cf_fmul(sx, 2.0f), 1.0f);
    const float cy = cf_fsub(cf_fmul(sy, 2.0f), 1.0f);
    const float vx = cf_mat4_row(inv_proj, 0, cx, cy, 0.0f, 1.0f);
    const float vy = cf_mat4_row(inv_proj, 1, cx, cy, 0.0f, 1.0f);
    const float vz = cf_mat4_row(inv_proj, 2, cx, cy, 0.0f, 1.0f);
    const float vw = cf_mat4_row(inv_proj, 3, cx, cy, 0.0f, 1.0f);
    return {cf_fdiv(vx, vw), cf_fdiv(vy, vw), cf_fdiv(vz, vw)};
}

// RayIntersectZPlane (AABBGenerator.comp:34-37): (incident * zOffset) / incident.z
__device__ __forceinline__ ViewPoint ray_z(const ViewPoint& p, float z)
{
    return {cf_fdiv(cf_fmul(p.x, z), p.z), cf_fdiv(cf_fmul(p.y, z), p.z), cf_fdiv(cf_fmul(p.z, z), p.z)};
}

__device__ __forceinline__ void aabb_body(const CfClusterForwardUBO& ubo, float4* __restrict__ out, uint32_t c)
{
    const uint32_t X = ubo.sliceCountX, Y = ubo.sliceCountY, Z = ubo.sliceCountZ;
    const uint32_t i = c % X, j = (c / X) % Y, k = c / (X * Y);
    const float npx = cf_fdiv(1.0f, (float)X);
    const float npy = cf_fdiv(1.0f, (float)Y);
    const ViewPoint max_vs = screen_to_view(ubo.cameraInverseProjection, cf_fmul(cf_fadd((float)i, 1.0f), npx),
                                            cf_fmul(cf_fadd((float)j, 1.0f), npy));
    const ViewPoint min_vs = screen_to_view(ubo.cameraInverseProjection, cf_fmul((float)i, npx), cf_fmul((float)j, npy));
    const float ratio = cf_fdiv(ubo.cameraFar, ubo.cameraNear);
    const float neg_near = -ubo.cameraNear;
    const float tile_near = cf_fmul(neg_near, cf_pow_pinned(ratio, cf_fdiv((float)k, (float)Z)));
    const float tile_far = cf_fmul(neg_near, cf_pow_pinned(ratio, cf_fdiv((float)(k + 1u), (float)Z)));
    const ViewPoint a = ray_z(min_vs, tile_near), b = ray_z(min_vs, tile_far);
    const ViewPoint d = ray_z(max_vs, tile_near), e = ray_z(max_vs, tile_far);
    float4 lo, hi;
    lo.x = cf_glsl_min(cf_glsl_min(a.x, b.x), cf_glsl_min(d.x, e.x));
    lo.y = cf_glsl_min(cf_glsl_min(a.y, b.y), cf_glsl_min(d.y, e.y));
    lo.z = cf_glsl_min(cf_glsl_min(a.z, b.z), cf_glsl_min(d.z, e.z));
    lo.w = 0.0f;
    hi.x = cf_glsl_max(cf_glsl_max(a.x, b.x), cf_glsl_max(d.x, e.x));
    hi.y = cf_glsl_max(cf_glsl_max(a.y, b.y), cf_glsl_max(d.y, e.y));
    hi.z = cf_glsl_max(cf_glsl_max(a.z, b.z), cf_glsl_max(d.z, e.z));
    hi.w = 0.0f;
    out[2 * (size_t)c] = lo;
    out[2 * (size_t)c + 1] = hi;
}

__global__ void __launch_bounds__(256) aabb_kernel(const CfClusterForwardUBO ubo, float4* __restrict__ out,
                                                   uint32_t clusters)
{
    const uint32_t c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c < clusters) aabb_body(ubo, out, c);
}

// ---------------------------------------------------------------------------
// Light transform: posView = cameraView * position, r^2 = radius * radius.
// One 256-thread block per flag granule.
// ---------------------------------------------------------------------------
struct Mat4 {
    float m[16];
};

// Granule blk (256 lights) of one view; every thread of the block takes part.
__device__ __forceinline__ void light_xform_body(const CfLightData* __restrict__ lights, uint32_t count,
                                                 uint32_t lpad, const float* view, float4* __restrict__ out,
                                                 uint32_t* __restrict__ nonfinite, uint32_t blk)
{
    const uint32_t i = blk * kFlagGranule + threadIdx.x;
    bool bad = false;
    if (i < count) {
        const float4 p = __ldg(reinterpret_cast<const float4*>(&lights[i].position[0]));
        const float r = __ldg(&lights[i].radius);
        const float x = cf_mat4_row(view, 0, p.x, p.y, p.z, p.w);
        const float y = cf_mat4_row(view, 1, p.x, p.y, p.z, p.w);
        const float z = cf_mat4_row(view, 2, p.x, p.y, p.z, p.w);
        bad = !(finite_bits(x) && finite_bits(y) && finite_bits(z));
        out[i] = make_float4(x, y, z, cf_fmul(r, r));
    } else if (i < lpad) {
        out[i] = make_float4(0.0f, 0.0f, 0.0f, __uint_as_float(0xff800000u));  // never hits
    }
    const int any_bad = __syncthreads_or(bad);
    if (threadIdx.x == 0) nonfinite[blk] = any_bad ? 1u : 0u;
}

__global__ void __launch_bounds__(kFlagGranule) light_xform_kernel(const CfLightData* __restrict__ lights,
                                                                   uint32_t count, uint32_t lpad, const Mat4 view,
                                                                   float4* __restrict__ out,
                                                                   uint32_t* __restrict__ nonfinite)
{
    grid_dependency_wait();
    launch_dependents();
    light_xform_body(lights, count, lpad, view.m, out, nonfinite, blockIdx.x);
}

// Index of the view whose range [prefix[v], prefix[v+1]) holds block b.
__device__ __forceinline__ uint32_t find_view(const uint32_t* __restrict__ prefix, uint32_t n_views, uint32_t b)
{
    uint32_t lo = 0, hi = n_views;  // prefix[lo] <= b < prefix[hi]
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (__ldg(&prefix[mid]) <= b) lo = mid;
        else hi = mid;
    }
    return lo;
}

// Batched light transform: block b is granule b - prefix[v] of view v.  Block
// 0 also resets the culling work queue of the same batch.
__global__ void __launch_bounds__(kFlagGranule) batch_xform_kernel(const ViewJob* __restrict__ jobs,
                                                                   const uint32_t* __restrict__ prefix,
                                                                   uint32_t n_views, uint32_t* __restrict__ queues,
                                                                   uint32_t n_queues)
{
    if (blockIdx.x == 0 && threadIdx.x < n_queues) queues[threadIdx.x] = 0;
    const uint32_t vi = find_view(prefix, n_views, blockIdx.x);
    const ViewJob& j = jobs[vi];
    light_xform_body(j.lights, j.light_count, j.v.lpad, j.view, const_cast<float4*>(j.v.vlights),
                     const_cast<uint32_t*>(j.v.nonfinite), blockIdx.x - __ldg(&prefix[vi]));
}

// Batched AABB generator: block b holds clusters [256 (b - prefix[v]), +256)
// of view v.
__global__ void __launch_bounds__(256) batch_aabb_kernel(const AabbJob* __restrict__ jobs,
                                                         const uint32_t* __restrict__ prefix, uint32_t n_views)
{
    const uint32_t vi = find_view(prefix, n_views, blockIdx.x);
    const AabbJob& j = jobs[vi];
    const uint32_t c = (blockIdx.x - __ldg(&prefix[vi])) * 256 + threadIdx.x;
    if (c < j.ubo.sliceCountX * j.ubo.sliceCountY * j.ubo.sliceCountZ)
        aabb_body(j.ubo, reinterpret_cast<float4*>(j.out), c);
}

// ---------------------------------------------------------------------------
// Culling (the sphere-box tests hit_fast / hit_exact are in cf_device.cuh).
// ---------------------------------------------------------------------------

template <int K>
struct WarpClusters {
    float mn[K][3];
    float mx[K][3];
    uint32_t cnt[K];
};

// Tests the lights of one shared-memory tile (lights base .. base + n - 1)
// against the warp's K clusters of the brute-force kernel; returns true once
// every cluster of the warp has reached the cap.
//   kExact   the shader's branchy test (tiles holding non-finite coordinates)
template <int K, bool kExact>
__device__ __forceinline__ bool scan_tile(const float4* __restrict__ tile, uint32_t n, uint32_t base, uint32_t lane,
                                          WarpClusters<K>& w, uint32_t cap, uint32_t* __restrict__ staging,
                                          uint32_t cl0, uint32_t cl_end, uint32_t& chunks_tested)
{
    const uint32_t lt_mask = (1u << lane) - 1u;
    for (uint32_t j = 0; j < n; j += 32) {
        const float4 L = tile[j + lane];
        ++chunks_tested;
        bool h[K];
        bool any = false;
#pragma unroll
        for (int k = 0; k < K; ++k) {
            h[k] = kExact ? hit_exact(L, w.mn[k], w.mx[k]) : hit_fast(L, w.mn[k], w.mx[k]);
            any |= h[k];
        }
        if (__any_sync(kFull, any)) {
            const uint32_t li = base + j + lane;
            bool all_capped = true;
#pragma unroll
            for (int k = 0; k < K; ++k) {
                const uint32_t m = __ballot_sync(kFull, h[k]);
                if (m) {
                    const uint32_t pos = w.cnt[k] + __popc(m & lt_mask);
                    if (h[k] && pos < cap) staging[(size_t)(cl0 + k) * cap + pos] = li;
                    w.cnt[k] += __popc(m);
                    if (w.cnt[k] >= cap) {
                        w.cnt[k] = cap;
                        const float inf = __uint_as_float(0x7f800000u);
#pragma unroll
                        for (int a = 0; a < 3; ++a) {
                            w.mn[k][a] = inf;
                            w.mx[k][a] = inf;
                        }
                    }
                }
                all_capped = all_capped && (w.cnt[k] >= cap || cl0 + k >= cl_end);
            }
            if (all_capped) return true;
        }
    }
    return false;
}

// Binned: the warp's K cluster boxes stay in the item's shared-memory AABB
// slot (wb: lo, hi per cluster; warp-uniform, read by broadcast) instead of
// K x 6 registers per lane; only the counts and the warp's union box are
// registers.  A capped cluster's box is set to +inf in the slot, so it never
// hits again.  Otherwise as scan_tile with kBinned.
template <int K>
struct WarpCounts {
    uint32_t cnt[K];
    float umn[3], umx[3];
};

template <int K, bool kExact>
__device__ __forceinline__ bool scan_tile_slot(const float4* __restrict__ tile, const uint32_t* __restrict__ idx_tile,
                                               uint32_t n, uint32_t lane, WarpCounts<K>& w, float4* wb,
                                               uint32_t cap, uint32_t* __restrict__ staging, uint32_t cl0,
                                               uint32_t cl_end, uint32_t& chunks_filtered, uint32_t& chunks_tested)
{
    const uint32_t lt_mask = (1u << lane) - 1u;
    const float inf = __uint_as_float(0x7f800000u);
    for (uint32_t j = 0; j < n; j += 32) {
        const float4 L = tile[j + lane];
        ++chunks_filtered;
        if (!__any_sync(kFull, hit_fast(L, w.umn, w.umx))) continue;
        ++chunks_tested;
        bool h[K];
        bool any = false;
#pragma unroll
        for (int k = 0; k < K; ++k) {
            const float4 lo = wb[2 * k], hi = wb[2 * k + 1];
            const float mn[3] = {lo.x, lo.y, lo.z}, mx[3] = {hi.x, hi.y, hi.z};
            h[k] = kExact ? hit_exact(L, mn, mx) : hit_fast(L, mn, mx);
            any |= h[k];
        }
        if (__any_sync(kFull, any)) {
            const uint32_t li = idx_tile[j + lane];
            bool all_capped = true;
#pragma unroll
            for (int k = 0; k < K; ++k) {
                const uint32_t m = __ballot_sync(kFull, h[k]);
                if (m) {
                    const uint32_t pos = w.cnt[k] + __popc(m & lt_mask);
                    if (h[k] && pos < cap) staging[(size_t)(cl0 + k) * cap + pos] = li;
                    w.cnt[k] += __popc(m);
                    if (w.cnt[k] >= cap) {
                        w.cnt[k] = cap;
                        if (lane == 0) {
                            wb[2 * k] = make_float4(inf, inf, inf, 0.f);
                            wb[2 * k + 1] = make_float4(inf, inf, inf, 0.f);
                        }
                        __syncwarp();
                    }
                }
                all_capped = all_capped && (w.cnt[k] >= cap || cl0 + k >= cl_end);
            }
            if (all_capped) return true;
        }
    }
    return false;
}

__device__ __forceinline__ bool tile_has_nonfinite(const uint32_t* __restrict__ flags, uint32_t base, uint32_t n)
{
    uint32_t f = 0;
    for (uint32_t g = base / kFlagGranule; g <= (base + n - 1) / kFlagGranule; ++g) f |= flags[g];
    return f != 0;
}

// Shared-memory carve-up of the brute-force culling kernel (dynamic shared
// memory): STAGES x TILE float4 tiles, the full/empty mbarriers, per-stage
// stop flags and the done-warp counter.
template <int K, int WARPS, int TILE, int STAGES>
struct CullSmem {
    float4* tiles;
    uint64_t* full;
    uint64_t* empty;
    volatile uint32_t* stop;
    uint32_t* done_warps;

    static constexpr size_t bytes()
    {
        return (size_t)STAGES * TILE * sizeof(float4) + 2 * STAGES * sizeof(uint64_t) + (STAGES + 1) * sizeof(uint32_t);
    }
    __device__ explicit CullSmem(unsigned char* smem)
    {
        tiles = reinterpret_cast<float4*>(smem);
        full = reinterpret_cast<uint64_t*>(smem + (size_t)STAGES * TILE * sizeof(float4));
        empty = full + STAGES;
        stop = reinterpret_cast<volatile uint32_t*>(empty + STAGES);
        done_warps = reinterpret_cast<uint32_t*>(empty + STAGES) + STAGES;
    }
    __device__ void init()
    {
        if (threadIdx.x == 0) {
            for (int s = 0; s < STAGES; ++s) {
                mbar_init(smem_u32(&full[s]), 1);
                mbar_init(smem_u32(&empty[s]), WARPS);
                stop[s] = 0;
            }
            *done_warps = 0;
            mbar_init_fence();
        }
    }
};

// Brute force, one view: CTA b owns cluster group b = clusters
// [b*W*K, (b+1)*W*K).  The producer warp streams every light of the view in
// tiles through the stages; each consumer warp tests its K clusters, 32
// lights at a time.  Every tile used (including one that only carries the
// stop signal, sent once every consumer warp is capped) completes one full
// phase and one empty phase.  A timed-out wait sets the error word and ends
// the group; the producer then lets its copies in flight land before it exits.
template <int K, int WARPS, int TILE, int STAGES>
__global__ void __launch_bounds__((WARPS + 1) * 32) cull_kernel(const ViewCull v, uint32_t* __restrict__ dev_error)
{
    static_assert(TILE % 32 == 0, "tiles hold whole warps of lights");
    extern __shared__ __align__(128) unsigned char smem[];
    CullSmem<K, WARPS, TILE, STAGES> sm(smem);
    sm.init();
    __syncthreads();
    grid_dependency_wait();
    launch_dependents();
    const uint32_t group = blockIdx.x;
    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t nsrc = v.lpad, first = group * (uint32_t)(WARPS * K), cl_end = v.clusters;
    const uint32_t ntiles = (nsrc + TILE - 1) / TILE;
    float4* const tiles = sm.tiles;
    uint64_t* const full = sm.full;
    uint64_t* const empty = sm.empty;
    volatile uint32_t* const stop = sm.stop;
    uint32_t* const done_warps = sm.done_warps;

    if (warp == WARPS) {
        if (lane != 0) return;
        uint32_t t = 0;
        bool stalled = false;
        // a test may make CTA 0 never send tile 0 (its consumers' waits run out)
        const bool skip_first = group == 0 && (g_inject_stall & kInjectBruteForceSkipTile);
        for (; t < ntiles; ++t) {
            const uint32_t s = t % STAGES;
            if (t >= STAGES && !mbar_wait_bounded(smem_u32(&empty[s]), ((t / STAGES) & 1u) ^ 1u)) {
                atomicOr(dev_error, kErrEmptyWaitTimeout);
                stalled = true;
                break;
            }
            if (*reinterpret_cast<volatile uint32_t*>(done_warps) >= (uint32_t)WARPS) {
                stop[s] = 1;  // every consumer is capped: release them without data
                mbar_arrive(smem_u32(&full[s]));
                ++t;
                break;
            }
            stop[s] = 0;
            if (skip_first && t == 0) continue;  // no arrival and no copy for this tile
            const uint32_t n = min((uint32_t)TILE, nsrc - t * TILE);
            mbar_arrive_expect_tx(smem_u32(&full[s]), n * (uint32_t)sizeof(float4));
            bulk_copy_g2s(smem_u32(tiles + (size_t)s * TILE), v.vlights + (size_t)t * TILE,
                          n * (uint32_t)sizeof(float4), smem_u32(&full[s]));
        }
        // After a stall, or with a tile withheld (the consumers may then leave
        // before the copies land), wait for the copies in flight before the
        // CTA can exit: the last tile of each stage completes last.  The
        // withheld tile's wait runs out after the bounded time.
        if (stalled || skip_first)
            for (uint32_t q = 0; q < STAGES && q < t; ++q) {
                const uint32_t g = t - 1 - q;
                mbar_wait_bounded(smem_u32(&full[g % STAGES]), (g / STAGES) & 1u);
            }
        return;
    }

    // Consumers.
    const uint32_t cl0 = first + warp * (uint32_t)K;
    const float inf = __uint_as_float(0x7f800000u);
    WarpClusters<K> w;
    bool done = true;
#pragma unroll
    for (int k = 0; k < K; ++k) {
        const uint32_t c = cl0 + k;
        // A cluster past the view starts full, so nothing is ever written for
        // it: its +inf box still reaches a light with a NaN coordinate (the
        // squared distance counts a NaN axis as 0).
        w.cnt[k] = c < cl_end ? 0u : v.cap;
        if (c < cl_end) {
            const float4 a = v.aabbs[2 * (size_t)c];
            const float4 b = v.aabbs[2 * (size_t)c + 1];
            w.mn[k][0] = a.x; w.mn[k][1] = a.y; w.mn[k][2] = a.z;
            w.mx[k][0] = b.x; w.mx[k][1] = b.y; w.mx[k][2] = b.z;
            done = false;
        } else {
            for (int q = 0; q < 3; ++q) { w.mn[k][q] = inf; w.mx[k][q] = inf; }
        }
    }
    if (done && lane == 0) atomicAdd(done_warps, 1u);

    uint32_t chunks_tested = 0;
    for (uint32_t t = 0; t < ntiles; ++t) {
        const uint32_t s = t % STAGES;
        if (!mbar_wait_bounded(smem_u32(&full[s]), (t / STAGES) & 1u)) {
            if (lane == 0) atomicOr(dev_error, kErrFullWaitTimeout);
            break;
        }
        if (stop[s]) {
            __syncwarp();
            if (lane == 0) mbar_arrive(smem_u32(&empty[s]));
            break;
        }
        if (!done) {
            const uint32_t base = t * TILE;
            const uint32_t n = min((uint32_t)TILE, nsrc - base);
            const float4* tile = tiles + (size_t)s * TILE;
            if (!tile_has_nonfinite(v.nonfinite, base, n))
                done = scan_tile<K, false>(tile, n, base, lane, w, v.cap, v.staging, cl0, cl_end, chunks_tested);
            else
                done = scan_tile<K, true>(tile, n, base, lane, w, v.cap, v.staging, cl0, cl_end, chunks_tested);
            if (done && lane == 0) atomicAdd(done_warps, 1u);
        }
        __syncwarp();
        if (lane == 0) mbar_arrive(smem_u32(&empty[s]));
    }

    __shared__ uint32_t s_gsum[WARPS];
    if (lane == 0) {
        uint32_t sum = 0;
#pragma unroll
        for (int k = 0; k < K; ++k)
            if (cl0 + k < cl_end) {
                v.counts[cl0 + k] = w.cnt[k];
                sum += w.cnt[k];
            }
        s_gsum[warp] = sum;
        if (v.work) atomicAdd(&v.work[1], 32ull * K * chunks_tested);  // no filter tests without binning
    }
    consumer_sync<WARPS * 32>();
    if (threadIdx.x == 0) {
        uint32_t sum = 0;
        for (int q = 0; q < WARPS; ++q) sum += s_gsum[q];
        v.group_sums[group] = sum;
    }
}

// Many views in one persistent launch (binned culling).  Each CTA takes
// (view, group) items from `items` in queue order (an atomic counter the
// light-transform launch resets) until none are left; items are ordered by
// decreasing expected work.  The producer warp runs ahead of the consumers:
// while they cull item n it already fetches item n + 1, writes its descriptor
// into a ring of kItemSlots shared-memory slots, loads the group's AABBs into
// the slot and starts streaming the item's candidate tiles through the stage
// ring.  So the latency of the item's global reads and first copies is hidden
// behind the previous item.  Stage tiles are numbered across items (the
// descriptor carries the item's first tile number), which fixes each tile's
// stage and mbarrier phases.
constexpr uint32_t kItemSlots = 2;

struct ItemDesc {
    uint32_t* staging;
    uint32_t* counts;
    uint32_t* group_sums;
    unsigned long long* work;
    uint32_t first, cl_end, nsrc, ntiles;
    uint32_t seq, group, cap, flags;  // flags: kItemTerminate | kItemExact
};
static_assert(sizeof(ItemDesc) % 16 == 0, "descriptor slots stay 16-byte aligned");
constexpr uint32_t kItemTerminate = 1u, kItemExact = 2u;

// Dynamic shared memory of cull_pipe_kernel: stage tiles and their light
// indices, kItemSlots groups of AABBs and their union boxes, the survivor
// buffer, kItemSlots descriptors, the mbarriers, then small words.
template <int K, int WARPS, int TILE, int STAGES>
struct PipeSmem {
    static constexpr uint32_t kGroup = (uint32_t)(K * WARPS);
    static constexpr size_t tiles = 0;
    static constexpr size_t idx = tiles + (size_t)STAGES * TILE * sizeof(float4);
    static constexpr size_t boxes = idx + (size_t)STAGES * TILE * sizeof(uint32_t);
    static constexpr size_t ubox = boxes + (size_t)kItemSlots * kGroup * sizeof(CfAABB);  // the group's union, per slot
    static constexpr size_t surv_l = ubox + (size_t)kItemSlots * sizeof(CfAABB);
    static constexpr size_t surv_i = surv_l + (size_t)TILE * sizeof(float4);
    static constexpr size_t desc = surv_i + (size_t)TILE * sizeof(uint32_t);
    static constexpr size_t bars = desc + kItemSlots * sizeof(ItemDesc);
    static constexpr size_t small = bars + (2 * STAGES + 2 * kItemSlots) * sizeof(uint64_t);
    // stop[STAGES], done[kItemSlots], chunk counts[TILE / 32], warp sums[WARPS], the consumers' abort
    // flag, the producer's abort flag
    static constexpr size_t bytes = small + (STAGES + kItemSlots + TILE / 32 + WARPS + 2) * 4;
    static_assert(boxes % 16 == 0 && ubox % 16 == 0 && desc % 16 == 0 && bars % 8 == 0, "shared-memory alignment");
};

template <int K, int WARPS, int TILE, int STAGES>
__global__ void __launch_bounds__((WARPS + 1) * 32, WARPS == 4 ? 5 : 3)
    cull_pipe_kernel(const ViewJob* __restrict__ jobs, const uint2* __restrict__ items, uint32_t n_items,
                     uint32_t* __restrict__ queue, uint32_t* __restrict__ dev_error, const ViewCull single)
{
    // jobs == nullptr: one view (`single`), item i is its group i
    static_assert(TILE % 32 == 0 && TILE / 32 <= 32, "tiles hold whole warps of lights, at most 32 chunks");
    using Lay = PipeSmem<K, WARPS, TILE, STAGES>;
    constexpr uint32_t kGroup = Lay::kGroup;
    extern __shared__ __align__(128) unsigned char smem[];
    float4* const tiles = reinterpret_cast<float4*>(smem + Lay::tiles);
    uint32_t* const idx_tiles = reinterpret_cast<uint32_t*>(smem + Lay::idx);
    float4* const boxes = reinterpret_cast<float4*>(smem + Lay::boxes);
    const float4* const uboxes = reinterpret_cast<const float4*>(smem + Lay::ubox);
    float4* const surv_l = reinterpret_cast<float4*>(smem + Lay::surv_l);
    uint32_t* const surv_i = reinterpret_cast<uint32_t*>(smem + Lay::surv_i);
    ItemDesc* const desc = reinterpret_cast<ItemDesc*>(smem + Lay::desc);
    uint64_t* const full = reinterpret_cast<uint64_t*>(smem + Lay::bars);
    uint64_t* const empty = full + STAGES;
    uint64_t* const ifull = empty + STAGES;
    uint64_t* const iempty = ifull + kItemSlots;
    volatile uint32_t* const stop = reinterpret_cast<volatile uint32_t*>(smem + Lay::small);
    uint32_t* const done = const_cast<uint32_t*>(stop) + STAGES;  // per slot: consumer warps all capped
    uint32_t* const s_cnt = done + kItemSlots;
    uint32_t* const s_gsum = s_cnt + TILE / 32;
    // s_abort is written only by consumer threads, before a consumer barrier,
    // so every consumer warp reads the same value after it; the producer
    // keeps its own flag and the consumers learn of its failure through their
    // own bounded waits.
    volatile uint32_t* const s_abort = s_gsum + WARPS;
    volatile uint32_t* const p_abort = s_gsum + WARPS + 1;

    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (threadIdx.x == 0) {
        for (int s = 0; s < STAGES; ++s) {
            mbar_init(smem_u32(&full[s]), 1);
            mbar_init(smem_u32(&empty[s]), WARPS);
            stop[s] = 0;
        }
        for (uint32_t r = 0; r < kItemSlots; ++r) {
            mbar_init(smem_u32(&ifull[r]), 1);
            mbar_init(smem_u32(&iempty[r]), WARPS);
            done[r] = 0;
        }
        *s_abort = 0;
        *p_abort = 0;
        mbar_init_fence();
    }
    __syncthreads();
    grid_dependency_wait();  // a single view's launch may overlap the binning launch's tail (no-op in a batch)
    launch_dependents();

    if (warp == WARPS) {
        // Producer: lane 0 fetches items, fills descriptors, loads AABBs and
        // streams candidate tiles; it never waits for the consumers to finish
        // an item, only for a free descriptor slot and free stages.
        if (lane != 0) return;
        uint32_t seq = 0;        // tiles issued so far
        uint32_t filled = 0;     // items whose descriptor and boxes were issued
        for (uint32_t n = 0;; ++n) {
            const uint32_t r = n % kItemSlots;
            if (n >= kItemSlots &&
                !mbar_wait_or_abort(smem_u32(&iempty[r]), ((n / kItemSlots) & 1u) ^ 1u, s_abort)) {
                if (!*s_abort) atomicOr(dev_error, kErrEmptyWaitTimeout);
                *p_abort = 1;
                break;
            }
            ItemDesc& d = desc[r];
            // each CTA's first item is its own index, the rest come from the
            // counter (one atomic round trip less before the first item)
            const uint32_t it = *s_abort ? n_items : n == 0 ? blockIdx.x : gridDim.x + atomicAdd(queue, 1u);
            if (it >= n_items) {
                d.flags = kItemTerminate;
                mbar_arrive(smem_u32(&ifull[r]));
                break;
            }
            const uint2 item = jobs ? items[it] : make_uint2(0u, it);
            const ViewCull& v = jobs ? jobs[item.x].v : single;
            const uint32_t xy = v.slice_clusters, gps = (xy + kGroup - 1) / kGroup;
            const uint32_t k = item.y / gps, g = item.y % gps;
            const uint32_t first = k * xy + g * kGroup, cl_end = (k + 1) * xy;
            const uint32_t nb = min(kGroup, cl_end - first);
            const uint32_t n0 = v.slice_count[2 * k], nsrc = n0 + v.slice_count[2 * k + 1];
            const uint32_t seg1 = list_split(v.lpad);  // where the list's second segment starts
            const uint32_t ntiles = (nsrc + TILE - 1) / TILE;
            d.staging = v.staging;
            d.counts = v.counts;
            d.group_sums = v.group_sums;
            d.work = v.work;
            d.first = first;
            d.cl_end = cl_end;
            d.nsrc = nsrc;
            d.ntiles = ntiles;
            d.seq = seq;
            d.group = item.y;
            d.cap = v.cap;
            d.flags = (v.slice_nonfinite[2 * k] | v.slice_nonfinite[2 * k + 1]) ? kItemExact : 0u;
            done[r] = 0;
            mbar_arrive_expect_tx(smem_u32(&ifull[r]), (nb + 1) * (uint32_t)sizeof(CfAABB));
            bulk_copy_g2s(smem_u32(boxes + (size_t)r * kGroup * 2), v.aabbs + 2 * (size_t)first,
                          nb * (uint32_t)sizeof(CfAABB), smem_u32(&ifull[r]));
            bulk_copy_g2s(smem_u32(uboxes + (size_t)r * 2), v.group_boxes + 2 * (size_t)item.y,
                          (uint32_t)sizeof(CfAABB), smem_u32(&ifull[r]));
            filled = n + 1;
            const float4* src = v.slice_lights + (size_t)k * v.lpad;
            const uint32_t* src_idx = v.slice_idx + (size_t)k * v.lpad;
            uint32_t t = 0;
            bool stalled = false;
            for (; t < ntiles; ++t) {
                const uint32_t gt = seq + t, s = gt % STAGES;
                if (gt >= STAGES &&
                    !mbar_wait_or_abort(smem_u32(&empty[s]), ((gt / STAGES) & 1u) ^ 1u, s_abort)) {
                    if (!*s_abort) atomicOr(dev_error, kErrEmptyWaitTimeout);
                    *p_abort = 1;
                    stalled = true;
                    break;
                }
                if (*reinterpret_cast<volatile uint32_t*>(&done[r]) >= (uint32_t)WARPS) {
                    stop[s] = 1;  // every consumer warp is capped: release them without data
                    mbar_arrive(smem_u32(&full[s]));
                    ++t;
                    break;
                }
                stop[s] = 0;
                // list entries [pos, pos + cnt): a from the first segment, b from the second
                const uint32_t pos = t * TILE, cnt = min((uint32_t)TILE, nsrc - pos);
                const uint32_t a = pos < n0 ? min(cnt, n0 - pos) : 0u, b = cnt - a;
                const uint32_t from1 = seg1 + (b ? pos + a - n0 : 0u);  // first second-segment entry
                mbar_arrive_expect_tx(smem_u32(&full[s]), cnt * (uint32_t)(sizeof(float4) + sizeof(uint32_t)));
                if (a) {
                    bulk_copy_g2s(smem_u32(tiles + (size_t)s * TILE), src + pos, a * (uint32_t)sizeof(float4),
                                  smem_u32(&full[s]));
                    bulk_copy_g2s(smem_u32(idx_tiles + (size_t)s * TILE), src_idx + pos,
                                  a * (uint32_t)sizeof(uint32_t), smem_u32(&full[s]));
                }
                if (b) {
                    bulk_copy_g2s(smem_u32(tiles + (size_t)s * TILE + a), src + from1, b * (uint32_t)sizeof(float4),
                                  smem_u32(&full[s]));
                    bulk_copy_g2s(smem_u32(idx_tiles + (size_t)s * TILE + a), src_idx + from1,
                                  b * (uint32_t)sizeof(uint32_t), smem_u32(&full[s]));
                }
            }
            seq += t;
            if (stalled) break;
        }
        if (*p_abort || *s_abort) {
            // Let every copy this CTA issued land before it exits: the last
            // tile of each stage and the last item's boxes complete last.
            for (uint32_t q = 0; q < STAGES && q < seq; ++q) {
                const uint32_t g = seq - 1 - q;
                mbar_wait_bounded(smem_u32(&full[g % STAGES]), (g / STAGES) & 1u);
            }
            if (filled) mbar_wait_bounded(smem_u32(&ifull[(filled - 1) % kItemSlots]), ((filled - 1) / kItemSlots) & 1u);
        }
        return;
    }

    // Consumers.
    constexpr uint32_t kChunks = TILE / 32;
    constexpr int kPer = (int)((kChunks + WARPS - 1) / WARPS);
    const float inf = __uint_as_float(0x7f800000u);
    const uint32_t lt_mask = (1u << lane) - 1u;
    for (uint32_t n = 0;; ++n) {
        const uint32_t r = n % kItemSlots;
        if (!mbar_wait_bounded(smem_u32(&ifull[r]), (n / kItemSlots) & 1u) && lane == 0) {
            atomicOr(dev_error, kErrFullWaitTimeout);
            *s_abort = 1;
        }
        consumer_sync<WARPS * 32>();  // every warp leaves together on a timeout
        if (*s_abort) break;
        const ItemDesc& d = desc[r];  // read in place: the slot is not refilled before this item's release
        if (d.flags & kItemTerminate) break;
        const uint32_t cl0 = d.first + warp * (uint32_t)K;
        float4* const gb = boxes + (size_t)r * kGroup * 2 + (size_t)warp * K * 2;  // this warp's boxes
        WarpCounts<K> w;
        bool wdone = true, union_nan = false;
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            w.umn[a] = inf;
            w.umx[a] = -inf;
        }
#pragma unroll
        for (int k = 0; k < K; ++k) {
            // a cluster past the item (the slice's short last group) starts
            // full, so nothing is written for it: its +inf box below still
            // reaches a light with a NaN coordinate
            w.cnt[k] = cl0 + k < d.cl_end ? 0u : d.cap;
            if (cl0 + k < d.cl_end) {
                const float4 lo = gb[2 * k], hi = gb[2 * k + 1];
                const float mn[3] = {lo.x, lo.y, lo.z}, mx[3] = {hi.x, hi.y, hi.z};
#pragma unroll
                for (int q = 0; q < 3; ++q) {
                    union_nan |= (mn[q] != mn[q]) | (mx[q] != mx[q]);
                    w.umn[q] = fminf(w.umn[q], mn[q]);
                    w.umx[q] = fmaxf(w.umx[q], mx[q]);
                }
                wdone = false;
            }
        }
        __syncwarp();  // every lane has read the slot before lane 0 marks the absent clusters
        if (lane == 0) {
#pragma unroll
            for (int k = 0; k < K; ++k)
                if (cl0 + k >= d.cl_end) {  // past the item: a box no finite light reaches
                    gb[2 * k] = make_float4(inf, inf, inf, 0.f);
                    gb[2 * k + 1] = make_float4(inf, inf, inf, 0.f);
                }
        }
        __syncwarp();
        if (union_nan) {
#pragma unroll
            for (int a = 0; a < 3; ++a) {
                w.umn[a] = -inf;
                w.umx[a] = inf;
            }
        }
        if (lane == 0 && wdone) atomicAdd(&done[r], 1u);
        const bool exact = (d.flags & kItemExact) != 0;
        uint32_t chunks_filtered = 0, chunks_tested = 0;
        for (uint32_t t = 0; t < d.ntiles; ++t) {
            const uint32_t g = d.seq + t, s = g % STAGES;
            if (!mbar_wait_bounded(smem_u32(&full[s]), (g / STAGES) & 1u) && lane == 0) {
                atomicOr(dev_error, kErrFullWaitTimeout);
                *s_abort = 1;
            }
            consumer_sync<WARPS * 32>();
            if (*s_abort) break;
            if (stop[s]) {
                __syncwarp();
                if (lane == 0) mbar_arrive(smem_u32(&empty[s]));
                break;
            }
            const uint32_t cnt = min((uint32_t)TILE, d.nsrc - t * TILE);
            const float4* tile = tiles + (size_t)s * TILE;
            const uint32_t* itile = idx_tiles + (size_t)s * TILE;
            // the group's union box (binning launch; infinite when a bound is NaN), read per tile so that
            // it is not held in registers across the loop
            const float4 ulo = uboxes[2 * r], uhi = uboxes[2 * r + 1];
            const float cmn[3] = {ulo.x, ulo.y, ulo.z}, cmx[3] = {uhi.x, uhi.y, uhi.z};
            float4 Ls[kPer];
            uint32_t Is[kPer], Ms[kPer];
#pragma unroll
            for (int q = 0; q < kPer; ++q) {
                const uint32_t ch = warp + q * WARPS;
                bool pass = false;
                if (ch < kChunks && ch * 32 < cnt) {
                    Ls[q] = tile[ch * 32 + lane];
                    Is[q] = itile[ch * 32 + lane];
                    pass = hit_fast(Ls[q], cmn, cmx);
                    ++chunks_filtered;
                }
                Ms[q] = __ballot_sync(kFull, pass);
                if (ch < kChunks && lane == 0) s_cnt[ch] = __popc(Ms[q]);
            }
            __syncwarp();
            if (lane == 0) mbar_arrive(smem_u32(&empty[s]));  // the stage is no longer read
            consumer_sync<WARPS * 32>();
            const uint32_t c = lane < kChunks ? s_cnt[lane] : 0u;
            const uint32_t incl = warp_inclusive_scan(c, lane);
            const uint32_t ns = __shfl_sync(kFull, incl, 31);
#pragma unroll
            for (int q = 0; q < kPer; ++q) {
                const uint32_t ch = warp + q * WARPS;
                const uint32_t excl = __shfl_sync(kFull, incl - c, ch & 31);
                if (ch < kChunks && ((Ms[q] >> lane) & 1u)) {
                    const uint32_t p = excl + __popc(Ms[q] & lt_mask);
                    surv_l[p] = Ls[q];
                    surv_i[p] = Is[q];
                }
            }
            const uint32_t nsp = (ns + 31) & ~31u;
            if (warp == 0 && ns + lane < nsp) surv_l[ns + lane] = make_float4(0.f, 0.f, 0.f, -inf);
            consumer_sync<WARPS * 32>();
            if (!wdone && ns) {
                wdone = exact ? scan_tile_slot<K, true>(surv_l, surv_i, nsp, lane, w, gb, d.cap, d.staging, cl0,
                                                        d.cl_end, chunks_filtered, chunks_tested)
                              : scan_tile_slot<K, false>(surv_l, surv_i, nsp, lane, w, gb, d.cap, d.staging, cl0,
                                                         d.cl_end, chunks_filtered, chunks_tested);
                if (wdone && lane == 0) atomicAdd(&done[r], 1u);
            }
            consumer_sync<WARPS * 32>();  // the survivor buffer is rewritten by the next tile
        }
        if (*s_abort) break;
        if (lane == 0) {
            uint32_t sum = 0;
#pragma unroll
            for (int k = 0; k < K; ++k)
                if (cl0 + k < d.cl_end) {
                    d.counts[cl0 + k] = w.cnt[k];
                    sum += w.cnt[k];
                }
            s_gsum[warp] = sum;
            if (d.work) {
                atomicAdd(&d.work[0], 32ull * chunks_filtered);
                atomicAdd(&d.work[1], 32ull * K * chunks_tested);
            }
        }
        consumer_sync<WARPS * 32>();
        if (threadIdx.x == 0) {
            uint32_t sum = 0;
            for (int q = 0; q < WARPS; ++q) sum += s_gsum[q];
            d.group_sums[d.group] = sum;
        }
        __syncwarp();
        if (lane == 0) mbar_arrive(smem_u32(&iempty[r]));  // slot r (descriptor, boxes, done count) is free
    }
}

// ---------------------------------------------------------------------------
// Slice binning: for depth slice k, the lights whose sphere can reach the
// slab between the slice's lowest AABB min.z and highest AABB max.z, in
// ascending light order, padded with never-hit entries to a multiple of 32.
// A light left out fails every cluster of the slice: its z distance to the
// slab is never larger than to a cluster's box, and the shader's sum of
// squares is never smaller than its z term.  NaN bounds make the slab
// infinite; a NaN coordinate contributes 0 and is kept; slices holding a
// light with a non-finite coordinate are flagged for the exact test.
// One CTA of WARPS warps bins one segment of SLICES consecutive slices: every
// light it reads is tested against each of their slabs, so the view-space
// lights are read once per SLICES slices (a batch bins 4 slices per
// 512-thread CTA into their lists' first segments; a single view, which has
// few slices, one slice per 1024-thread CTA and two CTAs per slice, one per
// segment, so that it keeps twice as many SMs busy).  Each step bins
// WARPS x 128 lights (4 chunks of 32 per warp) with ballot/popc and, per
// slice, a warp scan of the warps' counts.  Every thread stages its own four
// lights of the next step in shared memory with cp.async while it bins the
// current step (two slots per thread), so the step's global-load latency is
// hidden behind the previous step's work.
// ---------------------------------------------------------------------------
constexpr int kBinChunks = 4;
constexpr int kBinWarpsSingle = 32, kBinSlicesSingle = 1;
constexpr int kBinWarpsBatch = 16, kBinSlicesBatch = 4;

// dynamic shared memory of a binning CTA: two slots of kBinChunks lights per thread
constexpr size_t bin_stage_bytes(int warps) { return 2ull * kBinChunks * (size_t)warps * 32 * sizeof(float4); }

template <int kBinWarps, int kBinSlicesT, int kParts>
__device__ __forceinline__ void bin_slices_body(const ViewCull& v, uint32_t blk)
{
    static_assert(kParts == 1 || kParts == 2, "a list has two segments");
    constexpr uint32_t kBinSlices = (uint32_t)kBinSlicesT;
    __shared__ float s_lo[kBinSlices][kBinWarps], s_hi[kBinSlices][kBinWarps];
    __shared__ uint32_t s_cnt[kBinSlices][kBinWarps];
    __shared__ uint32_t s_nan, s_nonfinite;
    extern __shared__ __align__(16) float4 bin_stage[];  // [2 slots][kBinChunks][threads]
    constexpr uint32_t kThreads = kBinWarps * 32;
    constexpr uint32_t kStep = kBinWarps * kBinChunks * 32;
    const uint32_t tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const uint32_t h = kParts == 2 ? (blk & 1u) : 0u;  // the list segment this CTA writes
    const uint32_t xy = v.slice_clusters, k0 = (kParts == 2 ? blk >> 1 : blk) * kBinSlices;
    const uint32_t ns = min(kBinSlices, v.slices - k0);
    const uint32_t seg_lo = h ? list_split(v.lpad) : 0u;                       // lights [seg_lo, seg_hi)
    const uint32_t seg_hi = kParts == 2 && h == 0 ? list_split(v.lpad) : v.lpad;
    const float inf = __uint_as_float(0x7f800000u);
    // this thread's lights of the step at `base` into slot `slot`
    auto stage = [&](uint32_t base, uint32_t slot) {
#pragma unroll
        for (int q = 0; q < kBinChunks; ++q) {
            const uint32_t i = base + warp * (kBinChunks * 32) + q * 32 + lane;
            if (i < seg_hi) cp_async16(smem_u32(&bin_stage[(slot * kBinChunks + q) * kThreads + tid]), &v.vlights[i]);
        }
        cp_async_commit();
    };
    stage(seg_lo, 0);  // in flight during the slab reduction
    if (tid == 0) {
        s_nan = 0;
        s_nonfinite = 0;
        if (k0 == 0 && h == 0 && v.queue) *v.queue = 0u;  // the single-view culling launch's item counter
    }
    __syncthreads();
    // One pass over each slice's cluster AABBs: the slab (lowest min.z,
    // highest max.z) and the union box of every cluster group, the culling
    // kernel's filter box.  Lanes of a warp hold consecutive clusters, so a
    // group (a power of two <= 32 wide) is an aligned run of lanes, reduced
    // with xor shuffles.  A NaN bound makes the slab, or the group's box,
    // infinite.
    const uint32_t gw = v.group_width, gps = (xy + gw - 1) / gw;
    const bool write_boxes = v.group_boxes && h == 0;  // the first segment's CTA writes the group boxes
    const uint32_t span = write_boxes ? gps * gw : xy;  // clusters a pass covers (groups padded)
#pragma unroll
    for (uint32_t sl = 0; sl < kBinSlices; ++sl) {
        float lo = inf, hi = -inf;
        bool nan = false;
        if (sl < ns) {
            const size_t c0 = (size_t)(k0 + sl) * xy;
            for (uint32_t cb = 0; cb < span; cb += kThreads) {  // uniform trip count: the shuffles below
                const uint32_t c = cb + tid;
                float4 a = make_float4(inf, inf, inf, 0.f), b = make_float4(-inf, -inf, -inf, 0.f);
                if (c < xy) {
                    a = v.aabbs[2 * (c0 + c)];
                    b = v.aabbs[2 * (c0 + c) + 1];
                    nan |= (a.z != a.z) | (b.z != b.z);
                    lo = fminf(lo, a.z);
                    hi = fmaxf(hi, b.z);
                }
                if (write_boxes) {
                    bool gnan = (a.x != a.x) | (a.y != a.y) | (a.z != a.z) | (b.x != b.x) | (b.y != b.y) | (b.z != b.z);
                    for (uint32_t o = 1; o < gw; o <<= 1) {
                        a.x = fminf(a.x, __shfl_xor_sync(kFull, a.x, o));
                        a.y = fminf(a.y, __shfl_xor_sync(kFull, a.y, o));
                        a.z = fminf(a.z, __shfl_xor_sync(kFull, a.z, o));
                        b.x = fmaxf(b.x, __shfl_xor_sync(kFull, b.x, o));
                        b.y = fmaxf(b.y, __shfl_xor_sync(kFull, b.y, o));
                        b.z = fmaxf(b.z, __shfl_xor_sync(kFull, b.z, o));
                    }
                    const uint32_t seg = gw == 32 ? kFull : ((1u << gw) - 1u) << (lane & ~(gw - 1));
                    gnan = (__ballot_sync(kFull, gnan) & seg) != 0;
                    if (c < gps * gw && (lane & (gw - 1)) == 0) {
                        const size_t g = (size_t)(k0 + sl) * gps + c / gw;
                        v.group_boxes[2 * g] = gnan ? make_float4(-inf, -inf, -inf, 0.f) : make_float4(a.x, a.y, a.z, 0.f);
                        v.group_boxes[2 * g + 1] = gnan ? make_float4(inf, inf, inf, 0.f) : make_float4(b.x, b.y, b.z, 0.f);
                    }
                }
            }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            lo = fminf(lo, __shfl_xor_sync(kFull, lo, o));
            hi = fmaxf(hi, __shfl_xor_sync(kFull, hi, o));
        }
        if (lane == 0) {
            s_lo[sl][warp] = lo;
            s_hi[sl][warp] = hi;
        }
        if (nan) atomicOr(&s_nan, 1u << sl);
    }
    __syncthreads();
    float lo[kBinSlices], hi[kBinSlices];
#pragma unroll
    for (uint32_t sl = 0; sl < kBinSlices; ++sl) {
        lo[sl] = s_lo[sl][0];
        hi[sl] = s_hi[sl][0];
        for (int q = 1; q < kBinWarps; ++q) {
            lo[sl] = fminf(lo[sl], s_lo[sl][q]);
            hi[sl] = fmaxf(hi[sl], s_hi[sl][q]);
        }
        if ((s_nan >> sl) & 1u) {
            lo[sl] = -inf;
            hi[sl] = inf;
        }
    }

    const uint32_t lt_mask = (1u << lane) - 1u;
    uint32_t running[kBinSlices] = {};
    uint32_t nonfinite = 0;  // bit sl: this thread binned a non-finite light into slice sl
    uint32_t slot = 0;
    for (uint32_t base = seg_lo; base < seg_hi; base += kStep, slot ^= 1u) {
        // the other slot was read into registers a step ago, before a barrier
        if (base + kStep < seg_hi) {
            stage(base + kStep, slot ^ 1u);
            cp_async_wait<1>();
        } else {
            cp_async_wait<0>();
        }
        float4 L[kBinChunks];
        bool fin[kBinChunks];
#pragma unroll
        for (int q = 0; q < kBinChunks; ++q) {
            const uint32_t i = base + warp * (kBinChunks * 32) + q * 32 + lane;
            L[q] = i < seg_hi ? bin_stage[(slot * kBinChunks + q) * kThreads + tid] : make_float4(0.f, 0.f, 0.f, -inf);
            fin[q] = finite_bits(L[q].x) && finite_bits(L[q].y) && finite_bits(L[q].z);
        }
        uint32_t m[kBinSlices][kBinChunks];
#pragma unroll
        for (uint32_t sl = 0; sl < kBinSlices; ++sl) {
            uint32_t wcount = 0;
#pragma unroll
            for (int q = 0; q < kBinChunks; ++q) {
                const float dz = max3f(__fsub_rn(lo[sl], L[q].z), __fsub_rn(L[q].z, hi[sl]), 0.0f);
                const bool pass = sl < ns && __fmul_rn(dz, dz) < L[q].w;
                nonfinite |= (pass && !fin[q]) ? (1u << sl) : 0u;
                m[sl][q] = __ballot_sync(kFull, pass);
                wcount += __popc(m[sl][q]);
            }
            if (lane == 0) s_cnt[sl][warp] = wcount;
        }
        __syncthreads();
#pragma unroll
        for (uint32_t sl = 0; sl < kBinSlices; ++sl) {
            if (sl >= ns) break;
            const uint32_t c = lane < kBinWarps ? s_cnt[sl][lane] : 0u;
            const uint32_t incl = warp_inclusive_scan(c, lane);
            uint32_t pos = running[sl] + __shfl_sync(kFull, incl - c, warp);
            float4* out_l = v.slice_lights + (size_t)(k0 + sl) * v.lpad + seg_lo;
            uint32_t* out_i = v.slice_idx + (size_t)(k0 + sl) * v.lpad + seg_lo;
#pragma unroll
            for (int q = 0; q < kBinChunks; ++q) {
                if ((m[sl][q] >> lane) & 1u) {
                    const uint32_t p = pos + __popc(m[sl][q] & lt_mask);
                    out_l[p] = L[q];
                    out_i[p] = base + warp * (kBinChunks * 32) + q * 32 + lane;
                }
                pos += __popc(m[sl][q]);
            }
            running[sl] += __shfl_sync(kFull, incl, 31);
        }
        __syncthreads();  // s_cnt is rewritten next step
    }
    if (nonfinite) atomicOr(&s_nonfinite, nonfinite);
#pragma unroll
    for (uint32_t sl = 0; sl < kBinSlices; ++sl) {
        if (sl >= ns) break;
        const uint32_t npad = (running[sl] + 31) & ~31u;  // <= seg_hi - seg_lo: both are multiples of 32
        float4* out_l = v.slice_lights + (size_t)(k0 + sl) * v.lpad + seg_lo;
        uint32_t* out_i = v.slice_idx + (size_t)(k0 + sl) * v.lpad + seg_lo;
        for (uint32_t p = running[sl] + tid; p < npad; p += kBinWarps * 32) {
            out_l[p] = make_float4(0.f, 0.f, 0.f, -inf);
            out_i[p] = 0;
        }
        if (tid == 0) {
            v.slice_count[2 * (k0 + sl) + h] = npad;
            if (kParts == 1) v.slice_count[2 * (k0 + sl) + 1] = 0u;  // an empty second segment
        }
    }
    __syncthreads();
    if (tid < ns) {
        v.slice_nonfinite[2 * (k0 + tid) + h] = (s_nonfinite >> tid) & 1u;
        if (kParts == 1) v.slice_nonfinite[2 * (k0 + tid) + 1] = 0u;
    }
    if (tid == 0 && v.work) atomicAdd(&v.work[0], (unsigned long long)(seg_hi - seg_lo) * ns);
}

__global__ void __launch_bounds__(kBinWarpsSingle * 32) bin_slices_kernel(const ViewCull v)
{
    // The slice's cluster AABBs do not come from the light transform this
    // launch waits for: pull them into L2 while it finishes (a hint only; the
    // loads below still read them after the wait).
    {
        const uint32_t k = (blockIdx.x >> 1) * kBinSlicesSingle;
        const uint32_t ns = min((uint32_t)kBinSlicesSingle, v.slices - k);
        const char* p = reinterpret_cast<const char*>(v.aabbs + 2 * (size_t)k * v.slice_clusters);
        const uint32_t lines = (ns * v.slice_clusters * (uint32_t)sizeof(CfAABB) + 127) / 128;
        for (uint32_t l = threadIdx.x; l < lines; l += blockDim.x)
            asm volatile("prefetch.global.L2 [%0];" ::"l"(p + 128 * (size_t)l));
    }
    grid_dependency_wait();
    launch_dependents();
    bin_slices_body<kBinWarpsSingle, kBinSlicesSingle, 2>(v, blockIdx.x);
}

// Batched binning: block b is slice block b - prefix[v] of view v.
__global__ void __launch_bounds__(kBinWarpsBatch * 32, 2) batch_bin_kernel(const ViewJob* __restrict__ jobs,
                                                                        const uint32_t* __restrict__ prefix,
                                                                        const uint32_t* __restrict__ order,
                                                                        uint32_t n_views)
{
    // block ranges follow `order` (when given), heaviest views first, so
    // that their long blocks start in the first wave
    const uint32_t r = find_view(prefix, n_views, blockIdx.x);
    const uint32_t vi = order ? __ldg(&order[r]) : r;
    bin_slices_body<kBinWarpsBatch, kBinSlicesBatch, 1>(jobs[vi].v, blockIdx.x - __ldg(&prefix[r]));
}

// ---------------------------------------------------------------------------
// Finalize: cells = exclusive scan of counts in cluster order, packed copy.
// ---------------------------------------------------------------------------

// Offset scan, one 1024-thread CTA per view: warp w owns the clusters
// [w*rows*32, (w+1)*rows*32) as `rows` coalesced rows of 32; pass 1 sums
// them, warp 0 scans the 32 warp sums, pass 2 scans each row with shuffles
// and writes the LightCells.  O(C) work and no dependency between CTAs.
constexpr uint32_t kScanThreads = 1024;
__device__ __forceinline__ void scan_body(const ViewCull& v)
{
    constexpr uint32_t NW = kScanThreads / 32;
    constexpr int R = 8;  // rows of 32 groups each warp holds in registers per pass
    __shared__ uint32_t s_warp[NW];
    __shared__ uint32_t s_total;
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t C = v.groups;
    uint32_t carry = 0;
    for (uint32_t p0 = 0; p0 < C; p0 += kScanThreads * R) {
        uint32_t n[R], inc[R], wsum = 0;
#pragma unroll
        for (int r = 0; r < R; ++r) {  // all loads issued before any is used
            const uint32_t c = p0 + (warp * R + r) * 32 + lane;
            n[r] = c < C ? v.group_sums[c] : 0u;
        }
#pragma unroll
        for (int r = 0; r < R; ++r) {
            inc[r] = warp_inclusive_scan(n[r], lane);
            wsum += __shfl_sync(kFull, inc[r], 31);
        }
        if (lane == 0) s_warp[warp] = wsum;
        __syncthreads();
        if (warp == 0) {
            const uint32_t x = s_warp[lane];
            const uint32_t i = warp_inclusive_scan(x, lane);
            s_warp[lane] = i - x;
            if (lane == 31) s_total = i;
        }
        __syncthreads();
        uint32_t base = carry + s_warp[warp];
#pragma unroll
        for (int r = 0; r < R; ++r) {
            const uint32_t c = p0 + (warp * R + r) * 32 + lane;
            if (c < C) v.group_offsets[c] = base + inc[r] - n[r];
            base += __shfl_sync(kFull, inc[r], 31);
        }
        carry += s_total;
        __syncthreads();  // s_warp / s_total are rewritten by the next pass
    }
    if (v.total && threadIdx.x == 0) *v.total = carry;
}

// LightCell and packed copy, one warp per cluster: its offset is its group's
// offset plus the counts of the group's earlier clusters (one coalesced load
// and a warp sum), then its staging slice is copied (at most cap / 32
// coalesced iterations).  Every warp's loads are independent of the others'.
constexpr uint32_t kCopyWarps = 8;
constexpr uint32_t kCopyIlp = 8;
__global__ void __launch_bounds__(kScanThreads) scan_kernel(const ViewCull v)
{
    grid_dependency_wait();
    launch_dependents();
    scan_body(v);
}

// Batched offset scan: one CTA per view.
__global__ void __launch_bounds__(kScanThreads) batch_scan_kernel(const ViewJob* __restrict__ jobs)
{
    scan_body(jobs[blockIdx.x].v);
}

// One warp per cluster group: the group's cells from its counts (a warp
// scan on top of the group's offset), then its hits moved from the staging
// rows to the packed list, 32 at a time across the group's clusters (each
// lane finds its cluster by a binary search over the warp's exclusive sums).
__device__ __forceinline__ void copy_body(const ViewCull& v, uint32_t blk)
{
    const uint32_t b = blk * kCopyWarps + (threadIdx.x >> 5), lane = threadIdx.x & 31;
    if (b >= v.groups) return;
    uint32_t first, end;
    group_range(v, b, &first, &end);
    const uint32_t c = first + lane;
    const uint32_t cnt = c < end ? v.counts[c] : 0u;
    const uint32_t incl = warp_inclusive_scan(cnt, lane);
    const uint32_t excl = incl - cnt;
    const uint32_t base = v.group_offsets[b];
    if (c < end) v.cells[c] = CfLightCell{base + excl, cnt};
    const uint32_t total = __shfl_sync(kFull, incl, 31);
    // kCopyIlp independent loads in flight per lane: a group of capped
    // clusters holds thousands of hits and its warp sets the launch's length
    for (uint32_t i0 = 0; i0 < total; i0 += 32 * kCopyIlp) {
        size_t src[kCopyIlp];
        uint32_t val[kCopyIlp];
#pragma unroll
        for (uint32_t u = 0; u < kCopyIlp; ++u) {
            const uint32_t i = i0 + u * 32 + lane;
            uint32_t q = 0;  // the last cluster whose exclusive sum is <= i (lanes past the group hold `total`)
#pragma unroll
            for (uint32_t step = 16; step; step >>= 1) {
                const uint32_t e = __shfl_sync(kFull, excl, q + step);
                if (e <= i) q += step;
            }
            const uint32_t eq = __shfl_sync(kFull, excl, q);
            src[u] = (size_t)(first + q) * v.cap + (i - eq);
        }
#pragma unroll
        for (uint32_t u = 0; u < kCopyIlp; ++u) val[u] = i0 + u * 32 + lane < total ? __ldg(&v.staging[src[u]]) : 0u;
#pragma unroll
        for (uint32_t u = 0; u < kCopyIlp; ++u)
            if (i0 + u * 32 + lane < total) v.indices[base + i0 + u * 32 + lane] = val[u];
    }
}

// A single view: one 256-thread CTA per cluster group (a view has too few
// groups to fill the GPU with one warp each, and a group of capped clusters
// holds thousands of hits).  Warp 0 writes the group's cells from its counts
// (a warp scan on top of the group's offset); then all threads move the hits
// from the staging rows to the packed list, each finding its cluster by a
// binary search over the exclusive sums, four loads in flight per thread.
constexpr uint32_t kCopyThreads = 256, kCopyBlockIlp = 4;
constexpr uint32_t kSumGroupsMax = 8192;  // views with more groups scan their totals in a launch of their own
// kSumGroups: the view has at most kSumGroupsMax groups and no scan launch
// ran; each block sums the totals of the groups before its own (from L2/L1,
// at most kSumGroupsMax / kCopyThreads loads per thread) and the last block
// writes the view's total.
template <bool kSumGroups>
__global__ void __launch_bounds__(kCopyThreads) copy_kernel(const ViewCull v)
{
    __shared__ uint32_t s_excl[33];
    __shared__ uint32_t s_base;
    __shared__ uint32_t s_part[kCopyThreads / 32];
    grid_dependency_wait();
    const uint32_t b = blockIdx.x, tid = threadIdx.x, lane = tid & 31;
    uint32_t first, end;
    group_range(v, b, &first, &end);
    const uint32_t c = first + lane;
    const uint32_t cnt = tid < 32 && c < end ? v.counts[c] : 0u;  // in flight during the sum below
    if constexpr (kSumGroups) {
        uint32_t part = 0;
#pragma unroll 4
        for (uint32_t j = tid; j < b; j += kCopyThreads) part += __ldg(&v.group_sums[j]);
        part = warp_sum(part);
        if (lane == 0) s_part[tid >> 5] = part;
        __syncthreads();
    }
    if (tid < 32) {
        const uint32_t incl = warp_inclusive_scan(cnt, lane);
        uint32_t base;
        if constexpr (kSumGroups) base = warp_sum(lane < kCopyThreads / 32 ? s_part[lane] : 0u);
        else base = v.group_offsets[b];
        if (c < end) v.cells[c] = CfLightCell{base + incl - cnt, cnt};
        s_excl[lane] = incl - cnt;  // lanes past the group hold the group's total
        if (lane == 31) {
            s_excl[32] = incl;
            s_base = base;
            if (kSumGroups && b == gridDim.x - 1 && v.total) *v.total = base + incl;
        }
    }
    __syncthreads();
    const uint32_t total = s_excl[32], base = s_base;
    const uint32_t* __restrict__ staging = v.staging;
    uint32_t* __restrict__ indices = v.indices;
    for (uint32_t i0 = 0; i0 < total; i0 += kCopyThreads * kCopyBlockIlp) {
        uint32_t val[kCopyBlockIlp];
#pragma unroll
        for (uint32_t u = 0; u < kCopyBlockIlp; ++u) {
            const uint32_t i = i0 + u * kCopyThreads + tid;
            val[u] = 0;
            if (i < total) {
                uint32_t q = 0;  // the last cluster whose exclusive sum is <= i
#pragma unroll
                for (uint32_t step = 16; step; step >>= 1)
                    if (s_excl[q + step] <= i) q += step;
                val[u] = __ldg(&staging[(size_t)(first + q) * v.cap + (i - s_excl[q])]);
            }
        }
#pragma unroll
        for (uint32_t u = 0; u < kCopyBlockIlp; ++u) {
            const uint32_t i = i0 + u * kCopyThreads + tid;
            if (i < total) indices[base + i] = val[u];
        }
    }
}

// Batched copy: block b is copy block b - prefix[v] of view v.
__global__ void __launch_bounds__(kCopyWarps * 32) batch_copy_kernel(const ViewJob* __restrict__ jobs,
                                                                     const uint32_t* __restrict__ prefix,
                                                                     uint32_t n_views)
{
    const uint32_t vi = find_view(prefix, n_views, blockIdx.x);
    copy_body(jobs[vi].v, blockIdx.x - __ldg(&prefix[vi]));
}

// Launches `kernel`; with `overlap`, with programmatic stream serialisation
// (see grid_dependency_wait): it may be scheduled while the stream's previous
// kernel is still running.  A single view's step uses it.  Batched passes do
// not: their kernels are long, and with several streams in flight (the
// server) CTAs launched early would hold SM slots while they wait.
template <typename... Params, typename... Args>
cudaError_t launch_kernel(bool overlap, void (*kernel)(Params...), dim3 grid, dim3 block, size_t smem,
                         cudaStream_t stream, Args&&... args)
{
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = stream;
    cfg.attrs = overlap ? attr : nullptr;
    cfg.numAttrs = overlap ? 1 : 0;
    return cudaLaunchKernelEx(&cfg, kernel, std::forward<Args>(args)...);
}

template <int K, int WARPS, int TILE, int STAGES, bool kBinned>
cudaError_t launch_cull_t(const ViewCull& v, uint32_t* dev_error, cudaStream_t stream)
{
    static_assert(WARPS * K <= 32, "a cluster group fits one warp of the copy kernel");
    if constexpr (kBinned) {
        // one persistent CTA per resident slot, taking the view's groups in order
        const size_t psmem = PipeSmem<K, WARPS, TILE, STAGES>::bytes;
        static const int resident = [psmem] {  // thread-safe one-time query
            int dev = 0, sms = 0, b = 0;
            cudaError_t e = cudaGetDevice(&dev);
            if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
            if (e == cudaSuccess && psmem > 48 * 1024)
                e = cudaFuncSetAttribute(cull_pipe_kernel<K, WARPS, TILE, STAGES>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)psmem);
            if (e == cudaSuccess)
                e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, cull_pipe_kernel<K, WARPS, TILE, STAGES>,
                                                                  (WARPS + 1) * 32, psmem);
            return e == cudaSuccess ? sms * (b > 0 ? b : 1) : 0;
        }();
        if (resident <= 0) return cudaErrorInvalidConfiguration;
        const uint32_t ctas = std::min<uint32_t>(v.groups, (uint32_t)resident);
        return launch_kernel(true, cull_pipe_kernel<K, WARPS, TILE, STAGES>, dim3(ctas), dim3((WARPS + 1) * 32), psmem,
                                 stream, static_cast<const ViewJob*>(nullptr), static_cast<const uint2*>(nullptr),
                                 v.groups, v.queue, dev_error, v);
    } else {
        const size_t smem = CullSmem<K, WARPS, TILE, STAGES>::bytes();
        if (smem > 48 * 1024) {  // opt in above the default 48 KB (a per-device attribute)
            const cudaError_t e = cudaFuncSetAttribute(cull_kernel<K, WARPS, TILE, STAGES>,
                                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            if (e != cudaSuccess) return e;
        }
        return launch_kernel(true, cull_kernel<K, WARPS, TILE, STAGES>, dim3(v.groups), dim3((WARPS + 1) * 32), smem,
                                 stream, v, dev_error);
    }
}

}  // namespace

// (clusters per warp, consumer warps, lights per stage, stages, binned)
#define CF_CULL_CONFIGS(X)  \
    X(1, 4, 512, 4, false)  \
    X(2, 4, 512, 4, false)  \
    X(4, 4, 512, 4, false)  \
    X(1, 8, 512, 4, false)  \
    X(2, 8, 512, 4, false)  \
    X(4, 8, 512, 4, false)  \
    X(1, 4, 256, 4, true)   \
    X(2, 4, 256, 4, true)   \
    X(4, 4, 256, 4, true)   \
    X(1, 8, 256, 4, true)   \
    X(2, 8, 256, 4, true)   \
    X(4, 8, 256, 4, true)   \
    X(2, 4, 512, 2, true)   \
    X(4, 4, 512, 2, true)   \
    X(2, 8, 512, 2, true)   \
    X(4, 8, 512, 2, true)   \
    X(2, 8, 1024, 2, true)  \
    X(4, 8, 1024, 2, true)

bool cull_config_supported(const CullConfig& c)
{
    if (c.binned == kModeOneLaunch)
        return c.clusters_per_warp >= 1 && (uint32_t)c.clusters_per_warp <= kOneLaunchMaxClustersPerCta &&
               c.stages == 1 && one_launch_shape_supported(c.warps, c.tile);
#define CF_MATCH(K, W, T, S, B) \
    if (c.clusters_per_warp == K && c.warps == W && c.tile == T && c.stages == S && (c.binned != 0) == B) return true;
    CF_CULL_CONFIGS(CF_MATCH)
#undef CF_MATCH
    return false;
}

// Slice binning pays off once a view has enough tests to amortise its extra
// launch and passes: on a GB300 the 2560x1600 32x18x48 view with 16384
// lights (453 M tests) culls five times faster binned than brute force.
// Below that, a view whose lights fit one launch's registers (at most
// kOneLaunchMaxLights) and whose clusters spread over the resident CTAs at
// most kOneLaunchMaxClustersPerCta each is culled in one launch; the rest
// brute force.
constexpr uint64_t kBinnedMinTests = 16ull << 20;

CullConfig default_cull_config(uint32_t clusters, uint32_t lights, uint32_t slices)
{
    if (slices >= 2 && (uint64_t)clusters * lights >= kBinnedMinTests) return CullConfig{2, 8, 1024, 2, 1};
    CullConfig one{};
    if (one_launch_config(clusters, lights, &one)) return one;
    if (clusters <= 8192) return CullConfig{1, 8, 512, 4, 0};
    return CullConfig{2, 8, 512, 4, 0};
}

WorkspaceLayout workspace_layout(uint32_t clusters, uint32_t lights, uint32_t cap, uint32_t slices, int mode,
                                 uint32_t groups)
{
    auto al = [](size_t x) { return (x + 255) & ~(size_t)255; };
    WorkspaceLayout w{};
    size_t off = 256;  // status words
    if (mode == kModeOneLaunch) {
        w.partials = off;
        off += al((size_t)groups * sizeof(unsigned long long));
        w.bytes = off;
        return w;
    }
    const bool binned = mode == kModeBinned;
    const uint32_t lpad = pad_lights(lights);
    w.vlights = off;
    off += al((size_t)lpad * sizeof(float4));
    w.nonfinite = off;
    off += al((size_t)granules(lpad) * sizeof(uint32_t));
    w.counts = off;
    off += al((size_t)clusters * sizeof(uint32_t));
    w.staging = off;
    off += al((size_t)clusters * cap * sizeof(uint32_t));
    w.group_sums = off;
    off += al((size_t)groups * sizeof(uint32_t));
    w.group_offsets = off;
    off += al((size_t)groups * sizeof(uint32_t));
    if (binned) {
        w.slice_lights = off;
        off += al((size_t)slices * lpad * sizeof(float4));
        w.slice_idx = off;
        off += al((size_t)slices * lpad * sizeof(uint32_t));
        w.slice_count = off;
        off += al((size_t)2 * slices * sizeof(uint32_t));
        w.slice_nonfinite = off;
        off += al((size_t)2 * slices * sizeof(uint32_t));
        w.group_boxes = off;
        off += al((size_t)groups * 2 * sizeof(float4));
    }
    w.bytes = off;
    return w;
}

cudaError_t set_test_knobs_kernels(uint64_t wait_limit_ns, uint32_t inject)
{
    const unsigned long long w = wait_limit_ns;
    const unsigned int i = inject;
    cudaError_t e = cudaMemcpyToSymbol(g_wait_limit_ns, &w, sizeof(w));
    if (e == cudaSuccess) e = cudaMemcpyToSymbol(g_inject_stall, &i, sizeof(i));
    return e;
}

cudaError_t launch_aabb(const CfClusterForwardUBO& ubo, CfAABB* aabbs, cudaStream_t stream)
{
    const uint32_t C = ubo.sliceCountX * ubo.sliceCountY * ubo.sliceCountZ;
    if (C == 0) return cudaSuccess;
    aabb_kernel<<<(C + 255) / 256, 256, 0, stream>>>(ubo, reinterpret_cast<float4*>(aabbs), C);
    return cudaGetLastError();
}

cudaError_t launch_light_xform(const CfLightData* lights, uint32_t count, const float view[16], float4* vlights,
                               uint32_t* nonfinite, cudaStream_t stream)
{
    const uint32_t lpad = pad_lights(count);
    if (lpad == 0) return cudaSuccess;
    Mat4 m;
    for (int i = 0; i < 16; ++i) m.m[i] = view[i];
    return launch_kernel(true, light_xform_kernel, dim3(granules(lpad)), dim3(kFlagGranule), 0, stream, lights, count,
                             lpad, m, vlights, nonfinite);
}

cudaError_t launch_bin(const ViewCull& v, cudaStream_t stream)
{
    if (v.slices == 0) return cudaSuccess;
    constexpr size_t smem = bin_stage_bytes(kBinWarpsSingle);
    static const cudaError_t attr =  // one-time opt-in above 48 KB
        cudaFuncSetAttribute(bin_slices_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (attr != cudaSuccess) return attr;
    return launch_kernel(true, bin_slices_kernel, dim3((v.slices + kBinSlicesSingle - 1) / kBinSlicesSingle * 2),
                             dim3(kBinWarpsSingle * 32), smem, stream, v);
}

cudaError_t launch_cull(const ViewCull& v, const CullConfig& cfg, uint32_t* dev_error, cudaStream_t stream)
{
    if (v.clusters == 0) return cudaSuccess;
#define CF_DISPATCH(K, W, T, S, B)                                                                              \
    if (cfg.clusters_per_warp == K && cfg.warps == W && cfg.tile == T && cfg.stages == S && (cfg.binned != 0) == B) \
        return launch_cull_t<K, W, T, S, B>(v, dev_error, stream);
    CF_CULL_CONFIGS(CF_DISPATCH)
#undef CF_DISPATCH
    return cudaErrorInvalidValue;
}

cudaError_t launch_finalize(const ViewCull& v, cudaStream_t stream)
{
    if (v.clusters == 0) {
        if (v.total) return cudaMemsetAsync(v.total, 0, sizeof(uint32_t), stream);
        return cudaSuccess;
    }
    if (v.groups <= kSumGroupsMax)  // each copy block sums the earlier groups' totals itself
        return launch_kernel(true, copy_kernel<true>, dim3(v.groups), dim3(kCopyThreads), 0, stream, v);
    const cudaError_t e = launch_kernel(true, scan_kernel, dim3(1), dim3(kScanThreads), 0, stream, v);
    if (e != cudaSuccess) return e;
    return launch_kernel(true, copy_kernel<false>, dim3(v.groups), dim3(kCopyThreads), 0, stream, v);
}

// ---------------------------------------------------------------------------
// Read-back into host memory the device can address (pinned and mapped, on
// this system over NVLink-C2C): the hit total, the LightCells and the first
// min(total, capacity) indices, in one launch with no host round trip for the
// count.  Grid-stride over 32-bit words, 16 bytes per access where both sides
// are 16-byte aligned.
// ---------------------------------------------------------------------------
namespace {

__device__ __forceinline__ void copy_words(const uint32_t* __restrict__ src, uint32_t* __restrict__ dst, uint64_t n,
                                           bool vec, uint64_t tid, uint64_t stride)
{
    uint64_t head = 0;
    if (vec) {
        const uint64_t n4 = n / 4;
        const uint4* s4 = reinterpret_cast<const uint4*>(src);
        uint4* d4 = reinterpret_cast<uint4*>(dst);
        for (uint64_t i = tid; i < n4; i += stride) d4[i] = s4[i];
        head = n4 * 4;
    }
    for (uint64_t i = head + tid; i < n; i += stride) dst[i] = src[i];
}

__global__ void __launch_bounds__(256) readback_kernel(const uint32_t* __restrict__ cells, uint32_t cell_words,
                                                       const uint32_t* __restrict__ indices,
                                                       const uint32_t* __restrict__ d_total, uint64_t capacity,
                                                       uint32_t* __restrict__ h_cells, uint32_t* __restrict__ h_indices,
                                                       uint32_t* __restrict__ h_total, bool vec_cells, bool vec_indices)
{
    const uint32_t total = *d_total;
    const uint64_t tid = (uint64_t)blockIdx.x * 256 + threadIdx.x, stride = (uint64_t)gridDim.x * 256;
    if (tid == 0) *h_total = total;
    if (h_cells) copy_words(cells, h_cells, cell_words, vec_cells, tid, stride);
    if (h_indices) copy_words(indices, h_indices, total < capacity ? total : capacity, vec_indices, tid, stride);
}

}  // namespace

cudaError_t launch_readback(const CfLightCell* cells, uint32_t clusters, const uint32_t* indices,
                            const uint32_t* d_total, uint64_t capacity, CfLightCell* h_cells, uint32_t* h_indices,
                            uint32_t* h_total, cudaStream_t stream)
{
    auto al16 = [](const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; };
    const uint64_t words = std::max<uint64_t>(2ull * clusters, h_indices ? capacity : 0ull);
    const uint32_t blocks = (uint32_t)std::min<uint64_t>(std::max<uint64_t>((words + 1023) / 1024, 1ull), 1216ull);
    readback_kernel<<<blocks, 256, 0, stream>>>(reinterpret_cast<const uint32_t*>(cells), 2u * clusters, indices,
                                                d_total, capacity, reinterpret_cast<uint32_t*>(h_cells), h_indices,
                                                h_total, al16(cells) && al16(h_cells), al16(indices) && al16(h_indices));
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Light jitter: dst = src with every position coordinate moved by sigma times
// an Irwin-Hall variate (the sum of 12 uniforms in [0, 1) minus 6, mean 0,
// variance 1, a close stand-in for a unit Gaussian).  The uniforms come from
// a splitmix64 finaliser over (seed, light, axis, term), so the host can
// reproduce every bit: u = (hash >> 40) * 2^-24, summed in term order with
// round-to-nearest adds, then scaled and added with one rounding each.
// ---------------------------------------------------------------------------
namespace {

__device__ __forceinline__ uint64_t splitmix_finalise(uint64_t x)
{
    x ^= x >> 30;
    x *= 0xBF58476D1CE4E5B9ull;
    x ^= x >> 27;
    x *= 0x94D049BB133111EBull;
    x ^= x >> 31;
    return x;
}

// Light i of a jitter: its position moved by sigma * (Irwin-Hall variate - 6)
// per axis, the variate from (seed, i, axis).
__device__ __forceinline__ void jitter_light(const CfLightData* __restrict__ src, CfLightData* __restrict__ dst,
                                             uint32_t i, uint64_t seed, float sigma)
{
    CfLightData L = src[i];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        float s = 0.0f;
        for (int k = 0; k < 12; ++k) {
            const uint64_t h = splitmix_finalise(seed + (uint64_t)i * 0x9E3779B97F4A7C15ull +
                                                 (uint64_t)(a * 12 + k) * 0xD1B54A32D192ED03ull);
            s = __fadd_rn(s, __fmul_rn((float)(uint32_t)(h >> 40), 0x1p-24f));
        }
        L.position[a] = __fadd_rn(L.position[a], __fmul_rn(sigma, __fsub_rn(s, 6.0f)));
    }
    dst[i] = L;
}

// Many jitters in one launch: block b belongs to task j where
// block_start[j] <= b < block_start[j + 1].
struct JitterTaskTable {
    JitterTask t[kMaxJitterTasks];
    uint32_t block_start[kMaxJitterTasks + 1];
    uint32_t count;
};

__global__ void __launch_bounds__(256) jitter_tasks_kernel(const JitterTaskTable T)
{
    uint32_t lo = 0, hi = T.count;  // block_start[lo] <= blockIdx.x < block_start[hi]
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (T.block_start[mid] <= blockIdx.x) lo = mid;
        else hi = mid;
    }
    const JitterTask& t = T.t[lo];
    const uint32_t i = (blockIdx.x - T.block_start[lo]) * 256 + threadIdx.x;
    if (i < t.n) jitter_light(t.src, t.dst, i, t.seed, t.sigma);
}

// Copies of many light sets from device-mapped pinned host memory in one
// launch: block b belongs to task j where block_start[j] <= b <
// block_start[j + 1] and copies 16-byte words [256*4*(b - block_start[j]),
// +1024) of it, four loads in flight per thread (the reads cross the
// host link, so the latency is hidden by loads in flight, not by occupancy).
struct UploadTaskTable {
    UploadTask t[kMaxUploadTasks];
    uint32_t block_start[kMaxUploadTasks + 1];
    uint32_t count;
};

__global__ void __launch_bounds__(256) upload_tasks_kernel(const UploadTaskTable T)
{
    uint32_t lo = 0, hi = T.count;
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (T.block_start[mid] <= blockIdx.x) lo = mid;
        else hi = mid;
    }
    const UploadTask& t = T.t[lo];
    const uint32_t base = (blockIdx.x - T.block_start[lo]) * 1024 + threadIdx.x;
    uint4 w[4];
#pragma unroll
    for (int k = 0; k < 4; ++k)
        if (base + k * 256 < t.words) w[k] = t.src[base + k * 256];
#pragma unroll
    for (int k = 0; k < 4; ++k)
        if (base + k * 256 < t.words) t.dst[base + k * 256] = w[k];
}

// Moves each light `frames` steps along its orbit (CfLightOrbit), in place:
// per step x' = c*x - s*z, z' = s*x + c*z (products, then the difference or
// sum, each rounded to nearest), then position = center + (x', 0, z').  Reads
// 32 bytes and writes 32 bytes per light.
__global__ void __launch_bounds__(256) orbit_kernel(CfLightData* __restrict__ lights,
                                                    CfLightOrbit* __restrict__ orbits, uint64_t n, uint32_t frames)
{
    for (uint64_t i = blockIdx.x * 256ull + threadIdx.x; i < n; i += (uint64_t)gridDim.x * 256ull) {
        float4* o = reinterpret_cast<float4*>(&orbits[i]);
        float4 st = o[0];
        const float4 ctr = o[1];
        float x = st.x, z = st.y;
        for (uint32_t f = 0; f < frames; ++f) {
            const float nx = __fsub_rn(__fmul_rn(st.z, x), __fmul_rn(st.w, z));
            const float nz = __fadd_rn(__fmul_rn(st.w, x), __fmul_rn(st.z, z));
            x = nx;
            z = nz;
        }
        st.x = x;
        st.y = z;
        o[0] = st;
        *reinterpret_cast<float4*>(&lights[i].position[0]) =
            make_float4(__fadd_rn(ctr.x, x), ctr.y, __fadd_rn(ctr.z, z), ctr.w);
    }
}

}  // namespace

cudaError_t launch_jitter_tasks(const JitterTask* tasks, uint32_t n, cudaStream_t stream)
{
    for (uint32_t first = 0; first < n;) {
        JitterTaskTable T{};
        uint32_t blocks = 0;
        T.count = 0;
        // a task that reads what an earlier task of this launch writes goes into the next launch
        while (first + T.count < n && T.count < kMaxJitterTasks) {
            const JitterTask& t = tasks[first + T.count];
            bool reads_earlier = false;
            for (uint32_t q = 0; q < T.count; ++q) reads_earlier |= T.t[q].dst == t.src;
            if (reads_earlier) break;
            T.t[T.count] = t;
            T.block_start[T.count] = blocks;
            blocks += (t.n + 255) / 256;
            ++T.count;
        }
        T.block_start[T.count] = blocks;
        if (blocks) jitter_tasks_kernel<<<blocks, 256, 0, stream>>>(T);
        const cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
        first += T.count;
    }
    return cudaSuccess;
}

cudaError_t launch_upload_tasks(const UploadTask* tasks, uint32_t n, cudaStream_t stream)
{
    for (uint32_t first = 0; first < n;) {
        UploadTaskTable T{};
        uint32_t blocks = 0;
        T.count = 0;
        while (first + T.count < n && T.count < kMaxUploadTasks) {
            const UploadTask& t = tasks[first + T.count];
            T.t[T.count] = t;
            T.block_start[T.count] = blocks;
            blocks += (uint32_t)((t.words + 1023) / 1024);
            ++T.count;
        }
        T.block_start[T.count] = blocks;
        if (blocks) upload_tasks_kernel<<<blocks, 256, 0, stream>>>(T);
        const cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
        first += T.count;
    }
    return cudaSuccess;
}

cudaError_t launch_orbits(CfLightData* lights, CfLightOrbit* orbits, uint64_t n, uint32_t frames, cudaStream_t stream)
{
    if (n == 0) return cudaSuccess;
    // grid-stride: at most 16 resident 256-thread blocks on each of 152 SMs
    const uint64_t blocks = std::min<uint64_t>((n + 255) / 256, 152ull * 16ull);
    orbit_kernel<<<(unsigned)blocks, 256, 0, stream>>>(lights, orbits, n, frames);
    return cudaGetLastError();
}

cudaError_t launch_batch_aabb(const AabbJob* jobs, const uint32_t* prefix, uint32_t n_views, uint32_t blocks,
                              cudaStream_t stream)
{
    if (blocks == 0) return cudaSuccess;
    batch_aabb_kernel<<<blocks, 256, 0, stream>>>(jobs, prefix, n_views);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Batches.
// ---------------------------------------------------------------------------
namespace {

// Batches are always binned: a plain configuration has no batched kernel.
template <int K, int WARPS, int TILE, int STAGES, bool kBinned>
cudaError_t launch_cull_batch_t(const BatchCull& b, int ctas, uint32_t* dev_error, cudaStream_t stream)
{
    static_assert(WARPS * K <= 32, "a cluster group fits one warp of the copy kernel");
    if constexpr (!kBinned) {
        return cudaErrorInvalidValue;
    } else {
        const size_t smem = PipeSmem<K, WARPS, TILE, STAGES>::bytes;
        if (smem > 48 * 1024) {
            const cudaError_t e = cudaFuncSetAttribute(cull_pipe_kernel<K, WARPS, TILE, STAGES>,
                                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            if (e != cudaSuccess) return e;
        }
        return launch_kernel(false, cull_pipe_kernel<K, WARPS, TILE, STAGES>, dim3(ctas), dim3((WARPS + 1) * 32), smem,
                                 stream, b.jobs, b.items, b.n_items, b.queue, dev_error, ViewCull{});
    }
}

template <int K, int WARPS, int TILE, int STAGES, bool kBinned>
cudaError_t batch_occupancy_t(int* blocks)
{
    if constexpr (!kBinned) {
        *blocks = 0;
        return cudaErrorInvalidValue;
    } else {
        // the opt-in above 48 KB must precede the query, or it reports 0 blocks
        const size_t smem = PipeSmem<K, WARPS, TILE, STAGES>::bytes;
        if (smem > 48 * 1024) {
            const cudaError_t e = cudaFuncSetAttribute(cull_pipe_kernel<K, WARPS, TILE, STAGES>,
                                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            if (e != cudaSuccess) return e;
        }
        return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks, cull_pipe_kernel<K, WARPS, TILE, STAGES>,
                                                             (WARPS + 1) * 32, smem);
    }
}

}  // namespace

cudaError_t launch_batch_xform(const ViewJob* jobs, const uint32_t* prefix, uint32_t n_views, uint32_t blocks,
                               uint32_t* queues, uint32_t n_queues, cudaStream_t stream)
{
    if (blocks == 0) {  // no lights anywhere: only the queues need resetting
        return n_queues ? cudaMemsetAsync(queues, 0, n_queues * sizeof(uint32_t), stream) : cudaSuccess;
    }
    return launch_kernel(false, batch_xform_kernel, dim3(blocks), dim3(kFlagGranule), 0, stream, jobs, prefix, n_views,
                             queues, n_queues);
}

cudaError_t launch_batch_bin(const ViewJob* jobs, const uint32_t* prefix, const uint32_t* order, uint32_t n_views,
                             uint32_t blocks,
                             cudaStream_t stream)
{
    if (blocks == 0) return cudaSuccess;
    constexpr size_t smem = bin_stage_bytes(kBinWarpsBatch);
    static const cudaError_t attr =  // one-time opt-in above 48 KB
        cudaFuncSetAttribute(batch_bin_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (attr != cudaSuccess) return attr;
    return launch_kernel(false, batch_bin_kernel, dim3(blocks), dim3(kBinWarpsBatch * 32), smem, stream, jobs, prefix,
                             order, n_views);
}

cudaError_t launch_batch_cull(const BatchCull& b, const CullConfig& cfg, int ctas, uint32_t* dev_error,
                              cudaStream_t stream)
{
    if (b.n_items == 0 || ctas <= 0) return cudaSuccess;
#define CF_DISPATCH(K, W, T, S, B)                                                                              \
    if (cfg.clusters_per_warp == K && cfg.warps == W && cfg.tile == T && cfg.stages == S && (cfg.binned != 0) == B) \
        return launch_cull_batch_t<K, W, T, S, B>(b, ctas, dev_error, stream);
    CF_CULL_CONFIGS(CF_DISPATCH)
#undef CF_DISPATCH
    return cudaErrorInvalidValue;
}

cudaError_t batch_cull_resident_ctas(const CullConfig& cfg, int* ctas)
{
    // per device and configuration, queried once: a server asks for every
    // batch it launches, and each query is several CUDA calls
    constexpr int kDevices = 16, kConfigs = 32;
    static std::atomic<int> cache[kDevices][kConfigs];  // 0: not yet known
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    int slot = -1, index = 0;
#define CF_SLOT(K, W, T, S, B)                                                                                  \
    if (cfg.clusters_per_warp == K && cfg.warps == W && cfg.tile == T && cfg.stages == S && (cfg.binned != 0) == B) \
        slot = index;                                                                                             \
    ++index;
    CF_CULL_CONFIGS(CF_SLOT)
#undef CF_SLOT
    static_assert(kConfigs >= 18, "one cache slot per configuration");
    const bool cached = dev >= 0 && dev < kDevices && slot >= 0;
    if (cached) {
        const int c = cache[dev][slot].load(std::memory_order_relaxed);
        if (c > 0) {
            *ctas = c;
            return cudaSuccess;
        }
    }
    int sms = 0, per_sm = 0;
    e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return e;
#define CF_OCC(K, W, T, S, B)                                                                                   \
    if (cfg.clusters_per_warp == K && cfg.warps == W && cfg.tile == T && cfg.stages == S && (cfg.binned != 0) == B) \
        e = batch_occupancy_t<K, W, T, S, B>(&per_sm);
    CF_CULL_CONFIGS(CF_OCC)
#undef CF_OCC
    if (e != cudaSuccess) return e;
    *ctas = sms * (per_sm > 0 ? per_sm : 1);
    if (cached) cache[dev][slot].store(*ctas, std::memory_order_relaxed);
    return cudaSuccess;
}

cudaError_t launch_batch_scan(const ViewJob* jobs, uint32_t n_views, cudaStream_t stream)
{
    if (n_views == 0) return cudaSuccess;
    return launch_kernel(false, batch_scan_kernel, dim3(n_views), dim3(kScanThreads), 0, stream, jobs);
}

cudaError_t launch_batch_copy(const ViewJob* jobs, const uint32_t* prefix, uint32_t n_views, uint32_t blocks,
                              cudaStream_t stream)
{
    if (blocks == 0) return cudaSuccess;
    return launch_kernel(false, batch_copy_kernel, dim3(blocks), dim3(kCopyWarps * 32), 0, stream, jobs, prefix,
                             n_views);
}

uint32_t copy_blocks(uint32_t groups) { return (groups + kCopyWarps - 1) / kCopyWarps; }
uint32_t bin_blocks(uint32_t slices) { return (slices + kBinSlicesBatch - 1) / kBinSlicesBatch; }

}  // namespace cfk
