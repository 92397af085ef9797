// cf_kernels.cu — sm_103a kernels of the clustered-forward light-culling path.
//
//   aabb_kernel        HelloVulkan/Shaders/ClusteredForward/AABBGenerator.comp:39-89
//                      one thread per cluster, float4 stores
//   light_xform_kernel the `ubo.cameraView * posWorld` and `radius * radius` of
//                      LightCulling.comp:51-56, hoisted to once per light
//   cull_kernel        LightCulling.comp:59-77: a producer warp streams tiles of
//                      view-space lights into shared memory with bulk async
//                      copies (cp.async.bulk + mbarrier); each consumer warp owns
//                      K clusters, its 32 lanes test 32 consecutive lights, and
//                      __ballot_sync/__popc compact the hits in ascending light
//                      order up to the cap
//   finalize_kernel    LightCulling.comp:79-87 with the global atomicAdd replaced
//                      by an exclusive scan of the counts in cluster order, then
//                      the packed copy of each cluster's hits
//
// Floating point follows include/cf_pinned_math.h: every product and sum is an
// explicit round-to-nearest intrinsic, so nothing is contracted into an FMA.
#include "cf_kernels.cuh"

#include <algorithm>

#include "cf_pinned_math.h"

namespace cfk {
namespace {

constexpr unsigned kFull = 0xffffffffu;
constexpr uint64_t kWaitLimitNs = 2000000000ull;  // 2 s per bounded wait
constexpr uint32_t kWaitLimitIters = 1u << 26;

// ---------------------------------------------------------------------------
// PTX helpers: mbarrier and bulk async copy.
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t smem_u32(const void* p)
{
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ uint64_t global_timer_ns()
{
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
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

// Waits for the phase of `parity` to complete; gives up after kWaitLimitNs
// (or kWaitLimitIters polls) and returns false.
__device__ __noinline__ bool mbar_wait_bounded(uint32_t bar, uint32_t parity)
{
    if (mbar_try_wait(bar, parity)) return true;
    const uint64_t t0 = global_timer_ns();
    for (uint32_t it = 0; it < kWaitLimitIters; ++it) {
        if (mbar_try_wait(bar, parity)) return true;
        if (global_timer_ns() - t0 > kWaitLimitNs) break;
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

__device__ __forceinline__ float max3f(float a, float b, float c)
{
    float r;
    asm("max.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
    return r;
}

__device__ __forceinline__ bool finite_bits(float x)
{
    return (__float_as_uint(x) & 0x7f800000u) != 0x7f800000u;
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

__global__ void __launch_bounds__(256) aabb_kernel(const CfClusterForwardUBO ubo, float4* __restrict__ out,
                                                   uint32_t clusters)
{
    const uint32_t c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= clusters) return;
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

// ---------------------------------------------------------------------------
// Light transform: posView = cameraView * position, r^2 = radius * radius.
// One 256-thread block per flag granule.
// ---------------------------------------------------------------------------
struct Mat4 {
    float m[16];
};

__global__ void __launch_bounds__(kFlagGranule) light_xform_kernel(const CfLightData* __restrict__ lights,
                                                                   uint32_t count, uint32_t lpad, const Mat4 view,
                                                                   float4* __restrict__ out,
                                                                   uint32_t* __restrict__ nonfinite)
{
    const uint32_t i = blockIdx.x * kFlagGranule + threadIdx.x;
    bool bad = false;
    if (i < count) {
        const float4 p = __ldg(reinterpret_cast<const float4*>(&lights[i].position[0]));
        const float r = __ldg(&lights[i].radius);
        const float x = cf_mat4_row(view.m, 0, p.x, p.y, p.z, p.w);
        const float y = cf_mat4_row(view.m, 1, p.x, p.y, p.z, p.w);
        const float z = cf_mat4_row(view.m, 2, p.x, p.y, p.z, p.w);
        bad = !(finite_bits(x) && finite_bits(y) && finite_bits(z));
        out[i] = make_float4(x, y, z, cf_fmul(r, r));
    } else if (i < lpad) {
        out[i] = make_float4(0.0f, 0.0f, 0.0f, __uint_as_float(0xff800000u));  // never hits
    }
    const int any_bad = __syncthreads_or(bad);
    if (threadIdx.x == 0) nonfinite[blockIdx.x] = any_bad ? 1u : 0u;
}

// ---------------------------------------------------------------------------
// Culling.
// ---------------------------------------------------------------------------

// Exact for every finite light coordinate against boxes with min <= max on
// each axis (or NaN bounds), which every generated AABB satisfies:
//   v < min:  max3(min - v, v - max, 0) = min - v
//   v > max:  = v - max, and (v - max)^2 == (max - v)^2 bit for bit
//   inside:   both differences are <= 0, so d = 0 and the axis adds +0,
//             which leaves the reference's partial sum unchanged
// NaN bounds are ignored by max.f32 exactly like the reference's false
// comparisons.  Boxes set to +inf on every bound never hit (the capped and
// out-of-range clusters).
__device__ __forceinline__ bool hit_fast(const float4& L, const float* mn, const float* mx)
{
    const float dx = max3f(__fsub_rn(mn[0], L.x), __fsub_rn(L.x, mx[0]), 0.0f);
    const float dy = max3f(__fsub_rn(mn[1], L.y), __fsub_rn(L.y, mx[1]), 0.0f);
    const float dz = max3f(__fsub_rn(mn[2], L.z), __fsub_rn(L.z, mx[2]), 0.0f);
    const float sq = __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz));
    return sq < L.w;
}

// SquaredDistancePointAABB + TestSphereAABB (LightCulling.comp:26-57) as
// written, for granules holding a non-finite light coordinate.
__device__ __forceinline__ bool hit_exact(const float4& L, const float* mn, const float* mx)
{
    const float v[3] = {L.x, L.y, L.z};
    float sq = 0.0f;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        if (v[a] < mn[a]) {
            const float d = __fsub_rn(mn[a], v[a]);
            sq = __fadd_rn(sq, __fmul_rn(d, d));
        } else if (v[a] > mx[a]) {
            const float d = __fsub_rn(mx[a], v[a]);
            sq = __fadd_rn(sq, __fmul_rn(d, d));
        }
    }
    return sq < L.w;
}

template <int K>
struct WarpClusters {
    float mn[K][3];
    float mx[K][3];
    uint32_t cnt[K];
};

// Tests the lights of one shared-memory tile against the warp's K clusters;
// returns true once every cluster of the warp has reached the cap.
template <int K, bool kExact>
__device__ __forceinline__ bool scan_tile(const float4* __restrict__ tile, uint32_t n, uint32_t base, uint32_t lane,
                                          WarpClusters<K>& w, uint32_t cap, uint32_t* __restrict__ staging,
                                          uint32_t cl0, uint32_t clusters)
{
    const uint32_t lt_mask = (1u << lane) - 1u;
    for (uint32_t j = 0; j < n; j += 32) {
        const float4 L = tile[j + lane];
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
                all_capped = all_capped && (w.cnt[k] >= cap || cl0 + k >= clusters);
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

// blockDim = (WARPS + 1) * 32: warps 0..WARPS-1 consume, warp WARPS produces.
// Dynamic shared memory: STAGES x TILE float4, then the full/empty mbarriers,
// the per-stage stop flags and the done-warp counter.
template <int K, int WARPS, int TILE, int STAGES>
__global__ void __launch_bounds__((WARPS + 1) * 32) cull_kernel(const ViewCull v, uint32_t* __restrict__ dev_error)
{
    static_assert(TILE % 32 == 0, "tiles hold whole warps of lights");
    extern __shared__ __align__(128) unsigned char smem[];
    float4* tiles = reinterpret_cast<float4*>(smem);
    uint64_t* full = reinterpret_cast<uint64_t*>(smem + (size_t)STAGES * TILE * sizeof(float4));
    uint64_t* empty = full + STAGES;
    volatile uint32_t* stop = reinterpret_cast<volatile uint32_t*>(empty + STAGES);
    uint32_t* done_warps = reinterpret_cast<uint32_t*>(empty + STAGES) + STAGES;

    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t ntiles = (v.lpad + TILE - 1) / TILE;

    if (threadIdx.x == 0) {
        for (int s = 0; s < STAGES; ++s) {
            mbar_init(smem_u32(&full[s]), 1);
            mbar_init(smem_u32(&empty[s]), WARPS);
            stop[s] = 0;
        }
        *done_warps = 0;
        mbar_init_fence();
    }
    __syncthreads();

    if (warp == WARPS) {
        // Producer: one lane streams the tiles through the ring of stages.
        if (lane == 0) {
            for (uint32_t t = 0; t < ntiles; ++t) {
                const uint32_t s = t % STAGES;
                if (t >= STAGES && !mbar_wait_bounded(smem_u32(&empty[s]), ((t / STAGES) & 1u) ^ 1u)) {
                    atomicOr(dev_error, kErrEmptyWaitTimeout);
                    break;
                }
                if (*reinterpret_cast<volatile uint32_t*>(done_warps) >= (uint32_t)WARPS) {
                    stop[s] = 1;  // every consumer is capped: release them without data
                    mbar_arrive(smem_u32(&full[s]));
                    break;
                }
                stop[s] = 0;
                const uint32_t n = min((uint32_t)TILE, v.lpad - t * TILE);
                mbar_arrive_expect_tx(smem_u32(&full[s]), n * (uint32_t)sizeof(float4));
                bulk_copy_g2s(smem_u32(tiles + (size_t)s * TILE), v.vlights + (size_t)t * TILE,
                              n * (uint32_t)sizeof(float4), smem_u32(&full[s]));
            }
        }
        return;
    }

    // Consumers.
    const uint32_t cl0 = blockIdx.x * (uint32_t)(WARPS * K) + warp * (uint32_t)K;
    WarpClusters<K> w;
    bool done = true;
#pragma unroll
    for (int k = 0; k < K; ++k) {
        w.cnt[k] = 0;
        const uint32_t c = cl0 + k;
        if (c < v.clusters) {
            const float4 a = v.aabbs[2 * (size_t)c];
            const float4 b = v.aabbs[2 * (size_t)c + 1];
            w.mn[k][0] = a.x; w.mn[k][1] = a.y; w.mn[k][2] = a.z;
            w.mx[k][0] = b.x; w.mx[k][1] = b.y; w.mx[k][2] = b.z;
            done = false;
        } else {
            const float inf = __uint_as_float(0x7f800000u);
            for (int a = 0; a < 3; ++a) { w.mn[k][a] = inf; w.mx[k][a] = inf; }
        }
    }
    if (done && lane == 0) atomicAdd(done_warps, 1u);

    for (uint32_t t = 0; t < ntiles; ++t) {
        const uint32_t s = t % STAGES;
        if (!mbar_wait_bounded(smem_u32(&full[s]), (t / STAGES) & 1u)) {
            if (lane == 0) atomicOr(dev_error, kErrFullWaitTimeout);
            break;
        }
        if (stop[s]) break;
        if (!done) {
            const uint32_t base = t * TILE;
            const uint32_t n = min((uint32_t)TILE, v.lpad - base);
            const float4* tile = tiles + (size_t)s * TILE;
            if (!tile_has_nonfinite(v.nonfinite, base, n))
                done = scan_tile<K, false>(tile, n, base, lane, w, v.cap, v.staging, cl0, v.clusters);
            else
                done = scan_tile<K, true>(tile, n, base, lane, w, v.cap, v.staging, cl0, v.clusters);
            if (done && lane == 0) atomicAdd(done_warps, 1u);
        }
        __syncwarp();
        if (lane == 0) mbar_arrive(smem_u32(&empty[s]));
    }

    if (lane == 0) {
#pragma unroll
        for (int k = 0; k < K; ++k)
            if (cl0 + k < v.clusters) v.counts[cl0 + k] = w.cnt[k];
    }
}

// ---------------------------------------------------------------------------
// Finalize: cells = exclusive scan of counts in cluster order, packed copy.
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t warp_sum(uint32_t x)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(kFull, x, o);
    return x;
}

__device__ __forceinline__ uint32_t warp_inclusive_scan(uint32_t x, uint32_t lane)
{
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(kFull, x, o);
        if (lane >= (uint32_t)o) x += y;
    }
    return x;
}

__global__ void __launch_bounds__(1024) finalize_kernel(const ViewCull v)
{
    static_assert(kFinalizeChunk == 2 * 1024, "two clusters per thread");
    __shared__ uint32_t s_off[kFinalizeChunk];
    __shared__ uint32_t s_warp[32];
    __shared__ uint32_t s_base;
    const uint32_t tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const uint32_t c0 = blockIdx.x * kFinalizeChunk;
    const uint32_t C = v.clusters;

    // Sum of the counts of every cluster before this chunk.
    uint32_t acc = 0;
    for (uint32_t i = tid; i < c0; i += 1024) acc += v.counts[i];
    acc = warp_sum(acc);
    if (lane == 0) s_warp[warp] = acc;
    __syncthreads();
    if (warp == 0) {
        const uint32_t x = warp_sum(s_warp[lane]);
        if (lane == 0) s_base = x;
    }
    __syncthreads();
    const uint32_t base = s_base;

    // Exclusive scan of this chunk, two clusters per thread.
    const uint32_t ca = c0 + 2 * tid, cb = ca + 1;
    const uint32_t na = ca < C ? v.counts[ca] : 0u;
    const uint32_t nb = cb < C ? v.counts[cb] : 0u;
    const uint32_t mine = na + nb;
    const uint32_t incl = warp_inclusive_scan(mine, lane);
    if (lane == 31) s_warp[warp] = incl;
    __syncthreads();
    if (warp == 0) s_warp[lane] = warp_inclusive_scan(s_warp[lane], lane);
    __syncthreads();
    const uint32_t off_a = base + (warp ? s_warp[warp - 1] : 0u) + (incl - mine);
    const uint32_t off_b = off_a + na;
    if (ca < C) v.cells[ca] = CfLightCell{off_a, na};
    if (cb < C) v.cells[cb] = CfLightCell{off_b, nb};
    s_off[2 * tid] = off_a;
    s_off[2 * tid + 1] = off_b;
    if (v.total && blockIdx.x == gridDim.x - 1 && tid == 0) *v.total = base + s_warp[31];
    __syncthreads();

    // Packed copy: warp w moves clusters [w*64, w*64+64) of the chunk.
    for (uint32_t q = 0; q < kFinalizeChunk / 32; ++q) {
        const uint32_t local = warp * (kFinalizeChunk / 32) + q;
        const uint32_t c = c0 + local;
        if (c >= C) break;
        const uint32_t n = v.counts[c];
        const uint32_t o = s_off[local];
        const uint32_t* src = v.staging + (size_t)c * v.cap;
        for (uint32_t i = lane; i < n; i += 32) v.indices[o + i] = src[i];
    }
}

template <int K, int WARPS, int TILE, int STAGES>
cudaError_t launch_cull_t(const ViewCull& v, uint32_t* dev_error, cudaStream_t stream)
{
    const size_t smem = (size_t)STAGES * TILE * sizeof(float4) + 2 * STAGES * sizeof(uint64_t) +
                        (STAGES + 1) * sizeof(uint32_t);
    if (smem > 48 * 1024) {  // opt in above the default 48 KB (a per-device attribute)
        const cudaError_t e = cudaFuncSetAttribute(cull_kernel<K, WARPS, TILE, STAGES>,
                                                   cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
    }
    const uint32_t per_cta = (uint32_t)(WARPS * K);
    const uint32_t grid = (v.clusters + per_cta - 1) / per_cta;
    cull_kernel<K, WARPS, TILE, STAGES><<<grid, (WARPS + 1) * 32, smem, stream>>>(v, dev_error);
    return cudaGetLastError();
}

}  // namespace

#define CF_CULL_CONFIGS(X) \
    X(1, 4, 512, 4)        \
    X(2, 4, 512, 4)        \
    X(4, 4, 512, 4)        \
    X(1, 8, 512, 4)        \
    X(2, 8, 512, 4)        \
    X(4, 8, 512, 4)

bool cull_config_supported(const CullConfig& c)
{
#define CF_MATCH(K, W, T, S) \
    if (c.clusters_per_warp == K && c.warps == W && c.tile == T && c.stages == S) return true;
    CF_CULL_CONFIGS(CF_MATCH)
#undef CF_MATCH
    return false;
}

CullConfig default_cull_config(uint32_t clusters, uint32_t lights)
{
    (void)lights;
    if (clusters <= 8192) return CullConfig{1, 8, 512, 4};
    return CullConfig{2, 8, 512, 4};
}

WorkspaceLayout workspace_layout(uint32_t clusters, uint32_t lights, uint32_t cap)
{
    auto al = [](size_t x) { return (x + 255) & ~(size_t)255; };
    WorkspaceLayout w{};
    const uint32_t lpad = pad_lights(lights);
    size_t off = 256;  // status words
    w.vlights = off;
    off += al((size_t)lpad * sizeof(float4));
    w.nonfinite = off;
    off += al((size_t)granules(lpad) * sizeof(uint32_t));
    w.counts = off;
    off += al((size_t)clusters * sizeof(uint32_t));
    w.staging = off;
    off += al((size_t)clusters * cap * sizeof(uint32_t));
    w.bytes = off;
    return w;
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
    light_xform_kernel<<<granules(lpad), kFlagGranule, 0, stream>>>(lights, count, lpad, m, vlights, nonfinite);
    return cudaGetLastError();
}

cudaError_t launch_cull(const ViewCull& v, const CullConfig& cfg, uint32_t* dev_error, cudaStream_t stream)
{
    if (v.clusters == 0) return cudaSuccess;
#define CF_DISPATCH(K, W, T, S)                                                                   \
    if (cfg.clusters_per_warp == K && cfg.warps == W && cfg.tile == T && cfg.stages == S)         \
        return launch_cull_t<K, W, T, S>(v, dev_error, stream);
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
    finalize_kernel<<<(v.clusters + kFinalizeChunk - 1) / kFinalizeChunk, 1024, 0, stream>>>(v);
    return cudaGetLastError();
}

}  // namespace cfk
