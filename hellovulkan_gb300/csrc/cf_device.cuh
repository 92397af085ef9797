// cf_device.cuh — device helpers shared by the culling kernels: bounded-wait
// limits, the global timer, programmatic dependent launch, warp scans, and
// the two forms of LightCulling.comp's sphere-box test.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace cfk {

constexpr unsigned kFull = 0xffffffffu;
constexpr uint64_t kWaitLimitNs = 2000000000ull;  // 2 s per bounded wait
constexpr uint32_t kWaitLimitIters = 1u << 26;

// Test knobs (include/cfcull_testing.h), one copy per translation unit that
// includes this header: the library is built without relocatable device
// code, so each file sets its own with set_test_knobs_*.
//   g_wait_limit_ns  the time limit of every bounded wait (kWaitLimitNs
//                    unless a test shortens it)
//   g_inject_stall   0, or kInject* bits that make one CTA withhold a part
//                    so that the others' bounded waits run out
static __device__ unsigned long long g_wait_limit_ns = kWaitLimitNs;
static __device__ unsigned int g_inject_stall = 0;
constexpr unsigned kInjectOneLaunchSkipPublish = 1u;  // the one-launch kernel's CTA 0 does not publish its total
constexpr unsigned kInjectBruteForceSkipTile = 2u;    // the brute-force kernel's CTA 0 producer never sends tile 0

__device__ __forceinline__ uint64_t global_timer_ns()
{
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Programmatic dependent launch.  The kernels of one view's step are launched
// with programmatic stream serialisation, so each may be scheduled while the
// previous kernel of the stream is still running: it runs only its prologue
// (barrier init, parameters) before grid_dependency_wait(), which returns
// once every earlier kernel of the stream has completed and its writes are
// visible.  launch_dependents() lets the next kernel be scheduled early.
// Both are no-ops in a launch without a programmatic dependency.
__device__ __forceinline__ void grid_dependency_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void launch_dependents() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

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

// ---- packed float pairs ------------------------------------------------------
// sub/mul/add.rn.f32x2: two IEEE binary32 round-to-nearest operations per
// instruction, each the same bits as the scalar one (no contraction).
typedef unsigned long long f2;  // two floats in one 64-bit register pair: (lo, hi)

__device__ __forceinline__ f2 f2_pack(float lo, float hi)
{
    f2 r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(lo), "f"(hi));
    return r;
}
__device__ __forceinline__ void f2_unpack(f2 v, float& lo, float& hi)
{
    asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(v));
}
__device__ __forceinline__ f2 f2_sub(f2 a, f2 b)
{
    f2 r;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}
__device__ __forceinline__ f2 f2_mul(f2 a, f2 b)
{
    f2 r;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}
__device__ __forceinline__ f2 f2_add(f2 a, f2 b)
{
    f2 r;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}

// hit_fast (cf_device.cuh) for two lights against one box at once: light A
// in the low halves, light B in the high halves; the box bounds duplicated
// in both halves.  Each half is exactly hit_fast's arithmetic.
__device__ __forceinline__ void hit_pair(f2 lx, f2 ly, f2 lz, float ar2, float br2, f2 mnx, f2 mny, f2 mnz, f2 mxx,
                                         f2 mxy, f2 mxz, bool& ha, bool& hb)
{
    float a0, a1, b0, b1;
    f2_unpack(f2_sub(mnx, lx), a0, a1);
    f2_unpack(f2_sub(lx, mxx), b0, b1);
    const f2 dx = f2_pack(max3f(a0, b0, 0.0f), max3f(a1, b1, 0.0f));
    f2_unpack(f2_sub(mny, ly), a0, a1);
    f2_unpack(f2_sub(ly, mxy), b0, b1);
    const f2 dy = f2_pack(max3f(a0, b0, 0.0f), max3f(a1, b1, 0.0f));
    f2_unpack(f2_sub(mnz, lz), a0, a1);
    f2_unpack(f2_sub(lz, mxz), b0, b1);
    const f2 dz = f2_pack(max3f(a0, b0, 0.0f), max3f(a1, b1, 0.0f));
    const f2 sq = f2_add(f2_add(f2_mul(dx, dx), f2_mul(dy, dy)), f2_mul(dz, dz));
    float sa, sb;
    f2_unpack(sq, sa, sb);
    ha = sa < ar2;
    hb = sb < br2;
}

}  // namespace cfk
