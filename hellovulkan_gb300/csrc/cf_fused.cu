// cf_fused.cu — one-launch culling of a small view (LightCulling.comp:26-87).
//
// A view with at most kOneLaunchMaxLights lights (the 1920x1080 16x9x24 view
// with 1024 lights, say) is culled by one kernel: no light-transform, copy or
// scan launch, no staging rows, no launch gaps.
//
//   1. CTA b owns clusters [b*M, (b+1)*M) (M <= 32): their AABBs go to shared
//      memory, each bound stored twice so that a 64-bit load yields the pair
//      a packed instruction wants.
//   2. The CTA's W*S warps form S sets of W: warp w of a set owns light chunks
//      [w*J, (w+1)*J) of 32 lights each; every lane transforms its J lights
//      itself, two per packed operation (posView = cameraView * position in
//      the pinned order, r^2), and keeps them in registers.
//   3. Set s tests its chunks against boxes s, s+S, ... of the CTA, two
//      chunks per packed instruction (sub/mul/add.rn.f32x2: two IEEE
//      round-to-nearest operations each, the same bits as the scalar ones),
//      and stores each test's 32 results as one __ballot_sync mask:
//      mask[m][chunk].  A chunk holding a non-finite light coordinate takes
//      the shader's branchy test.
//   4. Cluster m's list is its masks' set bits in chunk order: a warp scan of
//      the popcounts gives every chunk's first position, capped at `cap` —
//      the first `cap` hits in ascending light order, as the shader keeps.
//   5. The CTA's capped total goes to partials[b] tagged with this launch's
//      epoch; each CTA sums the totals of the CTAs before it (reduce then
//      scan, every read in flight at once) to get its offset in the packed
//      list, which is the cluster-order exclusive scan the oracle computes.
//      The kernel is a cooperative launch, so every CTA a CTA waits for is
//      resident.
//   6. Cells and indices are written straight to the outputs.
// Every test of the view runs (no early stop at the cap): a small view's
// tests cost less than the bookkeeping would.
#include "cf_kernels.cuh"
#include "cf_device.cuh"

#include <atomic>

#include "cf_pinned_math.h"

namespace cfk {
namespace {

__device__ __forceinline__ void st_relaxed_gpu(unsigned long long* p, unsigned long long v)
{
    asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ unsigned long long ld_relaxed_gpu(const unsigned long long* p)
{
    unsigned long long v;
    asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}

// Predecessor totals a lane reads at most: kOneLaunchMaxCtas / 32.
constexpr int kLookSlots = (int)(kOneLaunchMaxCtas / 32);
// The CTAs publish within a fraction of a microsecond of each other, so a
// poll right after a CTA's own publish mostly finds the earlier CTAs' old
// words, and the polling traffic slows their stores: the first poll waits
// about one L2 round trip, later ones a little less.  (On a GB300 this took
// the wait from about 2.6 to 0.9 us on the 1920x1080 view.)
constexpr unsigned kFirstPollDelayNs = 300, kRepollDelayNs = 100;

// W warps per set, J chunks of 32 lights per warp, S sets splitting the boxes.
template <int W, int J, int S>
__global__ void __launch_bounds__(W * S * 32) one_launch_kernel(const FusedCull f, uint32_t* __restrict__ dev_error)
{
    static_assert(J % 2 == 0, "chunks are tested in pairs");
    constexpr int NW = W * S;                      // warps of the CTA
    constexpr int NCH = W * J;                     // chunk slots of the CTA
    constexpr int CPL = (NCH + 31) / 32;           // chunks per lane in the per-cluster scan
    constexpr int MPW = (int)(kOneLaunchMaxClustersPerCta + NW - 1) / NW;  // clusters per warp in the scan
    constexpr uint32_t kM = kOneLaunchMaxClustersPerCta;
    __shared__ __align__(16) f2 s_box[kM * 6];    // per cluster: mn.x, mn.y, mn.z, mx.x, mx.y, mx.z, each (v, v)
    __shared__ __align__(16) uint32_t s_mask[kM * NCH];
    __shared__ uint32_t s_cnt[kM], s_excl[kM];
    __shared__ uint32_t s_tag, s_base, s_ok;

    const uint32_t tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const uint32_t cw = warp % W, set = warp / W;  // chunk group and box set of this warp
    const uint32_t b = blockIdx.x, M = f.per_cta, c0 = b * M;
    const uint32_t Mb = min(M, f.clusters - c0);
    const uint32_t nch = (f.light_count + 31) / 32;
    const float inf = __uint_as_float(0x7f800000u);

    if (tid == 0) s_tag = *reinterpret_cast<volatile uint32_t*>(f.epoch) + 1u;
    if (tid < 2 * kM) {  // thread 2m + h: bound h (0 = min, 1 = max) of cluster m
        const uint32_t m = tid >> 1, h = tid & 1;
        float4 q = make_float4(inf, inf, inf, 0.0f);  // past the view: never hit
        if (m < Mb) q = __ldg(&f.aabbs[2 * (size_t)(c0 + m) + h]);
        s_box[m * 6 + 3 * h + 0] = f2_pack(q.x, q.x);
        s_box[m * 6 + 3 * h + 1] = f2_pack(q.y, q.y);
        s_box[m * 6 + 3 * h + 2] = f2_pack(q.z, q.z);
    }
    // This warp's lights in view space, in registers: chunk cw*J + j, lane.
    // Chunks 2q and 2q+1 are transformed together, one light per half of
    // each packed operation (cameraView * position in the pinned order).
    float lxs[J], lys[J], lzs[J], lr2[J];
    uint32_t bad = 0;  // bit j: chunk j holds a non-finite coordinate
#pragma unroll
    for (int q = 0; q < J / 2; ++q) {
        float4 pa = make_float4(0.0f, 0.0f, 0.0f, 0.0f), pb = pa;
        float ra = 0.0f, rb = 0.0f;
        const uint32_t ia = (cw * J + 2 * q) * 32 + lane, ib = ia + 32;
        if (ia < f.light_count) {
            pa = __ldg(reinterpret_cast<const float4*>(&f.lights[ia].position[0]));
            ra = __ldg(&f.lights[ia].radius);
        }
        if (ib < f.light_count) {
            pb = __ldg(reinterpret_cast<const float4*>(&f.lights[ib].position[0]));
            rb = __ldg(&f.lights[ib].radius);
        }
        const f2 px = f2_pack(pa.x, pb.x), py = f2_pack(pa.y, pb.y), pz = f2_pack(pa.z, pb.z), pw = f2_pack(pa.w, pb.w);
        float v[3][2];
#pragma unroll
        for (int row = 0; row < 3; ++row) {  // ((m[row]*x + m[4+row]*y) + m[8+row]*z) + m[12+row]*w
            const float* m = f.view;
            f2 acc = f2_add(f2_mul(f2_pack(m[row], m[row]), px), f2_mul(f2_pack(m[4 + row], m[4 + row]), py));
            acc = f2_add(acc, f2_mul(f2_pack(m[8 + row], m[8 + row]), pz));
            acc = f2_add(acc, f2_mul(f2_pack(m[12 + row], m[12 + row]), pw));
            f2_unpack(acc, v[row][0], v[row][1]);
        }
        float r2a, r2b;
        f2_unpack(f2_mul(f2_pack(ra, rb), f2_pack(ra, rb)), r2a, r2b);
        const uint32_t idx[2] = {ia, ib};
        const float r2[2] = {r2a, r2b};
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int j = 2 * q + h;
            bool nf = false;
            if (idx[h] < f.light_count) {
                lxs[j] = v[0][h];
                lys[j] = v[1][h];
                lzs[j] = v[2][h];
                lr2[j] = r2[h];
                // non-finite x, y or z makes the sum non-finite (an
                // overflowing sum of finite values only sends the chunk to
                // the exact test, which gives the same answer)
                nf = !finite_bits(__fadd_rn(__fadd_rn(lxs[j], lys[j]), lzs[j]));
            } else {  // pad: r^2 = -inf fails every test
                lxs[j] = lys[j] = lzs[j] = 0.0f;
                lr2[j] = __uint_as_float(0xff800000u);
            }
            if (__any_sync(kFull, nf)) bad |= 1u << j;
        }
    }
    __syncthreads();

    // Tests: mask[m][chunk] = ballot of the chunk's 32 lights against box m.
    if (cw * J < nch) {
        f2 px[J / 2], py[J / 2], pz[J / 2];
#pragma unroll
        for (int q = 0; q < J / 2; ++q) {
            px[q] = f2_pack(lxs[2 * q], lxs[2 * q + 1]);
            py[q] = f2_pack(lys[2 * q], lys[2 * q + 1]);
            pz[q] = f2_pack(lzs[2 * q], lzs[2 * q + 1]);
        }
        uint32_t* mrow = s_mask + cw * J;
#pragma unroll 2
        for (uint32_t m = set; m < Mb; m += S) {
            const f2* bx = s_box + m * 6;
            const f2 mnx = bx[0], mny = bx[1], mnz = bx[2], mxx = bx[3], mxy = bx[4], mxz = bx[5];
            uint32_t masks[J];
#pragma unroll
            for (int q = 0; q < J / 2; ++q) {
                bool ha, hb;
                if (!(bad & (3u << (2 * q)))) {
                    hit_pair(px[q], py[q], pz[q], lr2[2 * q], lr2[2 * q + 1], mnx, mny, mnz, mxx, mxy, mxz, ha, hb);
                } else {
                    float t0, t1;
                    float mn[3], mx[3];
                    f2_unpack(mnx, mn[0], t0);
                    f2_unpack(mny, mn[1], t0);
                    f2_unpack(mnz, mn[2], t0);
                    f2_unpack(mxx, mx[0], t1);
                    f2_unpack(mxy, mx[1], t1);
                    f2_unpack(mxz, mx[2], t1);
                    ha = hit_exact(make_float4(lxs[2 * q], lys[2 * q], lzs[2 * q], lr2[2 * q]), mn, mx);
                    hb = hit_exact(make_float4(lxs[2 * q + 1], lys[2 * q + 1], lzs[2 * q + 1], lr2[2 * q + 1]), mn, mx);
                }
                masks[2 * q] = __ballot_sync(kFull, ha);
                masks[2 * q + 1] = __ballot_sync(kFull, hb);
            }
            if (lane == 0) {
                uint32_t* dst = mrow + m * NCH;
                if constexpr (J == 2) {
                    *reinterpret_cast<uint2*>(dst) = make_uint2(masks[0], masks[1]);
                } else {
#pragma unroll
                    for (int q = 0; q < J; q += 4)
                        *reinterpret_cast<uint4*>(dst + q) = make_uint4(masks[q], masks[q + 1], masks[q + 2], masks[q + 3]);
                }
            }
        }
    }
    __syncthreads();

    // Per cluster: lane l scans chunks [l*CPL, (l+1)*CPL) of its masks.
    uint32_t mk[MPW][CPL];
    uint32_t ex[MPW];
#pragma unroll
    for (int q = 0; q < MPW; ++q) {
        const uint32_t m = warp + q * NW;
        ex[q] = 0;
#pragma unroll
        for (int u = 0; u < CPL; ++u) mk[q][u] = 0;
        if (m < Mb) {  // warp-uniform
            uint32_t c = 0;
#pragma unroll
            for (int u = 0; u < CPL; ++u) {
                const uint32_t ch = lane * CPL + u;
                mk[q][u] = ch < nch ? s_mask[m * NCH + ch] : 0u;
                c += __popc(mk[q][u]);
            }
            const uint32_t incl = warp_inclusive_scan(c, lane);
            ex[q] = incl - c;
            if (lane == 31) s_cnt[m] = min(incl, f.cap);
        }
    }
    __syncthreads();

    // The CTA's offsets and total; publish, then the sum of earlier CTAs'
    // totals.  Each word carries its own total, so relaxed accesses suffice:
    // nothing else written by another CTA is read here.
    if (warp == 0) {
        const uint32_t c = lane < Mb ? s_cnt[lane] : 0u;
        const uint32_t incl = warp_inclusive_scan(c, lane);
        s_excl[lane] = incl - c;
        const uint32_t total = __shfl_sync(kFull, incl, 31);
        const uint32_t tag = s_tag;
        // (a test may make CTA 0 withhold its total: the other CTAs' waits run out)
        const bool withhold = b == 0 && (g_inject_stall & kInjectOneLaunchSkipPublish);
        if (lane == 0 && !withhold) st_relaxed_gpu(&f.partials[b], ((unsigned long long)tag << 32) | total);
        uint32_t pending = 0, acc = 0;
#pragma unroll
        for (int k = 0; k < kLookSlots; ++k)
            if (lane + 32u * k < b) pending |= 1u << k;
        bool ok = true;
        if (__any_sync(kFull, pending != 0)) {
            __nanosleep(kFirstPollDelayNs);
            const uint64_t t0 = global_timer_ns();
            for (uint32_t it = 0; it < kWaitLimitIters; ++it) {
                unsigned long long w[kLookSlots];
#pragma unroll
                for (int k = 0; k < kLookSlots; ++k)  // every read in flight at once
                    w[k] = (pending >> k) & 1u ? ld_relaxed_gpu(&f.partials[lane + 32u * k]) : 0ull;
#pragma unroll
                for (int k = 0; k < kLookSlots; ++k)
                    if (((pending >> k) & 1u) && (uint32_t)(w[k] >> 32) == tag) {
                        acc += (uint32_t)w[k];
                        pending &= ~(1u << k);
                    }
                if (!__any_sync(kFull, pending != 0)) break;
                if (global_timer_ns() - t0 > g_wait_limit_ns) {
                    ok = false;
                    break;
                }
                __nanosleep(kRepollDelayNs);
            }
            ok = __all_sync(kFull, ok && pending == 0);
        }
        const uint32_t base = warp_sum(acc);
        if (lane == 0) {
            s_base = base;
            s_ok = ok ? 1u : 0u;
            if (!ok) atomicOr(dev_error, kErrLookbackTimeout);
            if (b == gridDim.x - 1) {
                if (ok && f.total) *f.total = base + total;
                // every CTA read the epoch before it published, and this CTA
                // has seen every publish (or gave up after its bounded wait):
                // the epoch is not read again in this launch.  (Had a CTA read
                // the new value, its tag would match no other CTA's and the
                // waits would time out: no silent mix of launches.)
                *reinterpret_cast<volatile uint32_t*>(f.epoch) = tag;
            }
            if (f.work && b == 0) atomicAdd(&f.work[1], (unsigned long long)f.clusters * f.light_count);
        }
    }
    __syncthreads();
    if (!s_ok) return;  // the outputs are left as they were; the error word says why
    const uint32_t base = s_base;
    if (warp == 0 && lane < Mb) f.cells[c0 + lane] = CfLightCell{base + s_excl[lane], s_cnt[lane]};
#pragma unroll
    for (int q = 0; q < MPW; ++q) {
        const uint32_t m = warp + q * NW;
        if (m < Mb) {
            const uint32_t first = base + s_excl[m];
            const uint32_t lim = first + s_cnt[m];
            uint32_t pos = first + ex[q];
#pragma unroll
            for (int u = 0; u < CPL; ++u) {
                uint32_t bits = mk[q][u];
                const uint32_t ch = lane * CPL + u;
                while (bits && pos < lim) {
                    const uint32_t bit = __ffs(bits) - 1;
                    bits &= bits - 1;
                    f.indices[pos++] = ch * 32 + bit;
                }
            }
        }
    }
}

// (warps per set, chunks per warp, sets) of each compiled shape: W*S warps
// per CTA, most lights = 32 * W * J.
#define CF_ONE_LAUNCH_SHAPES(X) \
    X(16, 2, 2)                 \
    X(16, 4, 1)                 \
    X(16, 2, 1)

constexpr int kMaxDevices = 64;

// Resident CTAs of shape (W, J) on the current device, queried once per
// device (every launch asks, so the answer is cached; concurrent first
// queries store the same value).
template <int W, int J, int S>
cudaError_t resident_t(int* ctas)
{
    static std::atomic<int> cache[kMaxDevices];
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev >= 0 && dev < kMaxDevices) {
        const int c = cache[dev].load(std::memory_order_relaxed);
        if (c > 0) {
            *ctas = c;
            return cudaSuccess;
        }
    }
    int sms = 0, per_sm = 0;
    e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, one_launch_kernel<W, J, S>, W * S * 32, 0);
    *ctas = e == cudaSuccess ? sms * per_sm : 0;
    if (*ctas > 0 && dev >= 0 && dev < kMaxDevices) cache[dev].store(*ctas, std::memory_order_relaxed);
    return e;
}

int sm_count()
{
    static std::atomic<int> cache[kMaxDevices];
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return 0;
    int n = cache[dev].load(std::memory_order_relaxed);
    if (n <= 0 && cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) == cudaSuccess && n > 0)
        cache[dev].store(n, std::memory_order_relaxed);
    return n;
}

}  // namespace

bool one_launch_shape_supported(int warps, int max_lights)
{
#define CF_MATCH(W, J, S) \
    if (warps == W * S && max_lights == 32 * W * J) return true;
    CF_ONE_LAUNCH_SHAPES(CF_MATCH)
#undef CF_MATCH
    return false;
}

cudaError_t one_launch_resident_ctas(int warps, int max_lights, int* ctas)
{
    *ctas = 0;
#define CF_MATCH(W, J, S) \
    if (warps == W * S && max_lights == 32 * W * J) return resident_t<W, J, S>(ctas);
    CF_ONE_LAUNCH_SHAPES(CF_MATCH)
#undef CF_MATCH
    return cudaErrorInvalidValue;
}

// One CTA per SM — 32 warps for up to 1024 lights, 16 warps for up to 2048;
// M = clusters spread over the SMs.  Views whose M would pass
// kOneLaunchMaxClustersPerCta, or whose CTAs could not all be resident at
// once (a cooperative launch needs that), take the other modes.
bool one_launch_config(uint32_t clusters, uint32_t lights, CullConfig* cfg)
{
    if (lights > kOneLaunchMaxLights || clusters == 0) return false;
    const int warps = lights <= 1024 ? 32 : 16, max_lights = lights <= 1024 ? 1024 : 2048;
    const int sms = sm_count();
    if (sms <= 0) return false;
    const uint32_t per_cta = (clusters + (uint32_t)sms - 1) / (uint32_t)sms;
    if (per_cta > kOneLaunchMaxClustersPerCta) return false;
    const uint32_t ctas = (clusters + per_cta - 1) / per_cta;
    int resident = 0;
    if (one_launch_resident_ctas(warps, max_lights, &resident) != cudaSuccess || ctas > (uint32_t)resident ||
        ctas > kOneLaunchMaxCtas)
        return false;
    *cfg = CullConfig{(int)per_cta, warps, max_lights, 1, kModeOneLaunch};
    return true;
}

cudaError_t set_test_knobs_one_launch(uint64_t wait_limit_ns, uint32_t inject)
{
    const unsigned long long w = wait_limit_ns;
    const unsigned int i = inject;
    cudaError_t e = cudaMemcpyToSymbol(g_wait_limit_ns, &w, sizeof(w));
    if (e == cudaSuccess) e = cudaMemcpyToSymbol(g_inject_stall, &i, sizeof(i));
    return e;
}

cudaError_t launch_one_launch(const FusedCull& f, int warps, int max_lights, uint32_t* dev_error, cudaStream_t stream)
{
    if (f.clusters == 0) return f.total ? cudaMemsetAsync(f.total, 0, sizeof(uint32_t), stream) : cudaSuccess;
    if (f.per_cta == 0 || f.per_cta > kOneLaunchMaxClustersPerCta || f.light_count > (uint32_t)max_lights ||
        f.ctas != (f.clusters + f.per_cta - 1) / f.per_cta || f.ctas > kOneLaunchMaxCtas)
        return cudaErrorInvalidValue;
    int resident = 0;
    cudaError_t e = one_launch_resident_ctas(warps, max_lights, &resident);
    if (e != cudaSuccess) return e;
    if (f.ctas > (uint32_t)resident) return cudaErrorCooperativeLaunchTooLarge;
    // cooperative: every CTA is resident at once, so a CTA may wait for the
    // totals of the CTAs before it
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = dim3(f.ctas);
    cfg.blockDim = dim3(warps * 32);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = stream;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
#define CF_LAUNCH(W, J, S)                                 \
    if (warps == W * S && max_lights == 32 * W * J)        \
        return cudaLaunchKernelEx(&cfg, one_launch_kernel<W, J, S>, f, dev_error);
    CF_ONE_LAUNCH_SHAPES(CF_LAUNCH)
#undef CF_LAUNCH
    return cudaErrorInvalidValue;
}

}  // namespace cfk
