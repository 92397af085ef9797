// cf_server.cpp — a culling server with continuous batching.
//
// Requests (a view's UBO + the id of a light set resident on the device) are
// submitted from any thread and admitted in arrival order by one worker
// thread.  Admission takes device memory for the request's scratch and
// outputs from one arena whose size is the server's HBM budget; light sets
// and the AABBs of each distinct projection live in the same arena and are
// evicted least-recently-used when admission needs room (never while a
// request in flight uses them).  Whenever one of the server's streams is
// free, every admissible pending request (up to max_batch_views) is launched
// there as one batch — so requests that arrive while earlier batches are
// still on the GPU start on another stream and overlap with them.  A host
// callback on the stream timestamps the batch's completion.
//
// Light-set updates are copy-on-write: requests already admitted keep the
// version they were admitted with, so a result never depends on what else is
// in flight.  The same request gives the same bits alone and in any mix.
//
// The reference has no counterpart (its one view per frame is recorded by
// AppBase::DrawFrame, Source/Apps/AppBase.cpp:94-196).
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <new>
#include <shared_mutex>
#include <thread>
#include <vector>

#include <unistd.h>

#include "cf_arena.h"
#include "cf_batch_internal.h"
#include "cf_kernels.cuh"
#include "cf_runtime_internal.h"
#include "cfcull.h"

using namespace cfrt;

namespace {

double now_s()
{
    using namespace std::chrono;
    return duration<double>(steady_clock::now().time_since_epoch()).count();
}

// Takes the server lock, trying for a few microseconds before sleeping: its
// critical sections last about a microsecond, less than a sleeping thread
// needs to be woken, and at 100 000 requests/s clients and the worker take it
// several hundred thousand times a second.
constexpr int kLockSpins = 256;
void spin_lock(std::mutex& m)
{
    for (int i = 0; i < kLockSpins; ++i)
        if (m.try_lock()) return;
    m.lock();
}
std::unique_lock<std::mutex> take_lock(std::mutex& m)
{
    spin_lock(m);
    return std::unique_lock<std::mutex>(m, std::adopt_lock);
}

// One version of a light set.  Every fill (host upload or jitter) is
// enqueued on the server's single upload stream, so fills run in the order
// they were enqueued, and a batch orders itself after all of them by waiting
// on a fence recorded on the upload stream when it is launched.  A version's
// memory may therefore go back to the arena as soon as no admitted request
// references it: a later fill reuses it behind the earlier ones on the same
// stream, and a later batch reuses it behind its fence.
struct LightVersion {
    unsigned char* d = nullptr;
    uint32_t count = 0;
    uint32_t refs = 0;
    bool retired = false;
    bool failed = false;  // its queued upload or jitter failed to launch: requests bound to it fail
};

// Work that writes a new version, waiting for the worker: a jitter of `src`,
// or (src null) a copy from `host`, pinned host memory the device reads
// directly.  Both versions are held by a reference until the launch is
// enqueued, after which the upload stream's order protects them like any
// fill.  `host` must stay unchanged until the first request that uses the
// version has completed, as for a copy from pinned memory.
struct VersionJob {
    LightVersion* dst;
    LightVersion* src;
    const void* host;
    uint64_t seed;
    float sigma;
};

// A host range the client declared pinned for the server's lifetime
// (cf_server_declare_pinned_host): [begin, end) on the host, read by the
// device at dev + (address - begin).
struct PinnedRange {
    uintptr_t begin, end, dev;
};

struct LightSet {
    LightVersion* cur = nullptr;
    uint64_t last_use = 0;
};

struct AabbEntry {
    CfClusterForwardUBO key{};
    unsigned char* d = nullptr;
    uint32_t refs = 0;
    bool generated = false;  // its generation has been enqueued
    bool complete = false;   // a batch that used it has finished, so it is in memory
    cudaEvent_t ready = nullptr;
    uint64_t last_use = 0;
};

struct Request {
    uint64_t id = 0;
    CfServerRequest req{};
    double t_submit = 0, t_launch = 0, t_complete = 0;
    LightVersion* lights = nullptr;
    AabbEntry* aabb = nullptr;
    unsigned char* ws = nullptr;
    unsigned char* out = nullptr;
    uint32_t clusters = 0, groups = 0;
    cfk::CullConfig cfg{};
    cfk::WorkspaceLayout layout{};
    int status = CF_SUCCESS;
};

struct Batch;

// The tables of one batch, in one pinned host block mirrored by one device
// block so that they go over in a single copy: the ViewJob records, the three
// block-prefix arrays, then the (view, group) work items, each section
// 256-byte aligned.
struct TableLayout {
    size_t jobs = 0, prefix = 0, items = 0, bytes = 0;
};

TableLayout table_layout(uint32_t views, uint32_t items)
{
    auto al = [](size_t x) { return (x + 255) & ~(size_t)255; };
    TableLayout t;
    t.prefix = al((size_t)views * sizeof(cfk::ViewJob));
    t.items = t.prefix + al((size_t)views * 3 * sizeof(uint32_t));
    t.bytes = t.items + al((size_t)items * sizeof(uint2));
    return t;
}

struct StreamSlot {
    cudaStream_t s = nullptr;
    bool busy = false;
    unsigned char* d_tables = nullptr;
    unsigned char* h_tables = nullptr;
    uint32_t* d_queues = nullptr;
    cudaEvent_t upload_fence = nullptr;  // recorded on the upload stream at each launch
};

// What a launch needs once the tables are written (everything but the CUDA
// calls is done with the server lock held; the calls themselves are not).
struct LaunchPlan {
    struct Bucket {
        cfk::CullConfig cfg;
        uint32_t begin, count;
    };
    std::vector<Bucket> buckets;
    std::vector<AabbEntry*> generate;  // AABBs this batch generates
    std::vector<AabbEntry*> wait;      // AABBs generated by batches that may still run
    TableLayout tables;
    uint32_t views = 0, items = 0, xform_blocks = 0, bin_blocks = 0, copy_blocks = 0;
};

struct Batch {
    CfServer* server = nullptr;
    int slot = 0;
    std::vector<Request*> reqs;
    double t_done = 0;
};

size_t output_bytes(uint32_t clusters, uint32_t cap)
{
    const size_t cells = ((size_t)clusters * sizeof(CfLightCell) + 255) & ~(size_t)255;
    const size_t idx = ((size_t)clusters * cap * sizeof(uint32_t) + 255) & ~(size_t)255;
    return cells + idx + 256;
}

void out_pointers(unsigned char* out, uint32_t clusters, uint32_t cap, CfLightCell** cells, uint32_t** idx,
                  uint32_t** total)
{
    const size_t cb = ((size_t)clusters * sizeof(CfLightCell) + 255) & ~(size_t)255;
    const size_t ib = ((size_t)clusters * cap * sizeof(uint32_t) + 255) & ~(size_t)255;
    *cells = reinterpret_cast<CfLightCell*>(out);
    *idx = reinterpret_cast<uint32_t*>(out + cb);
    *total = reinterpret_cast<uint32_t*>(out + cb + ib);
}

}  // namespace

struct CfServer {
    CfContext* ctx = nullptr;
    int device = 0;
    uint32_t* dev_error = nullptr;
    CfServerConfig cfg{};
    unsigned char* d_pool = nullptr;
    Arena arena;
    std::mutex mu;
    std::condition_variable cv, done_cv;
    std::deque<Request*> pending;
    std::vector<VersionJob> jobs;  // queued uploads and jitters, launched before the next batch
    // declared pinned host ranges, sorted and disjoint; read on every register
    // and update, written only by declarations, so behind their own lock
    std::shared_mutex pinned_mu;
    std::vector<PinnedRange> pinned;
    std::vector<StreamSlot> slots;
    std::map<uint64_t, LightSet> sets;
    std::vector<AabbEntry*> aabbs;
    std::map<uint64_t, Request*> holding;  // completed, outputs not yet released
    std::deque<CfServerCompletion> completions;
    // Finished batches, handed over by the stream host callback.  The callback
    // takes only done_mu (never `mu`), so no thread holding `mu` can ever wait
    // on a callback that waits on it.
    std::mutex done_mu;
    std::deque<Batch*> finished;
    std::atomic<uint32_t> finished_n{0};
    std::map<uint32_t, cfk::CullConfig> tuned;
    std::thread worker;
    bool stop = false;
    bool waiting_for_memory = false;  // the worker sleeps until memory returns to the arena
    cudaStream_t upload = nullptr;
    uint64_t next_set = 1, next_req = 1, tick = 0;
    uint64_t memory_epoch = 0;  // bumped whenever device memory returns to the arena
    uint32_t items_per_slot = 0;
    CfServerStats stats{};
    double t0 = 0;
};

namespace {

cfk::CullConfig server_config_for(const CfServer* s, uint32_t xy)
{
    auto it = s->tuned.find(xy);
    if (it != s->tuned.end()) return it->second;
    // what the batch autotuner picks for the served mix's four grids on a GB300
    if (xy <= 64) return cfk::CullConfig{2, 4, 512, 2, 1};
    if (xy <= 144) return cfk::CullConfig{4, 4, 512, 2, 1};
    return cfk::CullConfig{4, 8, 1024, 2, 1};
}

void free_version_if_dead(CfServer* s, LightVersion* v)
{
    if (v && v->retired && v->refs == 0) {
        s->arena.release(v->d);
        delete v;
    }
}

// Frees the least recently used light set or AABB entry nobody in flight
// uses; false when there is none.
bool evict_one(CfServer* s)
{
    uint64_t best = UINT64_MAX;
    int kind = -1;
    uint64_t set_id = 0;
    size_t aabb_i = 0;
    for (auto& kv : s->sets)
        if (kv.second.cur->refs == 0 && kv.second.last_use < best) {
            best = kv.second.last_use;
            kind = 0;
            set_id = kv.first;
        }
    for (size_t i = 0; i < s->aabbs.size(); ++i)
        if (s->aabbs[i]->refs == 0 && s->aabbs[i]->last_use < best) {
            best = s->aabbs[i]->last_use;
            kind = 1;
            aabb_i = i;
        }
    if (kind == 0) {
        LightVersion* v = s->sets[set_id].cur;
        v->retired = true;
        free_version_if_dead(s, v);
        s->sets.erase(set_id);
        s->stats.evictions++;
        return true;
    }
    if (kind == 1) {
        AabbEntry* a = s->aabbs[aabb_i];
        s->arena.release(a->d);
        if (a->ready) cudaEventDestroy(a->ready);
        delete a;
        s->aabbs.erase(s->aabbs.begin() + (long)aabb_i);
        s->stats.evictions++;
        return true;
    }
    return false;
}

unsigned char* arena_alloc(CfServer* s, size_t bytes)
{
    for (;;) {
        unsigned char* p = s->arena.alloc(bytes);
        if (p) {
            s->stats.arena_peak_bytes = std::max<uint64_t>(s->stats.arena_peak_bytes, s->arena.used());
            return p;
        }
        if (!evict_one(s)) return nullptr;
    }
}

void complete_request(CfServer* s, Request* r, int status)
{
    CfServerCompletion c{};
    c.request_id = r->id;
    c.user_tag = r->req.user_tag;
    c.status = status;
    c.t_submit = r->t_submit - s->t0;
    c.t_launch = r->t_launch ? r->t_launch - s->t0 : 0;
    c.t_complete = r->t_complete - s->t0;
    c.clusters = r->clusters;
    if (status == CF_SUCCESS) {
        CfLightCell* cells;
        uint32_t *idx, *total;
        out_pointers(r->out, r->clusters, r->req.max_lights_per_cluster, &cells, &idx, &total);
        c.d_cells = cells;
        c.d_indices = idx;
        c.d_total = total;
        s->holding[r->id] = r;
        s->stats.max_held_outputs = std::max<uint32_t>(s->stats.max_held_outputs, (uint32_t)s->holding.size());
    } else {
        s->arena.release(r->out);
        delete r;
    }
    s->completions.push_back(c);
    s->stats.completed++;  // pollers are woken once per worker pass (worker_main)
}

// Takes what request r needs; false (nothing taken) when the arena is full.
bool admit(CfServer* s, Request* r)
{
    const CfClusterForwardUBO& u = r->req.ubo;
    LightVersion* lv = r->lights;  // bound (and referenced) at submission
    if (lv->failed) {
        r->status = CF_ERROR_CUDA;  // its lights were never written
        return true;
    }
    const uint32_t xy = u.sliceCountX * u.sliceCountY, Z = u.sliceCountZ;
    r->cfg = server_config_for(s, xy);
    const uint32_t groups = cfk::group_count(r->clusters, xy, Z, (uint32_t)(r->cfg.warps * r->cfg.clusters_per_warp), true);
    if (groups > s->cfg.max_groups_per_view) {
        r->status = CF_ERROR_CAPACITY;
        return true;
    }
    r->groups = groups;
    r->layout = cfk::workspace_layout(r->clusters, lv->count, r->req.max_lights_per_cluster, Z, true, groups);
    AabbEntry* a = nullptr;
    for (AabbEntry* e : s->aabbs)
        if (projection_equal(e->key, u)) a = e;
    bool new_aabb = false;
    if (a) {
        a->refs++;  // the AABBs may not be evicted by the allocations below
    } else {
        a = new AabbEntry();
        a->key = u;
        a->d = arena_alloc(s, (size_t)r->clusters * sizeof(CfAABB));
        if (a->d && cudaEventCreateWithFlags(&a->ready, cudaEventDisableTiming) != cudaSuccess) {
            s->arena.release(a->d);
            a->d = nullptr;
            a->ready = nullptr;
        }
        if (!a->d) {
            delete a;
            return false;
        }
        a->refs = 1;
        s->aabbs.push_back(a);
        new_aabb = true;
    }
    r->ws = arena_alloc(s, r->layout.bytes);
    r->out = r->ws ? arena_alloc(s, output_bytes(r->clusters, r->req.max_lights_per_cluster)) : nullptr;
    if (!r->ws || !r->out) {
        s->arena.release(r->ws);
        r->ws = nullptr;
        a->refs--;
        if (new_aabb) {
            s->arena.release(a->d);
            cudaEventDestroy(a->ready);
            s->aabbs.erase(std::find(s->aabbs.begin(), s->aabbs.end(), a));
            delete a;
        }
        return false;
    }
    r->aabb = a;
    auto it = s->sets.find(r->req.light_set);
    if (it != s->sets.end()) it->second.last_use = ++s->tick;
    a->last_use = ++s->tick;
    return true;
}

void CUDART_CB on_batch_done(void* data)
{
    Batch* b = static_cast<Batch*>(data);
    b->t_done = now_s();
    CfServer* s = b->server;
    {
        std::lock_guard<std::mutex> lk(s->done_mu);
        s->finished.push_back(b);
    }
    s->finished_n.fetch_add(1);
    s->cv.notify_all();
}

// Moves the batches the callbacks finished into `out` (called with `mu` held).
void take_finished(CfServer* s, std::deque<Batch*>& out)
{
    std::lock_guard<std::mutex> lk(s->done_mu);
    out.swap(s->finished);
    s->finished_n.fetch_sub((uint32_t)out.size());
}

// Decides which AABB entries the batch generates and which it waits for
// (`mu` held: the entries' flags are shared with other batches).
void plan_batch(const std::vector<Request*>& reqs, LaunchPlan& plan)
{
    plan = LaunchPlan{};
    plan.views = (uint32_t)reqs.size();
    for (Request* r : reqs) {
        AabbEntry* a = r->aabb;
        if (!a->generated) {
            a->generated = true;
            plan.generate.push_back(a);
        } else if (!a->complete && std::find(plan.wait.begin(), plan.wait.end(), a) == plan.wait.end() &&
                   std::find(plan.generate.begin(), plan.generate.end(), a) == plan.generate.end()) {
            plan.wait.push_back(a);
        }
    }
}

// Writes the batch's tables into its slot's pinned block and plans its
// launches.  Called WITHOUT `mu`: the slot and the admitted requests (their
// memory, versions and AABB entries, all held by reference) are the worker's
// until the batch's host callback runs, and submitters should not wait while
// thousands of work items are written.
void fill_tables(CfServer* s, int slot_i, const std::vector<Request*>& reqs, LaunchPlan& plan)
{
    StreamSlot& sl = s->slots[slot_i];
    const uint32_t n = plan.views;
    // items are counted first: their section follows the jobs and prefixes
    uint32_t items = 0;
    for (Request* r : reqs) items += r->groups;
    plan.items = items;
    plan.tables = table_layout(n, items);
    cfk::ViewJob* jobs = reinterpret_cast<cfk::ViewJob*>(sl.h_tables);
    uint32_t* prefix = reinterpret_cast<uint32_t*>(sl.h_tables + plan.tables.prefix);
    uint2* it = reinterpret_cast<uint2*>(sl.h_tables + plan.tables.items);
    std::map<uint32_t, std::vector<uint32_t>> buckets;
    uint32_t xb = 0, bb = 0, cb = 0;
    for (uint32_t i = 0; i < n; ++i) {
        Request* r = reqs[i];
        const CfClusterForwardUBO& u = r->req.ubo;
        cfk::ViewJob& j = jobs[i];
        j = cfk::ViewJob{};
        const cfk::WorkspaceLayout& L = r->layout;
        unsigned char* w = r->ws;
        CfLightCell* cells;
        uint32_t *idx, *total;
        out_pointers(r->out, r->clusters, r->req.max_lights_per_cluster, &cells, &idx, &total);
        j.v.vlights = reinterpret_cast<const float4*>(w + L.vlights);
        j.v.nonfinite = reinterpret_cast<const uint32_t*>(w + L.nonfinite);
        j.v.aabbs = reinterpret_cast<const float4*>(r->aabb->d);
        j.v.counts = reinterpret_cast<uint32_t*>(w + L.counts);
        j.v.staging = reinterpret_cast<uint32_t*>(w + L.staging);
        j.v.cells = cells;
        j.v.indices = idx;
        j.v.total = total;
        j.v.slice_lights = reinterpret_cast<float4*>(w + L.slice_lights);
        j.v.slice_idx = reinterpret_cast<uint32_t*>(w + L.slice_idx);
        j.v.slice_count = reinterpret_cast<uint32_t*>(w + L.slice_count);
        j.v.slice_nonfinite = reinterpret_cast<uint32_t*>(w + L.slice_nonfinite);
        j.v.group_boxes = reinterpret_cast<float4*>(w + L.group_boxes);
        j.v.group_sums = reinterpret_cast<uint32_t*>(w + L.group_sums);
        j.v.group_offsets = reinterpret_cast<uint32_t*>(w + L.group_offsets);
        j.v.lpad = cfk::pad_lights(r->lights->count);
        j.v.clusters = r->clusters;
        j.v.cap = r->req.max_lights_per_cluster;
        j.v.slice_clusters = u.sliceCountX * u.sliceCountY;
        j.v.slices = u.sliceCountZ;
        j.v.group_width = (uint32_t)(r->cfg.warps * r->cfg.clusters_per_warp);
        j.v.groups = r->groups;
        j.v.binned = 1;
        j.lights = reinterpret_cast<const CfLightData*>(r->lights->d);
        j.light_count = r->lights->count;
        for (int q = 0; q < 16; ++q) j.view[q] = u.cameraView[q];
        prefix[i] = xb;
        prefix[n + i] = bb;
        prefix[2 * n + i] = cb;
        xb += cfk::granules(j.v.lpad);
        bb += cfk::bin_blocks(j.v.slices);
        cb += cfk::copy_blocks(r->groups);
        buckets[j.v.slice_clusters].push_back(i);
    }
    // largest grids first; consecutive grids with the same configuration share
    // one culling launch over their contiguous items (one launch tail fewer)
    uint32_t ni = 0;
    for (auto kv = buckets.rbegin(); kv != buckets.rend(); ++kv) {
        const cfk::CullConfig& cfg = reqs[kv->second[0]]->cfg;
        const uint32_t begin = ni;
        for (uint32_t vi : kv->second)
            for (uint32_t g = 0; g < jobs[vi].v.groups; ++g) it[ni++] = make_uint2(vi, g);
        LaunchPlan::Bucket* last = plan.buckets.empty() ? nullptr : &plan.buckets.back();
        if (last && last->cfg.clusters_per_warp == cfg.clusters_per_warp && last->cfg.warps == cfg.warps &&
            last->cfg.tile == cfg.tile && last->cfg.stages == cfg.stages && last->cfg.binned == cfg.binned)
            last->count = ni - last->begin;
        else
            plan.buckets.push_back(LaunchPlan::Bucket{cfg, begin, ni - begin});
    }
    plan.xform_blocks = xb;
    plan.bin_blocks = bb;
    plan.copy_blocks = cb;
}

// Enqueues a planned batch on its slot's stream (server lock NOT held: only
// the worker thread launches, and the slot, the requests and their memory are
// its own until the batch's host callback runs).
int enqueue_batch(CfServer* s, int slot_i, const LaunchPlan& plan, const std::vector<Request*>& reqs)
{
    TraceRange trace("Server_Batch");
    StreamSlot& sl = s->slots[slot_i];
    cudaStream_t st = sl.s;
    const uint32_t n = plan.views;
    // every fill enqueued so far (the versions these requests bound, and any
    // reader of memory they were given) before this batch's first kernel
    cudaError_t e = cudaEventRecord(sl.upload_fence, s->upload);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(st, sl.upload_fence, 0);
    if (e != cudaSuccess) return cuda_fail(e, "upload fence");
    for (AabbEntry* a : plan.generate) {
        const Request* r = *std::find_if(reqs.begin(), reqs.end(), [a](const Request* q) { return q->aabb == a; });
        e = cfk::launch_aabb(r->req.ubo, reinterpret_cast<CfAABB*>(a->d), st);
        if (e == cudaSuccess) e = cudaEventRecord(a->ready, st);
        if (e != cudaSuccess) return cuda_fail(e, "AABB generation");
    }
    for (AabbEntry* a : plan.wait) {
        e = cudaStreamWaitEvent(st, a->ready, 0);
        if (e != cudaSuccess) return cuda_fail(e, "wait for AABBs");
    }
    cfk::ViewJob* d_jobs = reinterpret_cast<cfk::ViewJob*>(sl.d_tables);
    const uint32_t* d_prefix = reinterpret_cast<const uint32_t*>(sl.d_tables + plan.tables.prefix);
    const uint2* d_items = reinterpret_cast<const uint2*>(sl.d_tables + plan.tables.items);
    e = cudaMemcpyAsync(sl.d_tables, sl.h_tables, plan.tables.items + (size_t)plan.items * sizeof(uint2),
                        cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess)
        e = cfk::launch_batch_xform(d_jobs, d_prefix, n, plan.xform_blocks, sl.d_queues,
                                    (uint32_t)plan.buckets.size(), st);
    if (e == cudaSuccess) e = cfk::launch_batch_bin(d_jobs, d_prefix + n, nullptr, n, plan.bin_blocks, st);
    for (size_t q = 0; q < plan.buckets.size() && e == cudaSuccess; ++q) {
        const LaunchPlan::Bucket& bk = plan.buckets[q];
        int ctas = 0;
        e = cfk::batch_cull_resident_ctas(bk.cfg, &ctas);
        if (e != cudaSuccess) break;
        cfk::BatchCull bc{d_jobs, d_items + bk.begin, bk.count, sl.d_queues + q};
        e = cfk::launch_batch_cull(bc, bk.cfg, std::min<int>(ctas, (int)bk.count), s->dev_error, st);
    }
    if (e == cudaSuccess) e = cfk::launch_batch_scan(d_jobs, n, st);
    if (e == cudaSuccess) e = cfk::launch_batch_copy(d_jobs, d_prefix + 2 * n, n, plan.copy_blocks, st);
    if (e != cudaSuccess) return cuda_fail(e, "server batch launch");
    Batch* b = new (std::nothrow) Batch();
    if (!b) return fail(CF_ERROR_OUT_OF_MEMORY, "host allocation");
    b->server = s;
    b->slot = slot_i;
    b->reqs = reqs;
    e = cudaLaunchHostFunc(st, on_batch_done, b);
    if (e != cudaSuccess) {
        delete b;
        return cuda_fail(e, "cudaLaunchHostFunc");
    }
    return CF_SUCCESS;
}

void finish_batch(CfServer* s, Batch* b)
{
    s->slots[b->slot].busy = false;
    for (Request* r : b->reqs) {
        r->t_complete = b->t_done;
        r->lights->refs--;
        free_version_if_dead(s, r->lights);
        r->aabb->refs--;
        r->aabb->complete = true;  // this batch waited for (or made) it and has finished
        s->arena.release(r->ws);
        r->ws = nullptr;
        complete_request(s, r, CF_SUCCESS);
    }
    delete b;
}

// Launches queued version jobs on the upload stream (no lock held): every
// upload, then every jitter in queue order.  Running the uploads first is
// safe: an upload writes fresh memory that no queued jitter writes or reads
// except as its source, and that makes it a dependency, never the reverse.
int launch_jobs(CfServer* s, const std::vector<VersionJob>& jobs)
{
    if (jobs.empty()) return CF_SUCCESS;
    if (take_injected_version_write_failure()) return fail(CF_ERROR_CUDA, "light set uploads and jitters (injected)");
    std::vector<cfk::UploadTask> uploads;
    std::vector<cfk::JitterTask> jitters;
    for (const VersionJob& j : jobs) {
        if (j.src)
            jitters.push_back(cfk::JitterTask{reinterpret_cast<const CfLightData*>(j.src->d),
                                              reinterpret_cast<CfLightData*>(j.dst->d), j.seed, j.src->count, j.sigma});
        else
            uploads.push_back(cfk::UploadTask{static_cast<const uint4*>(j.host), reinterpret_cast<uint4*>(j.dst->d),
                                              (uint32_t)((size_t)j.dst->count * sizeof(CfLightData) / 16)});
    }
    cudaError_t e = cfk::launch_upload_tasks(uploads.data(), (uint32_t)uploads.size(), s->upload);
    if (e == cudaSuccess) e = cfk::launch_jitter_tasks(jitters.data(), (uint32_t)jitters.size(), s->upload);
    return e == cudaSuccess ? CF_SUCCESS : cuda_fail(e, "light set uploads and jitters");
}

// The versions a failed launch did not write (lock held): every request bound
// to one fails at admission, and so does a jitter of one.
void mark_failed(const std::vector<VersionJob>& jobs)
{
    for (const VersionJob& j : jobs) j.dst->failed = true;
}

// Drops the jobs' holds on their versions (lock held).
void release_jobs(CfServer* s, const std::vector<VersionJob>& jobs)
{
    for (const VersionJob& j : jobs) {
        j.dst->refs--;
        free_version_if_dead(s, j.dst);
        if (j.src) {
            j.src->refs--;
            free_version_if_dead(s, j.src);
        }
    }
}

void worker_main(CfServer* s)
{
    DeviceGuard g(s->device);
    auto lk = take_lock(s->mu);
    uint64_t blocked_at = UINT64_MAX;  // memory epoch at which the head request did not fit
    for (;;) {
        const uint64_t completed_before = s->stats.completed;
        std::deque<Batch*> done;
        take_finished(s, done);
        for (Batch* b : done) finish_batch(s, b);
        if (!done.empty()) s->memory_epoch++;
        if (blocked_at != s->memory_epoch) blocked_at = UINT64_MAX;
        bool launched = false;
        for (size_t q = 0; q < s->slots.size() && !s->pending.empty() && blocked_at == UINT64_MAX; ++q) {
            if (s->slots[q].busy) continue;
            std::vector<Request*> batch;
            while (!s->pending.empty() && batch.size() < s->cfg.max_batch_views) {
                Request* r = s->pending.front();
                if (!admit(s, r)) {  // arena full: wait until memory is freed (arrival order is kept)
                    blocked_at = s->memory_epoch;
                    break;
                }
                s->pending.pop_front();
                if (r->status != CF_SUCCESS) {
                    r->lights->refs--;
                    free_version_if_dead(s, r->lights);
                    r->t_complete = now_s();
                    complete_request(s, r, r->status);
                    continue;
                }
                batch.push_back(r);
            }
            if (batch.empty()) {
                // Nothing fits.  With nothing in flight or held there is nothing
                // to wait for: the request alone exceeds the budget.
                const bool inflight = std::any_of(s->slots.begin(), s->slots.end(),
                                                  [](const StreamSlot& x) { return x.busy; });
                if (!inflight && s->holding.empty() && !s->pending.empty()) {
                    Request* r = s->pending.front();
                    s->pending.pop_front();
                    r->lights->refs--;
                    free_version_if_dead(s, r->lights);
                    r->t_complete = now_s();
                    complete_request(s, r, CF_ERROR_BUDGET);
                    blocked_at = UINT64_MAX;
                    continue;
                }
                break;
            }
            LaunchPlan plan;
            plan_batch(batch, plan);
            s->slots[q].busy = true;
            const double t_launch = now_s();
            for (Request* r : batch) r->t_launch = t_launch;
            // The uploads and jitters queued so far go first, on the upload
            // stream, ahead of the fence the batch waits on.  The CUDA calls go
            // without the lock, so that submitters, pollers and uploads are not
            // held up behind them.
            std::vector<VersionJob> jobs;
            jobs.swap(s->jobs);
            lk.unlock();
            fill_tables(s, (int)q, batch, plan);
            const int jst = launch_jobs(s, jobs);
            const int st = jst == CF_SUCCESS ? enqueue_batch(s, (int)q, plan, batch) : jst;
            lk = take_lock(s->mu);
            if (jst != CF_SUCCESS) mark_failed(jobs);
            release_jobs(s, jobs);
            if (st != CF_SUCCESS) {
                s->slots[q].busy = false;
                for (AabbEntry* a : plan.generate) a->generated = false;
                for (Request* r : batch) {
                    r->lights->refs--;
                    free_version_if_dead(s, r->lights);
                    r->aabb->refs--;
                    s->arena.release(r->ws);
                    r->t_complete = now_s();
                    complete_request(s, r, st);
                }
            } else {
                s->stats.batches++;
                s->stats.views_launched += batch.size();
                s->stats.max_batch_views = std::max<uint32_t>(s->stats.max_batch_views, (uint32_t)batch.size());
                launched = true;
            }
        }
        if (!launched && !s->jobs.empty()) {
            // No batch went out to carry them: launch the queued jobs alone, so
            // that their versions do not hold arena memory (nor their callers'
            // host buffers) while idle.  If the launch fails, the versions are
            // marked failed and their requests report it.
            std::vector<VersionJob> jobs;
            jobs.swap(s->jobs);
            lk.unlock();
            const int st = launch_jobs(s, jobs);
            lk = take_lock(s->mu);
            if (st != CF_SUCCESS) mark_failed(jobs);
            release_jobs(s, jobs);
        }
        if (s->stats.completed != completed_before) s->done_cv.notify_all();  // one wake-up per pass, not per request
        const bool busy = std::any_of(s->slots.begin(), s->slots.end(), [](const StreamSlot& x) { return x.busy; });
        if (s->stop && s->pending.empty() && !busy && s->finished_n.load() == 0) break;
        if (!launched) {
            s->waiting_for_memory = blocked_at != UINT64_MAX;  // only then does a release wake the worker
            s->cv.wait_for(lk, std::chrono::milliseconds(2), [s, blocked_at] {
                if (s->stop || s->finished_n.load() > 0) return true;
                if (blocked_at != UINT64_MAX) return s->memory_epoch != blocked_at;  // wait for freed memory
                return !s->pending.empty() &&
                       std::any_of(s->slots.begin(), s->slots.end(), [](const StreamSlot& x) { return !x.busy; });
            });
            s->waiting_for_memory = false;
        }
    }
}

int upload_version(CfServer* s, const CfLightData* host, uint32_t n, LightVersion** out)
{
    LightVersion* v = new (std::nothrow) LightVersion();
    if (!v) return fail(CF_ERROR_OUT_OF_MEMORY, "host allocation");
    v->count = n;
    v->d = arena_alloc(s, std::max<size_t>((size_t)n * sizeof(CfLightData), 256));
    if (!v->d) {
        delete v;
        return fail(CF_ERROR_BUDGET, "light set of %u lights does not fit the server's device budget", n);
    }
    (void)host;
    *out = v;
    return CF_SUCCESS;
}

// The device-side address of `host` when it lies in pinned host memory the
// device can read directly (16-byte aligned), else null: pageable memory is
// copied at once by fill_from_host, since its caller may reuse it on return.
const void* device_view_of_pinned(CfServer* s, const void* host)
{
    DeviceGuard g(s->device);
    cudaPointerAttributes a{};
    if (cudaPointerGetAttributes(&a, host) != cudaSuccess) {
        cudaGetLastError();  // clear it: an unknown pointer is simply not pinned
        return nullptr;
    }
    if (a.type != cudaMemoryTypeHost || !a.devicePointer || (reinterpret_cast<uintptr_t>(a.devicePointer) & 15u))
        return nullptr;
    return a.devicePointer;
}

// The device-side address of `host` .. `host` + bytes when the range lies
// inside one declared pinned range (and is 16-byte aligned there), else null.
// No CUDA call.
const void* declared_view(CfServer* s, const void* host, size_t bytes)
{
    const uintptr_t b = reinterpret_cast<uintptr_t>(host);
    std::shared_lock<std::shared_mutex> lk(s->pinned_mu);
    auto it = std::upper_bound(s->pinned.begin(), s->pinned.end(), b,
                               [](uintptr_t x, const PinnedRange& r) { return x < r.begin; });
    if (it == s->pinned.begin()) return nullptr;
    const PinnedRange& r = *std::prev(it);
    if (b < r.begin || bytes > r.end - b) return nullptr;
    const uintptr_t d = r.dev + (b - r.begin);
    return (d & 15u) ? nullptr : reinterpret_cast<const void*>(d);
}

// Where the device reads `count` lights at `host` from: a declared range, else
// whatever the CUDA runtime reports (null: pageable, copied at once).
const void* device_view_of(CfServer* s, const CfLightData* host, uint32_t count)
{
    if (!count) return nullptr;
    const void* d = declared_view(s, host, (size_t)count * sizeof(CfLightData));
    return d ? d : device_view_of_pinned(s, host);
}

// Enqueues the copy that fills v on the upload stream.  Called WITHOUT `mu`:
// a pageable copy blocks the calling thread, and nothing the worker or a
// stream callback needs may wait behind it.
int fill_from_host(CfServer* s, LightVersion* v, const CfLightData* host)
{
    DeviceGuard g(s->device);
    cudaError_t e = cudaSuccess;
    if (v->count)
        e = cudaMemcpyAsync(v->d, host, (size_t)v->count * sizeof(CfLightData), cudaMemcpyHostToDevice, s->upload);
    return e == cudaSuccess ? CF_SUCCESS : cuda_fail(e, "light set upload");
}

void drop_unpublished(CfServer* s, LightVersion* v)
{
    s->arena.release(v->d);
    delete v;
    s->memory_epoch++;
}

void destroy_slot(StreamSlot& sl)
{
    if (sl.s) cudaStreamDestroy(sl.s);
    if (sl.upload_fence) cudaEventDestroy(sl.upload_fence);
    cudaFree(sl.d_tables);
    cudaFree(sl.d_queues);
    cudaFreeHost(sl.h_tables);
}

}  // namespace

extern "C" {

int cf_server_create(CfContext* ctx, const CfServerConfig* config, CfServer** out)
{
    if (!ctx || !out) return fail(CF_ERROR_INVALID_ARGUMENT, "cf_server_create: null argument");
    CfServerConfig c{};
    if (config) c = *config;
    if (!c.hbm_budget_bytes) c.hbm_budget_bytes = 8ull << 30;
    if (!c.max_batch_views) c.max_batch_views = 64;
    if (!c.streams) c.streams = 4;
    if (!c.max_pending) c.max_pending = 4096;  // ~35 ms of queue at 120 000 req/s: refuse overload, do not pile it up
    if (!c.max_groups_per_view) c.max_groups_per_view = 16384;
    if (c.streams > 16 || c.max_batch_views > 4096)
        return fail(CF_ERROR_INVALID_ARGUMENT, "streams <= 16 and max_batch_views <= 4096");
    CfServer* s = new (std::nothrow) CfServer();
    if (!s) return fail(CF_ERROR_OUT_OF_MEMORY, "host allocation");
    s->ctx = ctx;
    s->cfg = c;
    s->device = context_device(ctx);
    s->dev_error = context_error_word(ctx);
    s->items_per_slot = c.max_batch_views * c.max_groups_per_view;
    s->t0 = now_s();
    DeviceGuard g(s->device);
    cudaError_t e = device_malloc(reinterpret_cast<void**>(&s->d_pool), c.hbm_budget_bytes);
    // The upload stream (light-set copies and jitters) at the highest priority:
    // the batch streams' persistent culling launches fill every SM, and its
    // small kernels must be scheduled ahead of their pending CTAs, or its
    // backlog grows until launching on it blocks the submitting threads.
    int prio_low = 0, prio_high = 0;
    if (e == cudaSuccess) e = cudaDeviceGetStreamPriorityRange(&prio_low, &prio_high);
    if (e == cudaSuccess) e = cudaStreamCreateWithPriority(&s->upload, cudaStreamNonBlocking, prio_high);
    s->slots.resize(c.streams);
    for (StreamSlot& sl : s->slots) {
        if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&sl.s, cudaStreamNonBlocking);
        const size_t tb = table_layout(c.max_batch_views, s->items_per_slot).bytes;
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&sl.upload_fence, cudaEventDisableTiming);
        if (e == cudaSuccess) e = device_malloc(reinterpret_cast<void**>(&sl.d_tables), tb);
        if (e == cudaSuccess) e = device_malloc(reinterpret_cast<void**>(&sl.d_queues), cfk::kMaxBatchQueues * sizeof(uint32_t));
        if (e == cudaSuccess) e = cudaMallocHost(&sl.h_tables, tb);
    }
    if (e != cudaSuccess) {
        for (StreamSlot& sl : s->slots) destroy_slot(sl);
        cudaFree(s->d_pool);
        if (s->upload) cudaStreamDestroy(s->upload);
        delete s;
        return cuda_fail(e, "server resources");
    }
    s->arena.reset(s->d_pool, c.hbm_budget_bytes);
    s->worker = std::thread(worker_main, s);
    *out = s;
    return CF_SUCCESS;
}

int cf_server_destroy(CfServer* s)
{
    if (!s) return CF_SUCCESS;
    {
        auto lk = take_lock(s->mu);
        s->stop = true;
        s->cv.notify_all();
    }
    if (s->worker.joinable()) s->worker.join();
    DeviceGuard g(s->device);
    cudaDeviceSynchronize();
    release_jobs(s, s->jobs);  // never launched: nothing will read their versions
    s->jobs.clear();
    for (auto& kv : s->holding) delete kv.second;
    for (auto& kv : s->sets) delete kv.second.cur;
    for (AabbEntry* a : s->aabbs) {
        if (a->ready) cudaEventDestroy(a->ready);
        delete a;
    }
    for (StreamSlot& sl : s->slots) destroy_slot(sl);
    cudaStreamDestroy(s->upload);
    cudaFree(s->d_pool);
    delete s;
    return CF_SUCCESS;
}

int cf_server_declare_pinned_host(CfServer* s, const void* host, size_t bytes)
{
    if (!s || !host || !bytes) return fail(CF_ERROR_INVALID_ARGUMENT, "null or empty range");
    const uintptr_t b = reinterpret_cast<uintptr_t>(host), e = b + bytes;
    if (e < b) return fail(CF_ERROR_INVALID_ARGUMENT, "range wraps around");
    long page = sysconf(_SC_PAGESIZE);
    if (page <= 0) page = 4096;
    // the first byte, every page start inside, the last byte: each pinned and
    // mapped at the same offset from the first, so the device may read any of it
    DeviceGuard g(s->device);
    uintptr_t dev0 = 0;
    for (uintptr_t p = b;;) {
        cudaPointerAttributes a{};
        if (cudaPointerGetAttributes(&a, reinterpret_cast<const void*>(p)) != cudaSuccess) {
            cudaGetLastError();
            return fail(CF_ERROR_INVALID_ARGUMENT, "host range is not known to CUDA");
        }
        if (a.type != cudaMemoryTypeHost || !a.devicePointer)
            return fail(CF_ERROR_INVALID_ARGUMENT, "host range is not pinned and mapped for the device");
        const uintptr_t d = reinterpret_cast<uintptr_t>(a.devicePointer);
        if (p == b) dev0 = d;
        else if (d - dev0 != p - b) return fail(CF_ERROR_INVALID_ARGUMENT, "host range is not one linear mapping");
        if (p == e - 1) break;
        const uintptr_t next = (p / (uintptr_t)page + 1) * (uintptr_t)page;
        p = next < e - 1 ? next : e - 1;
    }
    std::unique_lock<std::shared_mutex> lk(s->pinned_mu);
    auto it = std::upper_bound(s->pinned.begin(), s->pinned.end(), b,
                               [](uintptr_t x, const PinnedRange& r) { return x < r.begin; });
    if (it != s->pinned.begin()) {
        const PinnedRange& q = *std::prev(it);
        if (q.begin == b && q.end == e) return CF_SUCCESS;  // declared before
        if (q.end > b) return fail(CF_ERROR_INVALID_ARGUMENT, "overlaps a declared range");
    }
    if (it != s->pinned.end() && it->begin < e) return fail(CF_ERROR_INVALID_ARGUMENT, "overlaps a declared range");
    s->pinned.insert(it, PinnedRange{b, e, dev0});
    return CF_SUCCESS;
}

int cf_server_register_light_set(CfServer* s, const CfLightData* lights, uint32_t count, uint64_t* id)
{
    if (!s || !id || (count && !lights)) return fail(CF_ERROR_INVALID_ARGUMENT, "null argument");
    if (count > kMaxLights) return fail(CF_ERROR_INVALID_ARGUMENT, "too many lights");
    const void* mapped = device_view_of(s, lights, count);
    LightVersion* v = nullptr;
    {
        auto lk = take_lock(s->mu);
        const int st = upload_version(s, lights, count, &v);
        if (st) return st;
        if (mapped) {  // the worker copies it, with the other queued jobs
            v->refs++;
            s->jobs.push_back(VersionJob{v, nullptr, mapped, 0, 0.0f});
            const uint64_t sid = s->next_set++;
            s->sets[sid] = LightSet{v, ++s->tick};
            *id = sid;
            return CF_SUCCESS;
        }
    }
    const int st = fill_from_host(s, v, lights);  // not under `mu`
    auto lk = take_lock(s->mu);
    if (st) {
        drop_unpublished(s, v);
        return st;
    }
    const uint64_t sid = s->next_set++;
    s->sets[sid] = LightSet{v, ++s->tick};
    *id = sid;
    return CF_SUCCESS;
}

// Publishes v as the current version of set `id` (mu held); v is discarded
// (once its fill has finished) when the set was released meanwhile.
int publish_version(CfServer* s, uint64_t id, LightVersion* v, LightVersion* pinned_old)
{
    pinned_old->refs--;
    auto it = s->sets.find(id);
    if (it == s->sets.end()) {
        free_version_if_dead(s, pinned_old);
        s->arena.release(v->d);  // its fill may still run: later users order after it (see LightVersion)
        delete v;
        return fail(CF_ERROR_NOT_READY, "light set %llu was released", (unsigned long long)id);
    }
    LightVersion* old = it->second.cur;
    old->retired = true;
    free_version_if_dead(s, old);
    if (pinned_old != old) free_version_if_dead(s, pinned_old);
    it->second.cur = v;
    it->second.last_use = ++s->tick;
    return CF_SUCCESS;
}

int cf_server_update_light_set(CfServer* s, uint64_t id, const CfLightData* lights, uint32_t count)
{
    if (!s || (count && !lights)) return fail(CF_ERROR_INVALID_ARGUMENT, "null argument");
    const void* mapped = device_view_of(s, lights, count);
    LightVersion *v = nullptr, *old = nullptr;
    {
        auto lk = take_lock(s->mu);
        auto it = s->sets.find(id);
        if (it == s->sets.end()) return fail(CF_ERROR_NOT_READY, "light set %llu is not resident", (unsigned long long)id);
        old = it->second.cur;
        old->refs++;  // neither evictable nor freed while the new version is placed
        const int st = upload_version(s, lights, count, &v);
        if (st) {
            old->refs--;
            return st;
        }
        if (mapped) {  // the worker copies it, with the other queued jobs
            v->refs++;
            s->jobs.push_back(VersionJob{v, nullptr, mapped, 0, 0.0f});
            return publish_version(s, id, v, old);
        }
    }
    const int st = fill_from_host(s, v, lights);  // not under `mu`
    auto lk = take_lock(s->mu);
    if (st) {
        old->refs--;
        free_version_if_dead(s, old);
        drop_unpublished(s, v);
        return st;
    }
    return publish_version(s, id, v, old);
}

int cf_server_jitter_light_set(CfServer* s, uint64_t id, uint64_t seed, float sigma)
{
    if (!s) return fail(CF_ERROR_INVALID_ARGUMENT, "null server");
    auto lk = take_lock(s->mu);
    auto it = s->sets.find(id);
    if (it == s->sets.end()) return fail(CF_ERROR_NOT_READY, "light set %llu is not resident", (unsigned long long)id);
    LightVersion* old = it->second.cur;
    old->refs += 2;  // one for the queued jitter, one that publish_version releases; neither evictable meanwhile
    LightVersion* v = new (std::nothrow) LightVersion();
    unsigned char* d = v ? arena_alloc(s, std::max<size_t>((size_t)old->count * sizeof(CfLightData), 256)) : nullptr;
    if (!v || !d) {
        delete v;
        old->refs -= 2;
        return fail(CF_ERROR_BUDGET, "no room for a new version of light set %llu", (unsigned long long)id);
    }
    v->d = d;
    v->count = old->count;
    v->failed = old->failed;  // a jitter of an unwritten version is unwritten too
    // The jitter itself is queued: the worker launches the queued jobs on the
    // upload stream in one go before the next batch's upload fence, so a
    // request that binds the new version reads it only after it is written,
    // and the caller pays no CUDA call here.
    v->refs++;
    s->jobs.push_back(VersionJob{v, old, nullptr, seed, sigma});
    return publish_version(s, id, v, old);
}

int cf_server_release_light_set(CfServer* s, uint64_t id)
{
    if (!s) return fail(CF_ERROR_INVALID_ARGUMENT, "null server");
    auto lk = take_lock(s->mu);
    auto it = s->sets.find(id);
    if (it == s->sets.end()) return CF_SUCCESS;
    it->second.cur->retired = true;
    free_version_if_dead(s, it->second.cur);
    s->sets.erase(it);
    s->memory_epoch++;
    if (s->waiting_for_memory) s->cv.notify_all();
    return CF_SUCCESS;
}

int cf_server_is_light_set_resident(CfServer* s, uint64_t id, int* resident)
{
    if (!s || !resident) return fail(CF_ERROR_INVALID_ARGUMENT, "null argument");
    auto lk = take_lock(s->mu);
    *resident = s->sets.count(id) ? 1 : 0;
    return CF_SUCCESS;
}

int cf_server_submit(CfServer* s, const CfServerRequest* req, uint64_t* request_id)
{
    if (!s || !req || !request_id) return fail(CF_ERROR_INVALID_ARGUMENT, "cf_server_submit: null argument");
    uint32_t C = 0;
    const uint32_t cap = req->max_lights_per_cluster ? req->max_lights_per_cluster : CF_MAX_LIGHTS_PER_CLUSTER_DEFAULT;
    int st = validate_grid(req->ubo.sliceCountX, req->ubo.sliceCountY, req->ubo.sliceCountZ, cap, &C);
    if (st) return st;
    Request* r = new (std::nothrow) Request();
    if (!r) return fail(CF_ERROR_OUT_OF_MEMORY, "host allocation");
    r->req = *req;
    r->req.max_lights_per_cluster = cap;
    r->clusters = C;
    r->t_submit = now_s();
    auto lk = take_lock(s->mu);
    if (s->pending.size() >= s->cfg.max_pending) {
        delete r;
        return fail(CF_ERROR_BUDGET, "%zu requests pending", s->pending.size());
    }
    auto it = s->sets.find(req->light_set);
    if (it == s->sets.end()) {
        delete r;
        return fail(CF_ERROR_NOT_READY, "light set %llu is not resident", (unsigned long long)req->light_set);
    }
    r->lights = it->second.cur;  // this version, whatever updates follow
    r->lights->refs++;
    it->second.last_use = ++s->tick;
    r->id = s->next_req++;
    *request_id = r->id;
    s->pending.push_back(r);
    s->stats.submitted++;
    s->stats.max_pending = std::max<uint64_t>(s->stats.max_pending, s->pending.size());
    s->cv.notify_all();
    return CF_SUCCESS;
}

int cf_server_poll(CfServer* s, CfServerCompletion* out, uint32_t max, uint32_t* count, int wait_ms)
{
    if (!s || !count || (max && !out)) return fail(CF_ERROR_INVALID_ARGUMENT, "null argument");
    auto lk = take_lock(s->mu);
    if (s->completions.empty() && wait_ms > 0)
        s->done_cv.wait_for(lk, std::chrono::milliseconds(wait_ms), [s] { return !s->completions.empty(); });
    uint32_t n = 0;
    while (n < max && !s->completions.empty()) {
        out[n++] = s->completions.front();
        s->completions.pop_front();
    }
    *count = n;
    return CF_SUCCESS;
}

int cf_server_release(CfServer* s, uint64_t request_id)
{
    return cf_server_release_many(s, &request_id, 1);
}

int cf_server_release_many(CfServer* s, const uint64_t* request_ids, uint32_t n)
{
    if (!s || (n && !request_ids)) return fail(CF_ERROR_INVALID_ARGUMENT, "null argument");
    auto lk = take_lock(s->mu);
    uint64_t unknown = 0;
    uint32_t n_unknown = 0;
    for (uint32_t i = 0; i < n; ++i) {
        auto it = s->holding.find(request_ids[i]);
        if (it == s->holding.end()) {
            if (!n_unknown++) unknown = request_ids[i];
            continue;
        }
        s->arena.release(it->second->out);
        delete it->second;
        s->holding.erase(it);
    }
    if (n_unknown < n) {
        s->memory_epoch++;
        if (s->waiting_for_memory) s->cv.notify_all();
    }
    if (n_unknown)
        return fail(CF_ERROR_INVALID_ARGUMENT, "%u request(s) hold no outputs, the first %llu", n_unknown,
                    (unsigned long long)unknown);
    return CF_SUCCESS;
}

int cf_server_set_tuning(CfServer* s, uint32_t slice_clusters, int clusters_per_warp, int warps, int tile, int stages)
{
    if (!s) return fail(CF_ERROR_INVALID_ARGUMENT, "null server");
    auto lk = take_lock(s->mu);
    if (clusters_per_warp == 0) {
        s->tuned.erase(slice_clusters);
        return CF_SUCCESS;
    }
    const cfk::CullConfig c{clusters_per_warp, warps, tile, stages, 1};
    if (!cfk::cull_config_supported(c)) return fail(CF_ERROR_INVALID_ARGUMENT, "unsupported configuration");
    s->tuned[slice_clusters] = c;
    return CF_SUCCESS;
}

int cf_server_get_stats(CfServer* s, CfServerStats* out)
{
    if (!s || !out) return fail(CF_ERROR_INVALID_ARGUMENT, "null argument");
    auto lk = take_lock(s->mu);
    *out = s->stats;
    out->arena_used_bytes = s->arena.used();
    out->arena_bytes = s->arena.size();
    out->pending = s->pending.size();
    out->resident_light_sets = s->sets.size();
    out->resident_projections = s->aabbs.size();
    return CF_SUCCESS;
}

}  // extern "C"
