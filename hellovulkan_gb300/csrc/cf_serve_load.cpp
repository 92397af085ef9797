// cf_serve_load.cpp — a native Poisson load driver for the culling server.
//
// Replays a served stream of culling requests against a CfServer in real
// time: arrivals are a Poisson process of the given rate; each request draws
// a projection (grid + resolution) and a random camera; with probability
// p_reuse it re-references one of the submitting thread's recent light sets
// after moving every light by a jitter of the given sigma on the device
// (cf_server_jitter_light_set), otherwise it registers a new set copied from
// a pool of pre-generated light sets (declared to the server when pinned).
// Sets that leave a thread's window of recent sets are released.  A poller
// thread records each completion's latency from the scheduled arrival and
// releases the outputs of each poll in one cf_server_release_many call.  All
// random draws come from std::mt19937_64 seeded by `seed`.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <deque>
#include <random>
#include <thread>
#include <vector>

#include "cf_runtime_internal.h"
#include "cfcull.h"

using namespace cfrt;

namespace {

using clk = std::chrono::steady_clock;

double secs(clk::time_point t) { return std::chrono::duration<double>(t.time_since_epoch()).count(); }

// Right-handed look-at, column-major (element (col,row) at col*4+row).
void look_at(const double eye[3], const double tgt[3], float out[16])
{
    double f[3] = {tgt[0] - eye[0], tgt[1] - eye[1], tgt[2] - eye[2]};
    double fl = std::sqrt(f[0] * f[0] + f[1] * f[1] + f[2] * f[2]);
    for (double& x : f) x /= fl;
    const double up[3] = {0, 1, 0};
    double s[3] = {f[1] * up[2] - f[2] * up[1], f[2] * up[0] - f[0] * up[2], f[0] * up[1] - f[1] * up[0]};
    double sl = std::sqrt(s[0] * s[0] + s[1] * s[1] + s[2] * s[2]);
    for (double& x : s) x /= sl;
    const double u[3] = {s[1] * f[2] - s[2] * f[1], s[2] * f[0] - s[0] * f[2], s[0] * f[1] - s[1] * f[0]};
    double m[4][4] = {};  // m[row][col]
    for (int c = 0; c < 3; ++c) {
        m[0][c] = s[c];
        m[1][c] = u[c];
        m[2][c] = -f[c];
    }
    m[0][3] = -(s[0] * eye[0] + s[1] * eye[1] + s[2] * eye[2]);
    m[1][3] = -(u[0] * eye[0] + u[1] * eye[1] + u[2] * eye[2]);
    m[2][3] = f[0] * eye[0] + f[1] * eye[1] + f[2] * eye[2];
    m[3][3] = 1.0;
    for (int c = 0; c < 4; ++c)
        for (int r = 0; r < 4; ++r) out[c * 4 + r] = (float)m[r][c];
}

double percentile(std::vector<double> v, double p)
{
    if (v.empty()) return 0.0;
    std::sort(v.begin(), v.end());
    const double pos = p * (double)(v.size() - 1);
    const size_t i = (size_t)pos;
    const double f = pos - (double)i;
    return i + 1 < v.size() ? v[i] * (1 - f) + v[i + 1] * f : v[i];
}

}  // namespace

extern "C" int cf_serve_run_load(CfServer* server, const CfServeLoad* load, CfServeReport* report)
{
    if (!server || !load || !report || !load->projections || !load->n_projections || !load->n_base_sets ||
        !load->base_sets || !load->base_counts || load->rate_per_s <= 0 || load->duration_s <= 0)
        return fail(CF_ERROR_INVALID_ARGUMENT, "cf_serve_run_load: bad argument");
    // a client with a pinned pool declares it once, so that its registers make
    // no CUDA call (pageable sets fail the declaration and are copied per call)
    for (uint32_t b = 0; b < load->n_base_sets; ++b)
        if (load->base_sets[b] && load->base_counts[b])
            (void)cf_server_declare_pinned_host(server, load->base_sets[b],
                                                (size_t)load->base_counts[b] * sizeof(CfLightData));
    const uint32_t threads = std::max(1u, load->submit_threads);
    const uint32_t window = std::max(1u, load->recent_sets / threads);
    // arrival schedule
    std::mt19937_64 rng(load->seed);
    std::exponential_distribution<double> gap(load->rate_per_s);
    std::vector<double> arrival;
    for (double t = gap(rng); t < load->duration_s; t += gap(rng)) arrival.push_back(t);
    const size_t n = arrival.size();
    std::vector<double> submit_lag(n, 0.0), latency(n, -1.0), queue(n, -1.0), exec(n, -1.0);
    std::vector<double> set_call(n, -1.0), submit_call(n, -1.0);  // seconds in the set call / in submit
    std::vector<char> reused_set(n, 0);
    std::vector<uint64_t> tests(n, 0);
    std::vector<int> status(n, 0);
    std::atomic<size_t> submitted{0}, new_sets{0}, reused{0}, submit_errors{0};
    std::atomic<bool> submitting_done{false};
    const clk::time_point start = clk::now() + std::chrono::milliseconds(20);

    auto submitter = [&](uint32_t tid) {
        std::mt19937_64 r(load->seed * 1000003ull + tid + 1);
        std::uniform_real_distribution<double> U(0.0, 1.0);
        std::deque<std::pair<uint64_t, uint32_t>> recent;  // (set id, light count)
        for (size_t i = tid; i < n; i += threads) {
            const clk::time_point due = start + std::chrono::duration_cast<clk::duration>(
                                                    std::chrono::duration<double>(arrival[i]));
            std::this_thread::sleep_until(due);
            uint64_t set_id = 0;
            uint32_t count = 0;
            int st = CF_SUCCESS;
            const clk::time_point t_call = clk::now();
            if (!recent.empty() && U(r) < load->p_reuse) {
                reused_set[i] = 1;
                const auto& pick = recent[(size_t)(U(r) * (double)recent.size()) % recent.size()];
                set_id = pick.first;
                count = pick.second;
                st = cf_server_jitter_light_set(server, set_id, load->seed ^ (0x5851F42D4C957F2Dull * (i + 1)),
                                                load->jitter_sigma);
                reused++;
            } else {
                const uint32_t b = (uint32_t)(U(r) * load->n_base_sets) % load->n_base_sets;
                count = load->base_counts[b];
                st = cf_server_register_light_set(server, load->base_sets[b], count, &set_id);
                if (st == CF_SUCCESS) {
                    recent.emplace_back(set_id, count);
                    if (recent.size() > window) {
                        cf_server_release_light_set(server, recent.front().first);
                        recent.pop_front();
                    }
                }
                new_sets++;
            }
            set_call[i] = std::chrono::duration<double>(clk::now() - t_call).count();
            CfServerRequest q{};
            const uint32_t p = (uint32_t)(U(r) * load->n_projections) % load->n_projections;
            q.ubo = load->projections[p];
            double eye[3], tgt[3];
            for (int a = 0; a < 3; ++a) {
                eye[a] = load->eye_lo[a] + (load->eye_hi[a] - load->eye_lo[a]) * U(r);
                tgt[a] = load->target_lo[a] + (load->target_hi[a] - load->target_lo[a]) * U(r);
            }
            look_at(eye, tgt, q.ubo.cameraView);
            q.light_set = set_id;
            q.user_tag = i;
            q.max_lights_per_cluster = load->max_lights_per_cluster;
            submit_lag[i] = secs(clk::now()) - secs(due);
            tests[i] = (uint64_t)q.ubo.sliceCountX * q.ubo.sliceCountY * q.ubo.sliceCountZ * count;
            uint64_t rid = 0;
            const clk::time_point t_sub = clk::now();
            if (st == CF_SUCCESS) st = cf_server_submit(server, &q, &rid);
            submit_call[i] = std::chrono::duration<double>(clk::now() - t_sub).count();
            if (st != CF_SUCCESS) {
                submit_errors++;
                status[i] = -1;
                continue;
            }
            submitted++;
        }
    };

    std::vector<CfServerCompletion> buf(4096);
    std::vector<uint64_t> done_ids;
    done_ids.reserve(buf.size());
    std::atomic<size_t> completed{0}, failed{0};
    double last_done = 0.0;
    auto poller = [&]() {
        for (;;) {
            uint32_t got = 0;
            cf_server_poll(server, buf.data(), (uint32_t)buf.size(), &got, 1);
            const double now = secs(clk::now());
            done_ids.clear();
            for (uint32_t k = 0; k < got; ++k) {
                const CfServerCompletion& c = buf[k];
                const size_t i = (size_t)c.user_tag;
                if (c.status == CF_SUCCESS) {
                    done_ids.push_back(c.request_id);
                    latency[i] = submit_lag[i] + (c.t_complete - c.t_submit);
                    queue[i] = submit_lag[i] + (c.t_launch - c.t_submit);
                    exec[i] = c.t_complete - c.t_launch;
                    completed++;
                } else {
                    status[i] = c.status;
                    failed++;
                }
                last_done = now;
            }
            // every output of this poll back to the server under one lock
            if (!done_ids.empty()) cf_server_release_many(server, done_ids.data(), (uint32_t)done_ids.size());
            if (submitting_done && completed + failed >= submitted) break;
        }
    };

    std::thread poll_thread(poller);
    std::vector<std::thread> subs;
    for (uint32_t t = 0; t < threads; ++t) subs.emplace_back(submitter, t);
    for (std::thread& t : subs) t.join();
    submitting_done = true;
    poll_thread.join();

    std::vector<double> lat, q, lag, ex, reg_us, jit_us, sub_us;
    uint64_t tests_done = 0;
    for (size_t i = 0; i < n; ++i) {
        if (latency[i] >= 0) {
            lat.push_back(latency[i] * 1e3);
            q.push_back(queue[i] * 1e3);
            ex.push_back(exec[i] * 1e3);
            tests_done += tests[i];
        }
        lag.push_back(submit_lag[i] * 1e3);
        if (set_call[i] >= 0) (reused_set[i] ? jit_us : reg_us).push_back(set_call[i] * 1e6);
        if (submit_call[i] >= 0) sub_us.push_back(submit_call[i] * 1e6);
    }
    const double wall = std::max(1e-9, last_done - secs(start));
    CfServeReport rep{};
    rep.scheduled = n;
    rep.submitted = submitted;
    rep.completed = completed;
    rep.failed = failed + submit_errors;
    rep.new_sets = new_sets;
    rep.reused_sets = reused;
    rep.wall_s = wall;
    rep.offered_rate = (double)n / load->duration_s;
    rep.achieved_rate = (double)completed / wall;
    rep.latency_p50_ms = percentile(lat, 0.50);
    rep.latency_p90_ms = percentile(lat, 0.90);
    rep.latency_p99_ms = percentile(lat, 0.99);
    rep.latency_p999_ms = percentile(lat, 0.999);
    rep.latency_max_ms = lat.empty() ? 0 : *std::max_element(lat.begin(), lat.end());
    rep.queue_p50_ms = percentile(q, 0.50);
    rep.queue_p99_ms = percentile(q, 0.99);
    rep.submit_lag_p99_ms = percentile(lag, 0.99);
    rep.exec_p50_ms = percentile(ex, 0.50);
    rep.exec_p99_ms = percentile(ex, 0.99);
    rep.register_call_p50_us = percentile(reg_us, 0.50);
    rep.register_call_p99_us = percentile(reg_us, 0.99);
    rep.jitter_call_p50_us = percentile(jit_us, 0.50);
    rep.jitter_call_p99_us = percentile(jit_us, 0.99);
    rep.submit_call_p50_us = percentile(sub_us, 0.50);
    rep.submit_call_p99_us = percentile(sub_us, 0.99);
    auto vmax = [](const std::vector<double>& v) { return v.empty() ? 0.0 : *std::max_element(v.begin(), v.end()); };
    rep.register_call_max_us = vmax(reg_us);
    rep.jitter_call_max_us = vmax(jit_us);
    rep.submit_call_max_us = vmax(sub_us);
    size_t worst = 0;
    for (size_t i = 1; i < n; ++i)
        if (submit_lag[i] > submit_lag[worst]) worst = i;
    rep.worst_lag_arrival_s = n ? arrival[worst] : 0.0;
    rep.tests_brute_force = tests_done;
    *report = rep;
    return CF_SUCCESS;
}
