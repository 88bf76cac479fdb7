// server.cpp — continuous batching of render jobs (solrt_server_*).
//
// The reference renders one interactive view; serving many independent
// render requests is this library's addition. A serving thread runs ticks:
//   1. admission: queued jobs, in arrival order, while the job's image (and
//      its scene, unless an admitted job already counts it) fits the memory
//      budget; completed but unreleased results are evicted least recently
//      used first to make room;
//   2. one wavefront pass in which every active job advances by a share of
//      tick_paths (at least one sample; REF_STREAM jobs one sample);
//   3. jobs whose last samples were in the pass are finalized in the same
//      tick and reported with their latency; with a stopping rule
//      (stop_rmse), jobs whose estimated RMSE against their converged image
//      fell to the bound are finalized right after it, with the samples they
//      have.
// Ticks are sized to about tick_ms of device time at the measured rate
// unless the server was given a fixed tick_paths.
// Jobs arriving while a tick runs join at the next tick. A job's image is
// the same as solrt_render of that job alone: its samples are accumulated
// in order whatever ticks they fall in, and nothing is shared between jobs.
#include <algorithm>
#include <cmath>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <list>
#include <mutex>
#include <new>
#include <thread>
#include <unordered_map>
#include <vector>

#include "internal.h"

struct solrt_context : solrt::Context {};
struct solrt_scene : solrt::Scene {};
struct solrt_image : solrt::Image {};

namespace {

uint64_t now_ns() {
    return (uint64_t)std::chrono::duration_cast<std::chrono::nanoseconds>(
               std::chrono::steady_clock::now().time_since_epoch())
        .count();
}

enum JobState { kQueued, kActive, kDone, kFailed };

struct ServerJob {
    uint64_t ticket = 0;
    solrt_scene* scene = nullptr;
    solrt_camera cam{};
    solrt_render_params p{};
    solrt_image* image = nullptr;
    JobState state = kQueued;
    uint32_t spp_done = 0;
    uint32_t status = SOLRT_ERR_NOT_READY;
    uint64_t t_submit = 0, t_admit = 0, t_done = 0, last_use = 0;
    uint64_t image_bytes = 0;
    bool counted = false;  // image and scene counted against the budget
    bool cancel = false;   // cancelled while running: leaves after the tick in flight
    float* sq = nullptr;   // stopping rule: per-pixel squared sample sums (device)
    float rmse_est = -1.0f;
    bool stopped_early = false;
};

uint64_t image_bytes_of(const solrt_render_params& p, bool stop_rule) {
    const uint64_t np = (uint64_t)p.width * p.height;
    return np * (16 + 4 + 16 + 4) + (p.accum_mode == SOLRT_ACCUM_KAHAN ? np * 32 : 0) + (stop_rule ? np * 4 : 0);
}

}  // namespace

struct solrt_server {
    solrt_context* ctx = nullptr;
    uint64_t budget = 0;
    uint32_t tick_paths = 0;
    bool adaptive = false;    // tick_paths follows tick_ms at the measured rate
    double tick_ms = 40.0;
    double rate = 0.0;        // paths per ms of device time (moving average)
    float stop_rmse = 0.0f;
    uint32_t stop_min_spp = 4;
    uint32_t policy = SOLRT_SERVE_FAIR;
    uint32_t inject_alloc_failures = 0;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::thread th;
    bool stop = false;
    uint64_t next_ticket = 1;
    std::unordered_map<uint64_t, ServerJob> jobs;
    std::deque<uint64_t> queue;
    std::vector<uint64_t> active;
    std::list<uint64_t> done_lru;                     // completed, unreleased; front = least recently used
    std::deque<uint64_t> finished;                    // done / failed / cancelled, not yet fetched (completion queue)
    std::unordered_map<solrt_scene*, int> scene_refs;  // admitted (active or done) jobs per scene
    uint64_t bytes_in_use = 0;
    solrt_server_stats st{};
    solrt::TickBuffers tb;
    uint32_t kind = 0;
    bool kind_set = false;
};

namespace {

// A job reached its final state (done, failed or cancelled): its ticket
// joins the completion queue of solrt_server_finished, which keeps the
// newest kFinishedMax tickets (a client that never fetches them does not
// grow it without bound). Caller holds the lock.
constexpr size_t kFinishedMax = size_t(1) << 20;
void mark_finished(solrt_server* srv, uint64_t ticket) {
    if (srv->finished.size() >= kFinishedMax) srv->finished.pop_front();
    srv->finished.push_back(ticket);
}

uint64_t scene_bytes(solrt_scene* s) {
    uint64_t b = 0;
    solrt_scene_bytes(s, &b);
    return b;
}

// Frees a job's image and its budget share. Caller holds the lock.
void drop_job_memory(solrt_server* srv, ServerJob& j) {
    if (!j.counted) return;
    j.counted = false;
    if (j.sq) {
        cudaFree(j.sq);
        j.sq = nullptr;
    }
    if (j.image) {
        solrt_image_destroy(j.image);
        j.image = nullptr;
        srv->bytes_in_use -= j.image_bytes;
    }
    auto it = srv->scene_refs.find(j.scene);
    if (it != srv->scene_refs.end() && --it->second == 0) {
        srv->bytes_in_use -= scene_bytes(j.scene);
        srv->scene_refs.erase(it);
    }
}

void admit(solrt_server* srv) {
    while (!srv->queue.empty()) {
        ServerJob& j = srv->jobs[srv->queue.front()];
        const bool rule = srv->stop_rmse > 0.0f;
        const uint64_t need = image_bytes_of(j.p, rule) + (srv->scene_refs.count(j.scene) ? 0 : scene_bytes(j.scene));
        while (srv->bytes_in_use + need > srv->budget && !srv->done_lru.empty()) {
            const uint64_t victim = srv->done_lru.front();
            srv->done_lru.pop_front();
            ServerJob& v = srv->jobs[victim];
            drop_job_memory(srv, v);
            srv->jobs.erase(victim);
            ++srv->st.evicted;
        }
        if (srv->bytes_in_use + need > srv->budget) {
            if (srv->active.empty()) {  // can never fit
                j.state = kFailed;
                j.status = SOLRT_ERR_BUDGET;
                j.t_done = now_ns();
                mark_finished(srv, j.ticket);
                srv->queue.pop_front();
                srv->cv_done.notify_all();
                continue;
            }
            return;  // wait for active jobs to finish
        }
        solrt_image* img = nullptr;
        solrt_status s;
        if (srv->inject_alloc_failures) {  // host-side fault injection (tests)
            --srv->inject_alloc_failures;
            solrt::set_error("injected allocation failure");
            s = SOLRT_ERR_OOM;
        } else {
            s = solrt_image_create(srv->ctx, j.p.width, j.p.height, j.p.accum_mode, &img);
            if (s == SOLRT_OK && rule) {
                const size_t b = sizeof(float) * (size_t)j.p.width * j.p.height;
                if (cudaMalloc(&j.sq, b) != cudaSuccess ||
                    cudaMemsetAsync(j.sq, 0, b, srv->ctx->stream) != cudaSuccess) {
                    cudaGetLastError();
                    if (j.sq) cudaFree(j.sq);
                    j.sq = nullptr;
                    solrt_image_destroy(img);
                    img = nullptr;
                    solrt::set_error("cannot allocate the squared sums of the stopping rule");
                    s = SOLRT_ERR_OOM;
                }
            }
        }
        srv->queue.pop_front();
        if (s != SOLRT_OK) {
            j.state = kFailed;
            j.status = s;
            j.t_done = now_ns();
            mark_finished(srv, j.ticket);
            srv->cv_done.notify_all();
            continue;
        }
        j.image = img;
        j.counted = true;
        j.image_bytes = image_bytes_of(j.p, rule);
        srv->bytes_in_use += j.image_bytes;
        if (srv->scene_refs[j.scene]++ == 0) srv->bytes_in_use += scene_bytes(j.scene);
        j.state = kActive;
        j.t_admit = now_ns();
        srv->active.push_back(j.ticket);
        ++srv->st.admitted;
    }
}

void serve_loop(solrt_server* srv) {
    solrt::Context& ctx = *srv->ctx;
    cudaSetDevice(ctx.device);
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    std::vector<solrt::DevJob> jobs, fin, est_jobs;
    std::vector<solrt::DevItem> items;
    std::vector<uint64_t> tick_tickets, fin_tickets, est_tickets;
    std::vector<uint32_t> tick_k, est_n;
    std::vector<double> est_sum;
    for (;;) {
        solrt::PassPlan pp{0, 0, 0, 0, 0};
        {
            std::unique_lock<std::mutex> lock(srv->mu);
            srv->cv_work.wait_for(lock, std::chrono::milliseconds(20),
                                  [&] { return srv->stop || !srv->queue.empty() || !srv->active.empty(); });
            if (srv->stop) break;
            // running jobs cancelled since the last tick leave now (no tick
            // in flight uses their images)
            for (uint64_t t : srv->active) {
                ServerJob& j = srv->jobs[t];
                if (j.cancel) {
                    drop_job_memory(srv, j);
                    j.state = kFailed;
                    j.status = SOLRT_ERR_CANCELLED;
                    j.t_done = now_ns();
                    mark_finished(srv, j.ticket);
                }
            }
            srv->active.erase(std::remove_if(srv->active.begin(), srv->active.end(),
                                             [&](uint64_t t) { return srv->jobs[t].state != kActive; }),
                              srv->active.end());
            srv->cv_done.notify_all();
            admit(srv);
            if (srv->active.empty()) continue;
            // plan the tick: a fair share of tick_paths per active job
            jobs.clear();
            items.clear();
            fin.clear();
            tick_tickets.clear();
            fin_tickets.clear();
            tick_k.clear();
            const bool shortest = srv->policy == SOLRT_SERVE_SHORTEST_FIRST;
            if (shortest) {  // least remaining work first (ticket order breaks ties)
                std::sort(srv->active.begin(), srv->active.end(), [&](uint64_t a, uint64_t b) {
                    const ServerJob& x = srv->jobs[a];
                    const ServerJob& y = srv->jobs[b];
                    const uint64_t wx = (uint64_t)x.p.width * x.p.height * (x.p.spp - x.spp_done);
                    const uint64_t wy = (uint64_t)y.p.width * y.p.height * (y.p.spp - y.spp_done);
                    return wx != wy ? wx < wy : a < b;
                });
            }
            const uint32_t share = std::max<uint32_t>(1u, srv->tick_paths / (uint32_t)srv->active.size());
            for (uint64_t t : srv->active) {
                ServerJob& j = srv->jobs[t];
                const uint32_t np = j.p.width * j.p.height;
                const uint32_t left = j.p.spp - j.spp_done;
                // fair: an equal share; shortest first: what is left of the tick
                const uint32_t room = shortest ? (srv->tick_paths > pp.paths ? srv->tick_paths - pp.paths : 0u)
                                               : share;
                // a job larger than what is left waits for the next tick,
                // unless the tick is still empty (it then runs one sample, so
                // jobs larger than a whole tick are not starved)
                if (shortest && room < np && pp.paths > 0) continue;
                uint32_t k = j.p.rng_mode == SOLRT_RNG_REF_STREAM ? 1u : std::max(1u, std::min(left, room / np));
                if ((uint64_t)pp.paths + (uint64_t)np * k > ctx.capacity) {
                    if (pp.paths + np > ctx.capacity) continue;  // next tick
                    k = 1;
                }
                solrt::DevItem it{(uint32_t)jobs.size(), 0u, np, j.spp_done, k, pp.paths, pp.pixels, 0u};
                const solrt::Scene& sc = *static_cast<solrt::Scene*>(j.scene);
                const solrt::Image& img = *static_cast<solrt::Image*>(j.image);
                jobs.push_back(solrt::job_for(sc, img, j.cam, j.p));
                jobs.back().sq = j.sq;
                items.push_back(it);
                pp.item_count += 1;
                pp.paths += np * k;
                pp.pixels += np;
                pp.bounces = std::max(pp.bounces, j.p.max_bounces + 1u);
                if (j.p.integrator == SOLRT_INTEGRATOR_PATH_NEE) pp.nee = 1u;
                tick_tickets.push_back(t);
                tick_k.push_back(k);
                if (j.spp_done + k == j.p.spp) {
                    fin.push_back(jobs.back());
                    fin_tickets.push_back(t);
                }
            }
        }
        // run the tick outside the lock
        cudaEventRecord(e0, ctx.stream);
        const solrt_status s = solrt::serve_tick(ctx, srv->tb, srv->kind, jobs, items, pp, fin);
        cudaEventRecord(e1, ctx.stream);
        const cudaError_t e = cudaEventSynchronize(e1);
        float ms = 0.0f;
        cudaEventElapsedTime(&ms, e0, e1);
        const uint64_t t_end = now_ns();
        std::lock_guard<std::mutex> lock(srv->mu);
        ++srv->st.ticks;
        srv->st.busy_ms += ms;
        srv->st.tick_paths = pp.paths;
        if (srv->adaptive && pp.paths > 0 && ms > 0.0f) {
            // next tick: about tick_ms at the rate of the recent ticks
            const double r = (double)pp.paths / (double)ms;
            srv->rate = srv->rate > 0.0 ? 0.7 * srv->rate + 0.3 * r : r;
            const double want = srv->rate * srv->tick_ms;
            srv->tick_paths = (uint32_t)std::min<double>(ctx.capacity, std::max<double>(1u << 20, want));
        }
        for (size_t i = 0; i < tick_tickets.size(); ++i) {
            ServerJob& j = srv->jobs[tick_tickets[i]];
            if (s != SOLRT_OK || e != cudaSuccess) {
                j.state = kFailed;
                j.status = s != SOLRT_OK ? s : SOLRT_ERR_DEVICE;
                j.t_done = t_end;
                mark_finished(srv, j.ticket);
                continue;
            }
            j.spp_done += tick_k[i];
            if (j.spp_done == j.p.spp) {
                j.state = kDone;
                j.status = SOLRT_OK;
                j.t_done = t_end;
                mark_finished(srv, j.ticket);
                j.last_use = t_end;
                srv->done_lru.push_back(j.ticket);
                ++srv->st.completed;
            }
        }
        // stopping rule: estimate the jobs of this tick that continue
        est_jobs.clear();
        est_tickets.clear();
        est_n.clear();
        if (s == SOLRT_OK && e == cudaSuccess && srv->stop_rmse > 0.0f) {
            for (size_t i = 0; i < tick_tickets.size(); ++i) {
                ServerJob& j = srv->jobs[tick_tickets[i]];
                if (j.state != kActive || !j.sq || j.cancel || j.spp_done < srv->stop_min_spp) continue;
                est_jobs.push_back(jobs[i]);
                est_tickets.push_back(j.ticket);
                est_n.push_back(j.spp_done);
            }
        }
        if (!est_jobs.empty() && solrt::estimate_rmse(ctx, srv->tb, est_jobs, est_n, est_sum) == SOLRT_OK) {
            fin.clear();
            fin_tickets.clear();
            for (size_t i = 0; i < est_jobs.size(); ++i) {
                ServerJob& j = srv->jobs[est_tickets[i]];
                const double px = 3.0 * est_jobs[i].width * est_jobs[i].height;
                const double v = std::sqrt(est_sum[i] / px);
                j.rmse_est = (float)v;
                if (v <= (double)srv->stop_rmse) {  // converged: finalize with the samples it has
                    solrt_render_params q = j.p;
                    q.spp = j.spp_done;
                    const solrt::Scene& sc = *static_cast<solrt::Scene*>(j.scene);
                    const solrt::Image& img = *static_cast<solrt::Image*>(j.image);
                    fin.push_back(solrt::job_for(sc, img, j.cam, q));
                    fin_tickets.push_back(j.ticket);
                }
            }
            if (!fin.empty()) {
                const std::vector<solrt::DevJob> none_j;
                const std::vector<solrt::DevItem> none_i;
                const solrt::PassPlan none_p{0, 0, 0, 0, 0};
                const solrt_status fs = solrt::serve_tick(ctx, srv->tb, srv->kind, none_j, none_i, none_p, fin);
                const cudaError_t fe = cudaStreamSynchronize(ctx.stream);
                const uint64_t t_fin = now_ns();
                for (uint64_t t : fin_tickets) {
                    ServerJob& j = srv->jobs[t];
                    if (fs != SOLRT_OK || fe != cudaSuccess) {
                        j.state = kFailed;
                        j.status = fs != SOLRT_OK ? fs : SOLRT_ERR_DEVICE;
                        j.t_done = t_fin;
                        mark_finished(srv, j.ticket);
                        continue;
                    }
                    j.state = kDone;
                    j.status = SOLRT_OK;
                    j.stopped_early = true;
                    j.t_done = t_fin;
                    mark_finished(srv, j.ticket);
                    j.last_use = t_fin;
                    srv->done_lru.push_back(j.ticket);
                    ++srv->st.completed;
                    ++srv->st.stopped_early;
                }
            }
        }
        srv->active.erase(std::remove_if(srv->active.begin(), srv->active.end(),
                                         [&](uint64_t t) { return srv->jobs[t].state != kActive; }),
                          srv->active.end());
        srv->cv_done.notify_all();
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
}

void fill_result(const ServerJob& j, solrt_job_result* out) {
    out->status = j.status;
    out->spp_done = j.spp_done;
    out->latency_ns = j.t_done ? j.t_done - j.t_submit : 0;
    out->queue_ns = j.t_admit ? j.t_admit - j.t_submit : 0;
    out->image = j.image;
    out->rmse_estimate = j.rmse_est;
    out->stopped_early = j.stopped_early ? 1u : 0u;
}

}  // namespace

using solrt::set_error;

extern "C" {

solrt_status solrt_server_create(solrt_context* ctx, const solrt_server_desc* desc, solrt_server** out) {
    if (!ctx || !out) {
        set_error("null argument");
        return SOLRT_ERR_INVALID;
    }
    *out = nullptr;
    if (desc && desc->policy > SOLRT_SERVE_SHORTEST_FIRST) {
        set_error("unknown serving policy %u", desc->policy);
        return SOLRT_ERR_INVALID;
    }
    solrt_server* srv = new (std::nothrow) solrt_server();
    if (!srv) return SOLRT_ERR_OOM;
    srv->ctx = ctx;
    srv->budget = desc && desc->memory_budget ? desc->memory_budget : 150ull * 1000 * 1000 * 1000;
    // a fixed tick size, or adaptive ticks starting at 8M paths
    srv->adaptive = !(desc && desc->tick_paths);
    srv->tick_paths = desc && desc->tick_paths ? std::min(desc->tick_paths, ctx->capacity)
                                               : std::min(8u << 20, ctx->capacity);
    srv->tick_ms = desc && desc->tick_ms ? (double)desc->tick_ms : 40.0;
    if (desc && !(desc->stop_rmse >= 0.0f)) {
        delete srv;
        set_error("stop_rmse must be >= 0");
        return SOLRT_ERR_INVALID;
    }
    srv->stop_rmse = desc ? desc->stop_rmse : 0.0f;
    srv->stop_min_spp = desc && desc->stop_min_spp ? std::max(2u, desc->stop_min_spp) : 4u;
    srv->policy = desc ? desc->policy : (uint32_t)SOLRT_SERVE_FAIR;
    srv->inject_alloc_failures = desc ? desc->inject_alloc_failures : 0u;
    try {
        srv->th = std::thread(serve_loop, srv);
    } catch (...) {
        delete srv;
        set_error("cannot start the serving thread");
        return SOLRT_ERR_OOM;
    }
    *out = srv;
    return SOLRT_OK;
}

solrt_status solrt_server_submit(solrt_server* srv, solrt_scene* scene, const solrt_camera* camera,
                                 const solrt_render_params* params, uint64_t* ticket) {
    if (!srv || !scene || !camera || !params || !ticket) {
        set_error("null argument");
        return SOLRT_ERR_INVALID;
    }
    const solrt::Scene& sc = *static_cast<solrt::Scene*>(scene);
    if (sc.ctx != srv->ctx) {
        set_error("scene belongs to another context");
        return SOLRT_ERR_INVALID;
    }
    const solrt_render_params& p = *params;
    if (p.width == 0 || p.height == 0 || p.spp == 0 || p.max_bounces > SOLRT_MAX_BOUNCES ||
        p.kernel != SOLRT_KERNEL_WAVEFRONT || p.miss_mode > SOLRT_MISS_GRADIENT ||
        p.material_mode > SOLRT_MATERIAL_LAMBERT || p.rng_mode > SOLRT_RNG_PER_SAMPLE ||
        p.accum_mode > SOLRT_ACCUM_KAHAN || !(p.tmax >= 0.0f) ||
        (p.accum_mode != SOLRT_ACCUM_KAHAN && p.frame + 1u - p.accum_start_frame == 0u)) {
        set_error("invalid render parameters");
        return SOLRT_ERR_INVALID;
    }
    if ((p.integrator != SOLRT_INTEGRATOR_PATH && p.integrator != SOLRT_INTEGRATOR_PATH_NEE) ||
        (p.integrator == SOLRT_INTEGRATOR_PATH_NEE && p.material_mode != SOLRT_MATERIAL_LAMBERT)) {
        set_error("the server runs the path integrators (next-event estimation with Lambert materials)");
        return SOLRT_ERR_INVALID;
    }
    if ((uint64_t)p.width * p.height > srv->ctx->capacity) {
        set_error("job of %u x %u pixels exceeds the path capacity", p.width, p.height);
        return SOLRT_ERR_CAPACITY;
    }
    std::lock_guard<std::mutex> lock(srv->mu);
    if (!srv->kind_set) {
        srv->kind = sc.info.kind;
        srv->kind_set = true;
    } else if (sc.info.kind != srv->kind) {
        set_error("all scenes of a server need the same BVH kind");
        return SOLRT_ERR_INVALID;
    }
    if (p.integrator == SOLRT_INTEGRATOR_PATH_NEE) {  // before the serving thread can see the job
        const solrt_status s = solrt::ensure_shadow_queue(*srv->ctx);
        if (s != SOLRT_OK) return s;
    }
    ServerJob j;
    j.ticket = srv->next_ticket++;
    j.scene = scene;
    j.cam = *camera;
    j.p = p;
    j.t_submit = now_ns();
    srv->jobs[j.ticket] = j;
    srv->queue.push_back(j.ticket);
    ++srv->st.submitted;
    *ticket = j.ticket;
    srv->cv_work.notify_one();
    return SOLRT_OK;
}

solrt_status solrt_server_poll(solrt_server* srv, uint64_t ticket, solrt_job_result* out) {
    if (!srv || !out) {
        set_error("null argument");
        return SOLRT_ERR_INVALID;
    }
    std::lock_guard<std::mutex> lock(srv->mu);
    auto it = srv->jobs.find(ticket);
    if (it == srv->jobs.end()) {
        set_error("unknown, released or evicted ticket");
        return SOLRT_ERR_NOT_FOUND;
    }
    ServerJob& j = it->second;
    fill_result(j, out);
    if (j.state == kDone) {
        j.last_use = now_ns();
        srv->done_lru.remove(ticket);
        srv->done_lru.push_back(ticket);
        return SOLRT_OK;
    }
    if (j.state == kFailed) return (solrt_status)j.status;
    return SOLRT_ERR_NOT_READY;
}

solrt_status solrt_server_wait(solrt_server* srv, uint64_t ticket, uint32_t timeout_ms, solrt_job_result* out) {
    if (!srv || !out) {
        set_error("null argument");
        return SOLRT_ERR_INVALID;
    }
    {
        std::unique_lock<std::mutex> lock(srv->mu);
        srv->cv_done.wait_for(lock, std::chrono::milliseconds(timeout_ms), [&] {
            auto it = srv->jobs.find(ticket);
            return it == srv->jobs.end() || it->second.state == kDone || it->second.state == kFailed;
        });
    }
    const solrt_status s = solrt_server_poll(srv, ticket, out);
    if (s == SOLRT_ERR_NOT_READY) {
        set_error("ticket not complete within %u ms", timeout_ms);
        return SOLRT_ERR_TIMEOUT;
    }
    return s;
}

solrt_status solrt_server_release(solrt_server* srv, uint64_t ticket) {
    if (!srv) {
        set_error("null server");
        return SOLRT_ERR_INVALID;
    }
    std::lock_guard<std::mutex> lock(srv->mu);
    auto it = srv->jobs.find(ticket);
    if (it == srv->jobs.end()) return SOLRT_ERR_NOT_FOUND;
    ServerJob& j = it->second;
    if (j.state == kActive) {
        set_error("job still running");
        return SOLRT_ERR_NOT_READY;
    }
    if (j.state == kQueued) srv->queue.erase(std::find(srv->queue.begin(), srv->queue.end(), ticket));
    if (j.state == kDone) srv->done_lru.remove(ticket);
    drop_job_memory(srv, j);
    srv->jobs.erase(it);
    return SOLRT_OK;
}

solrt_status solrt_server_cancel(solrt_server* srv, uint64_t ticket) {
    if (!srv) {
        set_error("null server");
        return SOLRT_ERR_INVALID;
    }
    std::lock_guard<std::mutex> lock(srv->mu);
    auto it = srv->jobs.find(ticket);
    if (it == srv->jobs.end()) {
        set_error("unknown, released or evicted ticket");
        return SOLRT_ERR_NOT_FOUND;
    }
    ServerJob& j = it->second;
    if (j.state == kQueued) {
        srv->queue.erase(std::find(srv->queue.begin(), srv->queue.end(), ticket));
        j.state = kFailed;
        j.status = SOLRT_ERR_CANCELLED;
        j.t_done = now_ns();
        mark_finished(srv, j.ticket);
        srv->cv_done.notify_all();
        return SOLRT_OK;
    }
    if (j.state == kActive) {
        j.cancel = true;
        srv->cv_work.notify_all();
        return SOLRT_OK;
    }
    set_error("job already finished");
    return SOLRT_ERR_INVALID;
}

solrt_status solrt_server_finished(solrt_server* srv, uint64_t* tickets, uint32_t max, uint32_t* n) {
    if (!srv || !n || (max && !tickets)) {
        set_error("null argument");
        return SOLRT_ERR_INVALID;
    }
    std::lock_guard<std::mutex> lock(srv->mu);
    uint32_t k = 0;
    while (k < max && !srv->finished.empty()) {
        tickets[k++] = srv->finished.front();
        srv->finished.pop_front();
    }
    *n = k;
    return SOLRT_OK;
}

solrt_status solrt_server_get_stats(solrt_server* srv, solrt_server_stats* out) {
    if (!srv || !out) {
        set_error("null argument");
        return SOLRT_ERR_INVALID;
    }
    std::lock_guard<std::mutex> lock(srv->mu);
    *out = srv->st;
    out->queue_depth = (uint32_t)srv->queue.size();
    out->active = (uint32_t)srv->active.size();
    out->bytes_in_use = srv->bytes_in_use;
    solrt_stats cs;
    if (solrt_get_stats(srv->ctx, &cs) == SOLRT_OK) out->segments = cs.segments;
    return SOLRT_OK;
}

solrt_status solrt_server_destroy(solrt_server* srv) {
    if (!srv) return SOLRT_OK;
    {
        std::lock_guard<std::mutex> lock(srv->mu);
        srv->stop = true;
    }
    srv->cv_work.notify_all();
    if (srv->th.joinable()) srv->th.join();
    for (auto& kv : srv->jobs) {
        if (kv.second.image) solrt_image_destroy(kv.second.image);
        if (kv.second.sq) cudaFree(kv.second.sq);
    }
    delete srv;
    return SOLRT_OK;
}

}  // extern "C"
