// serve.cu — continuous-batching request loop over independent scenes.
//
// No counterpart in the reference (it simulates one scene per process).  A
// request is a scene (apic_scene_params + world properties), a step count
// and a frame dt.  Requests are admitted in arrival order while the scenes
// in the server (running or being prepared) are fewer than max_active and
// their estimated device memory fits the budget; the head of the queue waits
// rather than being overtaken.  An optional work limit also bounds the grid
// cells of the admitted scenes, so a mix of small scenes runs many at once
// and a mix of large ones few.  Two ways to run the admitted scenes:
//
//   continuous (default): every scene runs on its own stream and is
//     relaunched the moment its update completes, so short updates of small
//     scenes never wait for long ones and the GPU always holds every scene's
//     next update.  Admission work (generating the scene's particles,
//     allocating it, uploading, building its update graph) runs on
//     preparation threads while the GPU keeps running the other scenes.
//     apic_server_step returns once at least one update has completed.
//   rounds: apic_server_step admits (on the calling thread), runs one update
//     of every active scene (all enqueued before any is awaited) and returns
//     when all are done.  With max_active = 1 this is the plain path: one
//     scene at a time.
//
// Each scene computes exactly what it computes alone: the only shared
// resource is the GPU.  Scene buffers come from a stream-ordered pool, so a
// retired scene's memory is released without synchronising the device.
// Latency is recorded per update (launch to observed completion; in rounds
// mode the round's wall time) and per request (completion minus submission).
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <deque>
#include <map>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "apic_internal.h"

namespace {

using Clock = std::chrono::steady_clock;

struct Request {
    uint64_t id = 0;
    apic_scene_params scene{};
    apic_world_props props{};
    uint32_t steps = 0;
    float dt = 0.0f;
    int solver_mode = APIC_SOLVER_REL_MIXED;
    float rel_tol = 1e-6f;
    uint32_t max_iter = 500;
    double t_submit = 0, t_admit = -1, t_done = -1;  // ms since server creation
    double t_launch = 0;                             // launch of the running update
    bool in_flight = false;
    uint32_t done_steps = 0;
    uint64_t particles = 0, substeps = 0, pcg_iterations = 0;
    double max_true_residual = 0.0;
    double prepare_ms = 0.0;                         // host time to build the scene
    uint64_t bytes = 0;
    uint64_t cells = 0;                              // grid cells (admission work limit)
    apic_handle* h = nullptr;
    int status = APIC_OK;
    std::string error;
    std::vector<float> final_pos;  // Vec2x8 layout, when results are kept
};

double percentile(std::vector<double> v, double q) {
    if (v.empty()) return 0.0;
    std::sort(v.begin(), v.end());
    const double pos = q * double(v.size() - 1);
    const size_t i = size_t(pos);
    const double f = pos - double(i);
    return i + 1 < v.size() ? v[i] * (1.0 - f) + v[i + 1] * f : v[i];
}

// An update that has not completed after this long is reported as a timeout
// (apic_server_step returns APIC_ERR_TIMEOUT instead of waiting forever).
constexpr double kUpdateDeadlineMs = 120000.0;

struct SceneRule {
    int option, value;
    uint64_t min_cells, max_cells;
};

}  // namespace

struct apic_server {
    uint64_t budget = 0, used = 0, peak = 0;
    uint32_t max_active = 0;
    uint64_t max_cells = 0;          // grid cells of the admitted scenes at most (0: no limit)
    uint64_t active_cells = 0;
    bool keep = false;
    int mode = APIC_SERVER_CONTINUOUS;
    uint32_t workers = 4;
    int device = 0;
    Clock::time_point t0 = Clock::now();
    uint64_t next_id = 1;
    std::deque<Request*> queue;      // submitted, not admitted
    std::vector<Request*> active;    // on the GPU (or between updates in rounds mode)
    uint32_t pending = 0;            // admitted, being prepared (continuous mode)
    std::map<uint64_t, Request*> all;
    std::vector<SceneRule> rules;    // apic_set_option per scene size (read by the preparation threads)
    std::vector<double> step_ms, request_ms;
    uint64_t particle_substeps = 0, particle_updates = 0, rounds = 0, completed = 0, failed = 0, updates = 0;
    uint64_t kernels = 0;            // kernel launches of the completed updates
    double busy_ms = 0.0, prepare_ms = 0.0, host_ms = 0.0;

    // preparation threads (continuous mode)
    std::mutex mu;
    std::condition_variable cv_work, cv_ready;
    std::deque<Request*> to_prepare;  // guarded by mu
    std::vector<Request*> ready;      // guarded by mu
    std::atomic<uint32_t> n_ready{0};
    bool stop = false;                // guarded by mu
    std::vector<std::thread> pool;

    double now_ms() const { return std::chrono::duration<double, std::milli>(Clock::now() - t0).count(); }
};

namespace {

thread_local std::string g_err;

int bad(int code, const std::string& msg) {
    g_err = msg;
    apic::set_last_error(msg.c_str());
    return code;
}

// Build the request's scene: particles generated on the host, scene created
// on the device, solver and the size rules' options set, update graph built.
// Thread-safe: writes only the request (the preparation threads call it
// concurrently; the rules do not change while scenes are admitted).
int prepare(Request* r, const std::vector<SceneRule>& rules) {
    const auto t0 = Clock::now();
    const apic_scene_params& p = r->scene;
    apic_handle* h = nullptr;
    int rc = apic::create_scene(p.width, p.height, p.cell_size, &r->props, false, &h);
    if (rc == APIC_OK) {
        uint64_t n = 0;
        rc = apic_scene_count(&p, &n);
        if (rc == APIC_OK) {
            std::vector<float> px(n), py(n), vx(n), vy(n);
            rc = apic_scene_fill(&p, n, px.data(), py.data(), vx.data(), vy.data());
            if (rc == APIC_OK) rc = apic_set_particles(h, uint32_t(n), px.data(), py.data(), vx.data(), vy.data());
        }
        if (rc == APIC_OK) rc = apic_set_solver(h, r->solver_mode, r->rel_tol, r->max_iter);
        const uint64_t cells = uint64_t(p.width) * p.height;
        for (const SceneRule& q : rules)
            if (rc == APIC_OK && cells >= q.min_cells && cells <= q.max_cells) rc = apic_set_option(h, q.option, q.value);
        if (rc == APIC_OK) rc = apic::update_prepare(h);
        if (rc == APIC_OK) r->particles = n;
    }
    if (rc != APIC_OK) {
        r->error = apic_last_error();
        if (h) apic_destroy(h);
        h = nullptr;
    }
    r->h = h;
    r->status = rc;
    r->prepare_ms = std::chrono::duration<double, std::milli>(Clock::now() - t0).count();
    return rc;
}

void worker_loop(apic_server* sv) {
    cudaSetDevice(sv->device);
    for (;;) {
        Request* r = nullptr;
        {
            std::unique_lock<std::mutex> lock(sv->mu);
            sv->cv_work.wait(lock, [&] { return sv->stop || !sv->to_prepare.empty(); });
            if (sv->stop) return;
            r = sv->to_prepare.front();
            sv->to_prepare.pop_front();
        }
        prepare(r, sv->rules);
        {
            std::lock_guard<std::mutex> lock(sv->mu);
            sv->ready.push_back(r);
            sv->n_ready.fetch_add(1, std::memory_order_release);
        }
        sv->cv_ready.notify_all();
    }
}

void start_workers(apic_server* sv) {
    if (!sv->pool.empty() || sv->workers == 0) return;
    for (uint32_t i = 0; i < sv->workers; ++i) sv->pool.emplace_back(worker_loop, sv);
}

void stop_workers(apic_server* sv) {
    {
        std::lock_guard<std::mutex> lock(sv->mu);
        sv->stop = true;
    }
    sv->cv_work.notify_all();
    for (auto& t : sv->pool) t.join();
    sv->pool.clear();
}

void release(apic_server* sv, Request* r) {
    if (r->h) apic_destroy(r->h);
    r->h = nullptr;
    sv->used -= r->bytes;
    sv->active_cells -= r->cells;
}

// The head of the queue fits the work limit (a lone request always does).
bool fits_work(const apic_server* sv, const Request* r) {
    return sv->max_cells == 0 || sv->active_cells == 0 || sv->active_cells + r->cells <= sv->max_cells;
}

void retire(apic_server* sv, Request* r, int status) {
    r->status = status;
    r->in_flight = false;
    if (status == APIC_OK && sv->keep && r->h) {
        apic_info info{};
        if (apic_get_info(r->h, &info) == APIC_OK) {
            r->final_pos.resize(size_t(info.num_chunks) * 16);
            if (apic_read_vec2x8(r->h, 0, r->final_pos.data(), r->final_pos.size()) != APIC_OK) r->final_pos.clear();
        }
    }
    release(sv, r);
    r->t_done = sv->now_ms();
    if (status == APIC_OK) {
        sv->completed++;
        sv->request_ms.push_back(r->t_done - r->t_submit);
    } else {
        sv->failed++;
    }
}

// Statistics of a completed update of r.
void account(apic_server* sv, Request* r) {
    apic_step_stats st{};
    apic_get_stats(r->h, &st);
    r->done_steps++;
    r->substeps += st.substeps;
    r->pcg_iterations += st.pcg_iterations_total;
    r->max_true_residual = std::max(r->max_true_residual, st.true_residual_rel);
    sv->particle_substeps += r->particles * st.substeps;
    sv->particle_updates += r->particles;
    sv->updates++;
    sv->kernels += st.kernel_launches;
}

// ---- rounds mode -----------------------------------------------------------

int step_rounds(apic_server* sv, apic_server_round& rd) {
    // 1. admission in arrival order, on the calling thread
    while (!sv->queue.empty() && sv->active.size() < sv->max_active &&
           sv->used + sv->queue.front()->bytes <= sv->budget && fits_work(sv, sv->queue.front())) {
        Request* r = sv->queue.front();
        sv->queue.pop_front();
        r->t_admit = sv->now_ms();
        int rc = prepare(r, sv->rules);
        sv->prepare_ms += r->prepare_ms;
        if (rc != APIC_OK) {
            r->t_done = sv->now_ms();
            sv->failed++;
            continue;
        }
        sv->used += r->bytes;
        sv->active_cells += r->cells;
        sv->peak = std::max(sv->peak, sv->used);
        sv->active.push_back(r);
        rd.admitted++;
    }
    // 2. one update of every active scene, enqueued before any is awaited
    const double t_start = sv->now_ms();
    std::vector<int> rc(sv->active.size(), APIC_OK);
    for (size_t i = 0; i < sv->active.size(); ++i) rc[i] = apic::update_launch(sv->active[i]->h, 0u, sv->active[i]->dt);
    for (size_t i = 0; i < sv->active.size(); ++i) {
        if (rc[i] == APIC_OK) rc[i] = apic::update_finish(sv->active[i]->h);
        if (rc[i] == APIC_OK) account(sv, sv->active[i]);
    }
    const double t_end = sv->now_ms();
    rd.round_ms = t_end - t_start;
    if (!sv->active.empty()) {
        sv->busy_ms += rd.round_ms;
        sv->rounds++;
    }
    // 3. retirement
    std::vector<Request*> still;
    for (size_t i = 0; i < sv->active.size(); ++i) {
        Request* r = sv->active[i];
        if (rc[i] != APIC_OK) {
            retire(sv, r, rc[i]);
            rd.completed++;
            continue;
        }
        rd.stepped++;
        sv->step_ms.push_back(rd.round_ms);
        if (r->done_steps >= r->steps) {
            retire(sv, r, APIC_OK);
            rd.completed++;
        } else {
            still.push_back(r);
        }
    }
    sv->active.swap(still);
    return APIC_OK;
}

// ---- continuous mode -------------------------------------------------------

void launch(apic_server* sv, Request* r, apic_server_round& rd) {
    int rc = apic::update_launch(r->h, 0u, r->dt);
    r->t_launch = sv->now_ms();
    if (rc == APIC_OK) {
        r->in_flight = true;
    } else {
        retire(sv, r, rc);
        rd.completed++;
    }
}

// Scenes the preparation threads finished: failed ones are dropped, the
// others join the active set and launch their first update.
void take_ready(apic_server* sv, apic_server_round& rd) {
    if (sv->n_ready.load(std::memory_order_acquire) == 0) return;
    std::vector<Request*> got;
    {
        std::lock_guard<std::mutex> lock(sv->mu);
        got.swap(sv->ready);
        sv->n_ready.store(0, std::memory_order_relaxed);
    }
    for (Request* r : got) {
        sv->pending--;
        sv->prepare_ms += r->prepare_ms;
        if (r->status != APIC_OK) {
            sv->used -= r->bytes;
            sv->active_cells -= r->cells;
            r->t_done = sv->now_ms();
            sv->failed++;
            continue;
        }
        sv->active.push_back(r);
        launch(sv, r, rd);
    }
}

void admit_continuous(apic_server* sv, apic_server_round& rd) {
    bool any = false;
    while (!sv->queue.empty() && sv->active.size() + sv->pending < sv->max_active &&
           sv->used + sv->queue.front()->bytes <= sv->budget && fits_work(sv, sv->queue.front())) {
        Request* r = sv->queue.front();
        sv->queue.pop_front();
        r->t_admit = sv->now_ms();
        sv->used += r->bytes;  // reserved from admission on
        sv->active_cells += r->cells;
        sv->peak = std::max(sv->peak, sv->used);
        sv->pending++;
        rd.admitted++;
        if (sv->workers == 0) {
            prepare(r, sv->rules);
            std::lock_guard<std::mutex> lock(sv->mu);
            sv->ready.push_back(r);
            sv->n_ready.fetch_add(1, std::memory_order_release);
        } else {
            std::lock_guard<std::mutex> lock(sv->mu);
            sv->to_prepare.push_back(r);
            any = true;
        }
    }
    if (any) sv->cv_work.notify_all();
}

int step_continuous(apic_server* sv, apic_server_round& rd) {
    start_workers(sv);
    admit_continuous(sv, rd);
    const double t_start = sv->now_ms();
    take_ready(sv, rd);
    // drop scenes retired by a failed launch
    sv->active.erase(std::remove_if(sv->active.begin(), sv->active.end(), [](Request* r) { return !r->h; }),
                     sv->active.end());
    int result = APIC_OK;
    while (!sv->active.empty() || sv->pending > 0) {
        uint32_t done = 0;
        for (Request* r : sv->active) {
            if (!r->in_flight) continue;
            cudaError_t q = cudaStreamQuery(apic::scene_stream(r->h));
            if (q == cudaErrorNotReady) {
                if (sv->now_ms() - r->t_launch > kUpdateDeadlineMs) {
                    result = bad(APIC_ERR_TIMEOUT, "apic_server_step: an update did not complete in time");
                    break;
                }
                continue;
            }
            // completed (or failed: update_finish reports the error)
            r->in_flight = false;
            const double t = sv->now_ms();
            int rc = apic::update_finish(r->h);
            done++;
            if (rc != APIC_OK) {
                retire(sv, r, rc);
                rd.completed++;
                continue;
            }
            account(sv, r);
            rd.stepped++;
            sv->step_ms.push_back(t - r->t_launch);
            if (r->done_steps >= r->steps) {
                retire(sv, r, APIC_OK);
                rd.completed++;
            } else {
                launch(sv, r, rd);
            }
        }
        sv->active.erase(std::remove_if(sv->active.begin(), sv->active.end(), [](Request* r) { return !r->h; }),
                         sv->active.end());
        if (result != APIC_OK || done > 0) break;
        take_ready(sv, rd);
        if (sv->active.empty() && sv->pending > 0) {
            // nothing on the GPU yet: wait for a preparation thread
            std::unique_lock<std::mutex> lock(sv->mu);
            sv->cv_ready.wait_for(lock, std::chrono::milliseconds(1),
                                  [&] { return sv->n_ready.load(std::memory_order_acquire) > 0; });
        } else {
            std::this_thread::yield();
        }
    }
    const double t_end = sv->now_ms();
    rd.round_ms = t_end - t_start;
    if (rd.stepped || !sv->active.empty()) {
        sv->busy_ms += rd.round_ms;
        sv->rounds++;
    }
    return result;
}

}  // namespace

extern "C" {

int apic_scene_bytes(uint32_t width, uint32_t height, uint64_t particles, uint64_t* out) {
    if (!out || width == 0 || height == 0) return bad(APIC_ERR_INVALID_ARG, "apic_scene_bytes: bad argument");
    const uint64_t cells = uint64_t(width) * height;
    const uint64_t faces = uint64_t(width + 1) * height + uint64_t(width) * (height + 1);
    const uint64_t lanes = (particles + 7) / 8 * 8;
    // particles: two sets of 9 fields, Morton sort and P2G binning keys and
    // slots (two each), Vec2x8 staging, sort scratch; faces: accumulators,
    // velocities, forces, masks; cells: the base pressure system (padded,
    // FP32 and FP64 vectors), smoothing, P2G bin bounds and multigrid levels
    // (a third of the base); plus control blocks and allocation granularity.
    *out = lanes * 148 + faces * 48 + cells * 168 + (24ull << 20);
    return APIC_OK;
}

int apic_place_scenes(const uint64_t* bytes, const uint64_t* work, uint32_t count, const uint64_t* budgets,
                      uint32_t devices, int32_t* device_out) {
    if (count == 0) return APIC_OK;
    if (!bytes || !work || !budgets || !device_out || devices == 0)
        return bad(APIC_ERR_INVALID_ARG, "apic_place_scenes: bad argument");
    std::vector<uint32_t> order(count);
    for (uint32_t i = 0; i < count; ++i) order[i] = i;
    std::stable_sort(order.begin(), order.end(), [&](uint32_t a, uint32_t b) { return bytes[a] > bytes[b]; });
    std::vector<uint64_t> used(devices, 0), load(devices, 0);
    for (uint32_t i : order) {
        int32_t best = -1;
        for (uint32_t d = 0; d < devices; ++d) {
            if (budgets[d] < used[d] || bytes[i] > budgets[d] - used[d]) continue;
            if (best < 0 || load[d] < load[uint32_t(best)]) best = int32_t(d);
        }
        device_out[i] = best;
        if (best >= 0) {
            used[uint32_t(best)] += bytes[i];
            load[uint32_t(best)] += work[i];
        }
    }
    return APIC_OK;
}

int apic_server_create(uint64_t memory_budget_bytes, uint32_t max_active, uint32_t keep_results, apic_server** out) {
    if (!out || max_active == 0) return bad(APIC_ERR_INVALID_ARG, "apic_server_create: bad argument");
    apic_server* sv = new apic_server();
    sv->budget = memory_budget_bytes;
    sv->max_active = max_active;
    sv->keep = keep_results != 0;
    if (cudaGetDevice(&sv->device) != cudaSuccess) sv->device = 0;
    *out = sv;
    return APIC_OK;
}

int apic_server_set_mode(apic_server* sv, int mode, uint32_t prepare_threads) {
    if (!sv || (mode != APIC_SERVER_ROUNDS && mode != APIC_SERVER_CONTINUOUS) || prepare_threads > 64)
        return bad(APIC_ERR_INVALID_ARG, "apic_server_set_mode: bad argument");
    if (!sv->active.empty() || sv->pending > 0)
        return bad(APIC_ERR_INVALID_ARG, "apic_server_set_mode: scenes are running");
    stop_workers(sv);
    {
        std::lock_guard<std::mutex> lock(sv->mu);
        sv->stop = false;
    }
    sv->mode = mode;
    sv->workers = prepare_threads;
    return APIC_OK;
}

int apic_server_scene_option(apic_server* sv, int option, int value, uint64_t min_cells, uint64_t max_cells) {
    if (!sv || min_cells > max_cells) return bad(APIC_ERR_INVALID_ARG, "apic_server_scene_option: bad argument");
    if (option != APIC_OPT_PDL && option != APIC_OPT_DSM_VCYCLE && option != APIC_OPT_WARM_START &&
        option != APIC_OPT_STREAM_PRIORITY && option != APIC_OPT_P2G_ORDER)
        return bad(APIC_ERR_INVALID_ARG, "apic_server_scene_option: unknown option");
    if (!sv->active.empty() || sv->pending > 0)
        return bad(APIC_ERR_INVALID_ARG, "apic_server_scene_option: scenes are running");
    sv->rules.push_back(SceneRule{option, value, min_cells, max_cells});
    return APIC_OK;
}

int apic_server_set_work_limit(apic_server* sv, uint64_t max_active_cells) {
    if (!sv) return bad(APIC_ERR_INVALID_ARG, "apic_server_set_work_limit: null server");
    sv->max_cells = max_active_cells;
    return APIC_OK;
}

int apic_server_destroy(apic_server* sv) {
    if (!sv) return APIC_OK;
    stop_workers(sv);
    // scenes still on the GPU finish their update before their memory goes
    for (auto& kv : sv->all) {
        if (kv.second->h) apic_destroy(kv.second->h);
        delete kv.second;
    }
    delete sv;
    return APIC_OK;
}

int apic_server_submit(apic_server* sv, const apic_scene_params* scene, const apic_world_props* props,
                       uint32_t steps, float frame_dt, int solver_mode, float rel_tol, uint32_t max_iterations,
                       uint64_t* id_out) {
    if (!sv || !scene || !props || !id_out || steps == 0 || !(frame_dt > 0.0f))
        return bad(APIC_ERR_INVALID_ARG, "apic_server_submit: bad argument");
    uint64_t n = 0;
    int rc = apic_scene_count(scene, &n);
    if (rc != APIC_OK) return rc;
    Request* r = new Request();
    r->id = sv->next_id++;
    r->scene = *scene;
    r->props = *props;
    r->steps = steps;
    r->dt = frame_dt;
    r->solver_mode = solver_mode;
    r->rel_tol = rel_tol;
    r->max_iter = max_iterations;
    r->t_submit = sv->now_ms();
    r->cells = uint64_t(scene->width) * scene->height;
    apic_scene_bytes(scene->width, scene->height, n, &r->bytes);
    if (r->bytes > sv->budget) {
        delete r;
        return bad(APIC_ERR_OOM, "apic_server_submit: the scene alone exceeds the memory budget");
    }
    sv->all[r->id] = r;
    sv->queue.push_back(r);
    *id_out = r->id;
    return APIC_OK;
}

int apic_server_step(apic_server* sv, apic_server_round* out) {
    if (!sv) return bad(APIC_ERR_INVALID_ARG, "apic_server_step: null server");
    const double t_call = sv->now_ms();
    apic_server_round rd{};
    int rc = sv->mode == APIC_SERVER_ROUNDS ? step_rounds(sv, rd) : step_continuous(sv, rd);
    sv->host_ms += sv->now_ms() - t_call - rd.round_ms;
    rd.active = uint32_t(sv->active.size() + sv->pending);
    rd.queued = uint32_t(sv->queue.size());
    rd.memory_used = sv->used;
    if (out) *out = rd;
    return rc;
}

int apic_server_request(apic_server* sv, uint64_t id, apic_request_info* out) {
    if (!sv || !out) return bad(APIC_ERR_INVALID_ARG, "apic_server_request: bad argument");
    auto it = sv->all.find(id);
    if (it == sv->all.end()) return bad(APIC_ERR_INVALID_ARG, "apic_server_request: unknown request");
    const Request* r = it->second;
    apic_request_info info{};
    info.status = r->status;
    info.finished = r->t_done >= 0.0 ? 1u : 0u;
    info.steps_done = r->done_steps;
    info.particles = r->particles;
    info.substeps = r->substeps;
    info.pcg_iterations = r->pcg_iterations;
    info.max_true_residual = r->max_true_residual;
    info.submit_ms = r->t_submit;
    info.admit_ms = r->t_admit;
    info.done_ms = r->t_done;
    info.bytes = r->bytes;
    info.result_floats = r->final_pos.size();
    *out = info;
    return APIC_OK;
}

int apic_server_result_positions(apic_server* sv, uint64_t id, float* dst, uint64_t floats) {
    if (!sv) return bad(APIC_ERR_INVALID_ARG, "apic_server_result_positions: null server");
    auto it = sv->all.find(id);
    if (it == sv->all.end()) return bad(APIC_ERR_INVALID_ARG, "apic_server_result_positions: unknown request");
    const Request* r = it->second;
    if (r->final_pos.empty()) return bad(APIC_ERR_INVALID_ARG, "apic_server_result_positions: no kept result");
    if (floats != r->final_pos.size() || !dst) return bad(APIC_ERR_INVALID_ARG, "apic_server_result_positions: size");
    std::copy(r->final_pos.begin(), r->final_pos.end(), dst);
    return APIC_OK;
}

int apic_server_get_stats(apic_server* sv, apic_server_stats* out) {
    if (!sv || !out) return bad(APIC_ERR_INVALID_ARG, "apic_server_get_stats: bad argument");
    apic_server_stats st{};
    st.submitted = sv->next_id - 1;
    st.completed = sv->completed;
    st.failed = sv->failed;
    st.active = sv->active.size() + sv->pending;
    st.queued = sv->queue.size();
    st.rounds = sv->rounds;
    st.particle_substeps = sv->particle_substeps;
    st.particle_updates = sv->particle_updates;
    st.busy_ms = sv->busy_ms;
    st.elapsed_ms = sv->now_ms();
    st.step_p50_ms = percentile(sv->step_ms, 0.50);
    st.step_p99_ms = percentile(sv->step_ms, 0.99);
    st.request_p50_ms = percentile(sv->request_ms, 0.50);
    st.request_p99_ms = percentile(sv->request_ms, 0.99);
    st.memory_used = sv->used;
    st.memory_peak = sv->peak;
    st.updates = sv->updates;
    st.prepare_ms = sv->prepare_ms;
    st.host_ms = sv->host_ms;
    st.mode = sv->mode;
    st.prepare_threads = sv->workers;
    st.kernel_launches = sv->kernels;
    *out = st;
    return APIC_OK;
}

}  // extern "C"
