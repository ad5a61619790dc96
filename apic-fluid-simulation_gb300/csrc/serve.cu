// serve.cu — continuous-batching request loop over independent scenes.
//
// No counterpart in the reference (it simulates one scene per process).  A
// request is a scene (apic_scene_params + world properties), a step count
// and a frame dt.  apic_server_step runs one round:
//   1. admission: queued requests enter in arrival order while the active set
//      is below max_active and their estimated device memory fits the budget
//      (the head of the queue waits rather than being overtaken);
//   2. one update of every active scene: all updates are enqueued on the
//      scenes' own streams first, then all are completed, so the GPU runs
//      the scenes' kernels side by side (each update is one CUDA-graph launch
//      of the single-scene path);
//   3. retirement: scenes that reached their step count are destroyed and
//      their memory returns to the budget.
// Latency is recorded per step (the wall time of the round the step ran in)
// and per request (completion minus submission).  The scenes' state stays on
// the device between rounds.  Each scene computes exactly what it computes
// alone: the only shared resource is the GPU.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <deque>
#include <map>
#include <string>
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
    uint32_t done_steps = 0;
    uint64_t particles = 0, substeps = 0, pcg_iterations = 0;
    double max_true_residual = 0.0;
    uint64_t bytes = 0;
    apic_handle* h = nullptr;
    int status = APIC_OK;
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

}  // namespace

struct apic_server {
    uint64_t budget = 0, used = 0, peak = 0;
    uint32_t max_active = 0;
    bool keep = false;
    Clock::time_point t0 = Clock::now();
    uint64_t next_id = 1;
    std::deque<Request*> queue;
    std::vector<Request*> active;
    std::map<uint64_t, Request*> all;
    std::vector<double> step_ms, request_ms;
    uint64_t particle_substeps = 0, particle_updates = 0, rounds = 0, completed = 0, failed = 0;
    double busy_ms = 0.0;

    double now_ms() const { return std::chrono::duration<double, std::milli>(Clock::now() - t0).count(); }
    ~apic_server() {
        for (auto& kv : all) {
            if (kv.second->h) apic_destroy(kv.second->h);
            delete kv.second;
        }
    }
};

namespace {

thread_local std::string g_err;

int bad(int code, const std::string& msg) {
    g_err = msg;
    apic::set_last_error(msg.c_str());
    return code;
}

// Create the request's scene on the device.
int admit(apic_server* sv, Request* r) {
    const apic_scene_params& p = r->scene;
    apic_handle* h = nullptr;
    int rc = apic::create_scene(p.width, p.height, p.cell_size, &r->props, false, &h);
    if (rc != APIC_OK) return rc;
    uint64_t n = 0;
    rc = apic_scene_count(&p, &n);
    if (rc == APIC_OK) {
        std::vector<float> px(n), py(n), vx(n), vy(n);
        rc = apic_scene_fill(&p, n, px.data(), py.data(), vx.data(), vy.data());
        if (rc == APIC_OK) rc = apic_set_particles(h, uint32_t(n), px.data(), py.data(), vx.data(), vy.data());
    }
    if (rc == APIC_OK) rc = apic_set_solver(h, r->solver_mode, r->rel_tol, r->max_iter);
    if (rc != APIC_OK) {
        apic_destroy(h);
        return rc;
    }
    r->h = h;
    r->particles = n;
    r->t_admit = sv->now_ms();
    sv->used += r->bytes;
    sv->peak = std::max(sv->peak, sv->used);
    return APIC_OK;
}

void retire(apic_server* sv, Request* r, int status) {
    r->status = status;
    if (status == APIC_OK && sv->keep && r->h) {
        apic_info info{};
        if (apic_get_info(r->h, &info) == APIC_OK) {
            r->final_pos.resize(size_t(info.num_chunks) * 16);
            if (apic_read_vec2x8(r->h, 0, r->final_pos.data(), r->final_pos.size()) != APIC_OK) r->final_pos.clear();
        }
    }
    if (r->h) apic_destroy(r->h);
    r->h = nullptr;
    sv->used -= r->bytes;
    r->t_done = sv->now_ms();
    if (status == APIC_OK) {
        sv->completed++;
        sv->request_ms.push_back(r->t_done - r->t_submit);
    } else {
        sv->failed++;
    }
}

}  // namespace

extern "C" {

int apic_scene_bytes(uint32_t width, uint32_t height, uint64_t particles, uint64_t* out) {
    if (!out || width == 0 || height == 0) return bad(APIC_ERR_INVALID_ARG, "apic_scene_bytes: bad argument");
    const uint64_t cells = uint64_t(width) * height;
    const uint64_t faces = uint64_t(width + 1) * height + uint64_t(width) * (height + 1);
    const uint64_t lanes = (particles + 7) / 8 * 8;
    // particles: two sets of 9 fields, sort keys and slots (two each), Vec2x8
    // staging, sort scratch; faces: accumulators, velocities, forces, masks;
    // cells: the base pressure system (padded, FP32 and FP64 vectors),
    // smoothing and multigrid levels (a third of the base); plus control
    // blocks and allocation granularity.  Measured footprints of scenes from
    // 64^2 to 2048^2 (3 k to 6.7 M particles) stay below this bound.
    *out = lanes * 128 + faces * 48 + cells * 160 + (24ull << 20);
    return APIC_OK;
}

int apic_server_create(uint64_t memory_budget_bytes, uint32_t max_active, uint32_t keep_results, apic_server** out) {
    if (!out || max_active == 0) return bad(APIC_ERR_INVALID_ARG, "apic_server_create: bad argument");
    apic_server* sv = new apic_server();
    sv->budget = memory_budget_bytes;
    sv->max_active = max_active;
    sv->keep = keep_results != 0;
    *out = sv;
    return APIC_OK;
}

int apic_server_destroy(apic_server* sv) {
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
    apic_server_round rd{};
    // 1. admission in arrival order
    while (!sv->queue.empty() && sv->active.size() < sv->max_active &&
           sv->used + sv->queue.front()->bytes <= sv->budget) {
        Request* r = sv->queue.front();
        sv->queue.pop_front();
        int rc = admit(sv, r);
        if (rc != APIC_OK) {
            r->status = rc;
            r->t_done = sv->now_ms();
            sv->failed++;
            continue;
        }
        sv->active.push_back(r);
        rd.admitted++;
    }
    // 2. one update of every active scene, enqueued before any is awaited
    const double t_start = sv->now_ms();
    std::vector<int> rc(sv->active.size(), APIC_OK);
    for (size_t i = 0; i < sv->active.size(); ++i) rc[i] = apic::update_launch(sv->active[i]->h, 0u, sv->active[i]->dt);
    for (size_t i = 0; i < sv->active.size(); ++i) {
        Request* r = sv->active[i];
        if (rc[i] == APIC_OK) rc[i] = apic::update_finish(r->h);
        if (rc[i] == APIC_OK) {
            apic_step_stats st{};
            apic_get_stats(r->h, &st);
            r->done_steps++;
            r->substeps += st.substeps;
            r->pcg_iterations += st.pcg_iterations_total;
            r->max_true_residual = std::max(r->max_true_residual, st.true_residual_rel);
            sv->particle_substeps += r->particles * st.substeps;
            sv->particle_updates += r->particles;
        }
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
    rd.active = uint32_t(sv->active.size());
    rd.queued = uint32_t(sv->queue.size());
    rd.memory_used = sv->used;
    if (out) *out = rd;
    return APIC_OK;
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
    st.active = sv->active.size();
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
    *out = st;
    return APIC_OK;
}

}  // extern "C"
