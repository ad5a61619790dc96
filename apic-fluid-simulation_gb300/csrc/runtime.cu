// runtime.cu — scene lifetime, the substep loop and the C-ABI (include/apic_gpu.h).
//
// Apic::new (src/apic.rs:779-916) becomes apic_create: all grids, the solid
// border, the reference's default particle block, the multigrid hierarchy
// (halve while both sides are even and > 4, :900-908) and the open-face masks
// (update_world, :918-944) are set up on the device.  Apic::update
// (:2429-2474) becomes apic_update: the CFL substep size is computed on the
// device from the max speed that the previous G2P reduced, and every substep
// runs the stage kernels in the reference's order on the handle's stream.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <new>
#include <string>
#include <vector>

#include "apic_device.cuh"
#include "apic_graph.h"
#include "apic_internal.h"
#include "substep.cuh"

using namespace apic;

struct apic_handle {
    Scene s;
    std::vector<uint32_t> obstacle_host;  // u32 words
};

namespace {

thread_local std::string g_last_error = "";

int fail(int code, const std::string& msg) {
    g_last_error = msg;
    return code;
}

#define CK(call)                                                                                  \
    do {                                                                                          \
        cudaError_t e_ = (call);                                                                  \
        if (e_ != cudaSuccess) return fail(APIC_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

// ---- device control kernels ---------------------------------------------

__global__ void k_begin_update(Ctl* ctl, float frame_dt, uint32_t flags, uint32_t has_ext, uint32_t has_post) {
    ctl->frame_dt = frame_dt;
    ctl->t = 0.0f;
    ctl->flags = flags;
    ctl->substeps = 0;
    ctl->pcg_iters_total = 0;
    ctl->not_converged = 0;
    ctl->has_ext = has_ext;
    ctl->has_post = has_post;
    ctl->status = 0;
    ctl->pcg_done = 0;
    ctl->refinements_total = 0;
    ctl->sorted = 0;
    ctl->solve_ns = 0;
}

__global__ void k_plan_first(Ctl* ctl) { plan(ctl); }
__global__ void k_advance(Ctl* ctl) { advance(ctl); }

// Graph forms: the same planning, then the loop / sort conditions.
__global__ void k_plan_first_g(Ctl* ctl, cudaGraphConditionalHandle h_sort, cudaGraphConditionalHandle h_loop) {
    plan(ctl);
    cudaGraphSetConditional(h_sort, (ctl->go && ctl->sort_now) ? 1u : 0u);
    cudaGraphSetConditional(h_loop, ctl->go ? 1u : 0u);
}
__global__ void k_advance_g(Ctl* ctl, cudaGraphConditionalHandle h_loop) {
    advance(ctl);
    cudaGraphSetConditional(h_loop, ctl->go ? 1u : 0u);
}

__global__ void k_set_dt(Ctl* ctl, float dt, uint32_t has_ext, uint32_t has_post) {
    ctl->dt = dt;
    ctl->has_ext = has_ext;
    ctl->has_post = has_post;
}

__global__ void k_stage_finish(Ctl* ctl, float dt) {
    ctl->prev_dt = dt;
    ctl->timestamp += 1;
}

// add_radial_force, src/apic.rs:2352-2410: one thread per (x, y) of the box.
__device__ __forceinline__ int sat_i32(float v) {  // Rust `as i32`: saturating, NaN -> 0
    if (!(v == v)) return 0;
    if (v >= 2147483647.0f) return INT_MAX;
    if (v <= -2147483648.0f) return INT_MIN;
    return int(v);
}
__global__ void k_radial_force(int W, int H, float cs, float wx, float wy, float radius, float strength, uint32_t x0,
                               uint32_t y0, uint32_t nx, uint32_t ny, float* __restrict__ ext_u,
                               float* __restrict__ ext_v, float* __restrict__ post_u, float* __restrict__ post_v) {
    uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nx * ny) return;
    uint32_t x = x0 + k % nx, y = y0 + k / nx;
    float r2 = radius * radius;
    bool repel = strength > 0.0f;
    if (x <= uint32_t(W) && y < uint32_t(H)) {
        float dx = float(x) * cs - wx, dy = (float(y) + 0.5f) * cs - wy;
        float d2 = dx * dx + dy * dy;
        if (d2 < r2 && d2 > 1e-5f) {
            float d = sqrtf(d2);
            float fall = 1.0f - (d / radius);
            float force = (dx / d) * strength * fall;
            uint32_t ui = u_index(int(x), int(y), W, H);
            float* f = repel ? post_u : ext_u;
            f[ui] = f[ui] + force;
        }
    }
    if (x < uint32_t(W) && y <= uint32_t(H)) {
        float dx = (float(x) + 0.5f) * cs - wx, dy = float(y) * cs - wy;
        float d2 = dx * dx + dy * dy;
        if (d2 < r2 && d2 > 1e-5f) {
            float d = sqrtf(d2);
            float fall = 1.0f - (d / radius);
            float force = (dy / d) * strength * fall;
            uint32_t vi = v_index(int(x), int(y), W, H);
            float* f = repel ? post_v : ext_v;
            f[vi] = f[vi] + force;
        }
    }
}
__global__ void k_force_box(float wx, float wy, float radius, float cs, int W, int H, uint32_t* box) {
    int mnx = max(sat_i32(floorf((wx - radius) / cs)), 0);
    int mxx = min(sat_i32(ceilf((wx + radius) / cs)), W);
    int mny = max(sat_i32(floorf((wy - radius) / cs)), 0);
    int mxy = min(sat_i32(ceilf((wy + radius) / cs)), H);
    box[0] = uint32_t(mnx); box[1] = uint32_t(mxx); box[2] = uint32_t(mny); box[3] = uint32_t(mxy);
}

// ---- host helpers ---------------------------------------------------------

// Scene buffers come from a stream-ordered memory pool of the library's own
// (one per CUDA context, kept for the life of that context), allocated and
// released in order on the scene's stream.  Releasing them does not
// synchronise the whole device the way cudaFree does, so a scene retired
// while others run (the request server) never stalls the scenes still on the
// GPU; the pool keeps released memory for the next scene (no release
// threshold).  The pool is found by the current context's unique id, not by
// the device number: after cudaDeviceReset, or under a caller's own context,
// a pool made for an earlier context is never handed out.
struct PoolEntry {
    unsigned long long ctx;
    cudaMemPool_t pool;
};
std::mutex g_pool_mutex;
std::vector<PoolEntry> g_pools;

cudaError_t scene_pool(cudaMemPool_t* out) {
    unsigned long long ctx = 0;
    cudaError_t e = apic::current_context_key(&ctx);
    if (e != cudaSuccess) return e;
    int dev = 0;
    if ((e = cudaGetDevice(&dev)) != cudaSuccess) return e;
    std::lock_guard<std::mutex> lock(g_pool_mutex);
    for (const PoolEntry& p : g_pools)
        if (p.ctx == ctx) {
            *out = p.pool;
            return cudaSuccess;
        }
    cudaMemPoolProps props = {};
    props.allocType = cudaMemAllocationTypePinned;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = dev;
    cudaMemPool_t pool = nullptr;
    if ((e = cudaMemPoolCreate(&pool, &props)) != cudaSuccess) return e;
    uint64_t keep = ~0ull;
    if ((e = cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep)) != cudaSuccess) {
        cudaMemPoolDestroy(pool);
        return e;
    }
    g_pools.push_back({ctx, pool});
    *out = pool;
    return cudaSuccess;
}

// Zeroed device buffer of `count` T, in stream order on st: use it from
// another stream only after st has been synchronised.
template <class T> cudaError_t dalloc(T** p, size_t count, cudaStream_t st) {
    *p = nullptr;
    if (count == 0) count = 1;
    cudaMemPool_t pool = nullptr;
    cudaError_t e = scene_pool(&pool);
    if (e != cudaSuccess) return e;
    e = cudaMallocFromPoolAsync(reinterpret_cast<void**>(p), sizeof(T) * count, pool, st);
    if (e != cudaSuccess) return e;
    return cudaMemsetAsync(*p, 0, sizeof(T) * count, st);
}
template <class T> void dfree(T*& p, cudaStream_t st) {
    if (p) cudaFreeAsync(p, st);
    p = nullptr;
}

// Pinned host mirrors of the control blocks come from a process-wide free
// list, for the same reason: cudaFreeHost synchronises the device.
constexpr int kCtlPerSlab = 64;
std::mutex g_ctl_mutex;
std::vector<Ctl*> g_ctl_free;

Ctl* ctl_mirror_get() {
    std::lock_guard<std::mutex> lock(g_ctl_mutex);
    if (g_ctl_free.empty()) {
        Ctl* slab = nullptr;
        if (cudaMallocHost(reinterpret_cast<void**>(&slab), sizeof(Ctl) * kCtlPerSlab) != cudaSuccess) return nullptr;
        for (int i = kCtlPerSlab - 1; i >= 0; --i) g_ctl_free.push_back(slab + i);
    }
    Ctl* c = g_ctl_free.back();
    g_ctl_free.pop_back();
    return c;
}
void ctl_mirror_put(Ctl* c) {
    if (!c) return;
    std::lock_guard<std::mutex> lock(g_ctl_mutex);
    g_ctl_free.push_back(c);
}

uint32_t even_words(uint64_t bits) { return uint32_t(((bits + 63) / 64) * 2); }

void free_particles(Scene& s) {
    const cudaStream_t st = s.stream;
    for (int f = 0; f < NPF; ++f) { dfree(s.part[f], st); dfree(s.part_alt[f], st); }
    dfree(s.keys, st); dfree(s.vals, st); dfree(s.keys_alt, st); dfree(s.vals_alt, st);
    dfree(s.bin_keys, st); dfree(s.bin_vals, st); dfree(s.bin_keys_alt, st); dfree(s.bin_vals_alt, st);
    dfree(s.sort_hist, st); dfree(s.sort_scan_tmp, st);
    s.part_cap = 0;
}

// Pipelined host I/O: buffers, events and the two copy streams.
void free_pipeline(Scene& s) {
    if (s.up_stream) cudaStreamSynchronize(s.up_stream);
    if (s.down_stream) cudaStreamSynchronize(s.down_stream);
    for (int i = 0; i < 4; ++i)
        for (int b = 0; b < 2; ++b) {
            dfree(s.stage_buf[i][b], s.stream);
            dfree(s.read_buf[i][b], s.stream);
            s.read_floats[i][b] = 0;
            for (cudaEvent_t* e : {&s.stage_ready[i][b], &s.stage_used[i][b], &s.read_packed[i][b], &s.read_done[i][b]})
                if (*e) { cudaEventDestroy(*e); *e = nullptr; }
        }
    for (int i = 0; i < 4; ++i) { s.stage_next[i] = 0; s.stage_pending[i] = -1; s.read_next[i] = 0; }
    if (s.up_stream) cudaStreamDestroy(s.up_stream);
    if (s.down_stream) cudaStreamDestroy(s.down_stream);
    s.up_stream = s.down_stream = nullptr;
}

cudaError_t ensure_pipeline(Scene& s) {
    if (s.up_stream) return cudaSuccess;
    cudaError_t e = cudaStreamCreateWithFlags(&s.up_stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&s.down_stream, cudaStreamNonBlocking);
    for (int i = 0; i < 4 && e == cudaSuccess; ++i)
        for (int b = 0; b < 2 && e == cudaSuccess; ++b)
            for (cudaEvent_t* ev : {&s.stage_ready[i][b], &s.stage_used[i][b], &s.read_packed[i][b], &s.read_done[i][b]})
                if (e == cudaSuccess) e = cudaEventCreateWithFlags(ev, cudaEventDisableTiming);
    return e;
}

// Force fields staged by apic_stage_field: each pending one is copied into
// its field on the scene's stream once its upload finished, before the
// update that follows reads it.
cudaError_t apply_staged(Scene& s) {
    for (int i = 0; i < 4; ++i) {
        const int b = s.stage_pending[i];
        if (b < 0) continue;
        float* dst = i == 0 ? s.ext_u : i == 1 ? s.ext_v : i == 2 ? s.post_u : s.post_v;
        const size_t n = (i % 2 == 0) ? s.uf : s.vf;
        cudaError_t e = cudaStreamWaitEvent(s.stream, s.stage_ready[i][b], 0);
        if (e == cudaSuccess) e = cudaMemcpyAsync(dst, s.stage_buf[i][b], n * sizeof(float), cudaMemcpyDeviceToDevice, s.stream);
        if (e == cudaSuccess) e = cudaEventRecord(s.stage_used[i][b], s.stream);
        if (e != cudaSuccess) return e;
        if (i < 2) s.has_ext = true;
        else s.has_post = true;
        s.stage_pending[i] = -1;
    }
    return cudaSuccess;
}

void free_scene(Scene& s) {
    const cudaStream_t st = s.stream;
    free_particles(s);
    dfree(s.pp, st);
    float** fl[] = {&s.u, &s.v, &s.u_alt, &s.v_alt, &s.acc_u, &s.acc_uw, &s.acc_v, &s.acc_vw, &s.ext_u,
                    &s.ext_v, &s.post_u, &s.post_v, &s.density, &s.sm_a, &s.sm_b, &s.pressure, &s.search,
                    &s.ap, &s.corr, &s.cg_s, &s.cg_ap, &s.cg_r};
    for (float** p : fl) dfree(*p, st);
    dfree(s.valid_u, st); dfree(s.valid_v, st); dfree(s.valid_u_alt, st); dfree(s.valid_v_alt, st);
    dfree(s.u_open, st); dfree(s.v_open, st); dfree(s.obstacle, st);
    dfree(s.bin_lo, st); dfree(s.bin_hi, st);
    dfree(s.p64, st); dfree(s.b64, st);
    for (int l = 0; l < s.nlevels; ++l) {
        Level& L = s.lv[l];
        dfree(L.fluid, st); dfree(L.seg, st); dfree(L.diag, st); dfree(L.inv_diag, st); dfree(L.px, st);
        dfree(L.py, st); dfree(L.res, st); dfree(L.err, st);
    }
    free_render(s);
    dfree(s.vec_stage, st);
    s.vec_stage = nullptr;
    s.vec_stage_floats = 0;
    free_pipeline(s);
    dfree(s.ctl, st);
    ctl_mirror_put(s.ctl_host);
    s.ctl_host = nullptr;
    dfree(s.partials, st); dfree(s.scan_tmp, st); dfree(s.exact_parts, st); dfree(s.seg_pre, st);
    if (s.ev_a) cudaEventDestroy(s.ev_a);
    if (s.ev_b) cudaEventDestroy(s.ev_b);
    if (s.update_exec) cudaGraphExecDestroy(s.update_exec);
    s.update_exec = nullptr;
    if (s.cap_stream) cudaStreamDestroy(s.cap_stream);
    s.cap_stream = nullptr;
    if (s.stream) cudaStreamDestroy(s.stream);
    s.stream = nullptr;
}

// Graphs bake in launch shapes and solver settings: rebuild after changes.
void invalidate_graphs(Scene& s) {
    if (s.update_exec) cudaGraphExecDestroy(s.update_exec);
    s.update_exec = nullptr;
    s.graph_version++;  // batched updates that recorded this scene's kernels rebuild too
}

// Open-face masks from the obstacle mask (update_world, src/apic.rs:918-944).
void open_masks(const Scene& s, const std::vector<uint32_t>& obst, std::vector<uint32_t>& uo,
                std::vector<uint32_t>& vo) {
    auto is_obst = [&](int i, int j) -> uint32_t {
        if (i < 0 || i >= int(s.W) || j < 0 || j >= int(s.H)) return 1;
        uint32_t idx = uint32_t(j) * s.W + uint32_t(i);
        return (obst[idx >> 5] >> (idx & 31)) & 1u;
    };
    uo.assign(s.u_open_words, 0);
    vo.assign(s.v_open_words, 0);
    for (uint64_t idx = 0; idx < s.uf; ++idx) {
        int i = int(idx % (s.W + 1)), j = int(idx / (s.W + 1));
        if ((is_obst(i - 1, j) | is_obst(i, j)) == 0) uo[idx >> 5] |= 1u << (idx & 31);
    }
    for (uint64_t idx = 0; idx < s.vf; ++idx) {
        int i = int(idx % s.W), j = int(idx / s.W);
        if ((is_obst(i, j - 1) | is_obst(i, j)) == 0) vo[idx >> 5] |= 1u << (idx & 31);
    }
}

int upload_world(apic_handle* h) {
    Scene& s = h->s;
    std::vector<uint32_t> uo, vo;
    open_masks(s, h->obstacle_host, uo, vo);
    // in order on the scene's stream (pageable sources are staged before each call returns)
    CK(cudaMemcpyAsync(s.obstacle, h->obstacle_host.data(), sizeof(uint32_t) * h->obstacle_host.size(),
                       cudaMemcpyHostToDevice, s.stream));
    CK(cudaMemcpyAsync(s.u_open, uo.data(), sizeof(uint32_t) * uo.size(), cudaMemcpyHostToDevice, s.stream));
    CK(cudaMemcpyAsync(s.v_open, vo.data(), sizeof(uint32_t) * vo.size(), cudaMemcpyHostToDevice, s.stream));
    s.world_ready = true;
    return APIC_OK;
}

int alloc_particles(Scene& s, uint32_t npad, uint32_t n) {
    if (npad <= s.part_cap && s.part_cap > 0) return APIC_OK;
    free_particles(s);
    const cudaStream_t st = s.stream;
    for (int f = 0; f < NPF; ++f) {
        CK(dalloc(&s.part[f], npad, st));
        CK(dalloc(&s.part_alt[f], npad, st));
    }
    CK(dalloc(&s.keys, npad, st)); CK(dalloc(&s.vals, npad, st));
    CK(dalloc(&s.keys_alt, npad, st)); CK(dalloc(&s.vals_alt, npad, st));
    CK(dalloc(&s.bin_keys, npad, st)); CK(dalloc(&s.bin_vals, npad, st));
    CK(dalloc(&s.bin_keys_alt, npad, st)); CK(dalloc(&s.bin_vals_alt, npad, st));
    CK(dalloc(&s.sort_hist, sort_hist_words(n), st));
    CK(dalloc(&s.sort_scan_tmp, sort_scan_words(n), st));
    s.part_cap = npad;
    return APIC_OK;
}

// Upload particles (positions, velocities) with the reference's padding.
int load_particles(apic_handle* h, uint32_t n, const float* px, const float* py, const float* vx, const float* vy) {
    Scene& s = h->s;
    uint32_t nchunks = (n + 7) / 8, npad = nchunks * 8;
    int rc = alloc_particles(s, npad, n);
    if (rc != APIC_OK) return rc;
    // sort scratch may need to grow when n grows within the same capacity
    {
        dfree(s.sort_hist, s.stream); dfree(s.sort_scan_tmp, s.stream);
        CK(dalloc(&s.sort_hist, sort_hist_words(n), s.stream));
        CK(dalloc(&s.sort_scan_tmp, sort_scan_words(n), s.stream));
    }
    // a new particle set: the next mixed solve starts from zero pressure
    if (s.p64) CK(cudaMemsetAsync(s.p64, 0, sizeof(double) * (uint64_t(s.cells) + 2ull * s.W), s.stream));
    std::vector<float> buf(std::max<uint32_t>(npad, 1), 0.0f);
    auto put = [&](int f, const float* src, bool pad_last) -> int {
        std::fill(buf.begin(), buf.end(), 0.0f);
        if (src) std::memcpy(buf.data(), src, sizeof(float) * n);
        if (pad_last && n > 0 && src)
            for (uint32_t l = n; l < npad; ++l) buf[l] = src[n - 1];
        // from pageable memory: staged before the call returns, so buf can be refilled
        CK(cudaMemcpyAsync(s.part[f], buf.data(), sizeof(float) * npad, cudaMemcpyHostToDevice, s.stream));
        CK(cudaMemsetAsync(s.part_alt[f], 0, sizeof(float) * npad, s.stream));
        return APIC_OK;
    };
    if (npad) {
        if ((rc = put(PX, px, true)) || (rc = put(PY, py, true))) return rc;
        if ((rc = put(VX, vx, false)) || (rc = put(VY, vy, false))) return rc;
        for (int f = CUX; f < NPF; ++f)
            if ((rc = put(f, nullptr, false))) return rc;
    }
    PartPtrs t;
    for (int f = 0; f < NPF; ++f) { t.f[f] = s.part[f]; t.alt[f] = s.part_alt[f]; }
    CK(cudaMemcpyAsync(s.pp, &t, sizeof(PartPtrs), cudaMemcpyHostToDevice, s.stream));
    s.n = n;
    s.nchunks = nchunks;
    s.npad = npad;
    CK(launch_vmax(s));
    s.vmax_valid = true;
    return APIC_OK;
}

PartPtrs read_ptrs(Scene& s) {
    PartPtrs t;
    cudaMemcpy(&t, s.pp, sizeof(PartPtrs), cudaMemcpyDeviceToHost);
    return t;
}

int sync_ctl(Scene& s) {
    CK(cudaMemcpyAsync(s.ctl_host, s.ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, s.stream));
    CK(cudaStreamSynchronize(s.stream));
    return APIC_OK;
}

// ---- stage timing --------------------------------------------------------
struct StageTimer {
    Scene& s;
    int stage;
    StageTimer(Scene& sc, int st) : s(sc), stage(st) {
        if (s.profiling) cudaEventRecord(s.ev_a, s.stream);
    }
    ~StageTimer() {
        if (!s.profiling) return;
        cudaEventRecord(s.ev_b, s.stream);
        cudaEventSynchronize(s.ev_b);
        float ms = 0;
        cudaEventElapsedTime(&ms, s.ev_a, s.ev_b);
        s.stage_ms[stage] += ms;
        s.stage_launches[stage] += 1;
    }
};

// P2G writes every accumulator entry; it needs empty cell runs and a clear
// fluid mask.
cudaError_t clear_p2g_targets(Scene& s) {
    cudaStream_t st = s.stream;
    cudaMemsetAsync(s.bin_lo, 0, sizeof(uint32_t) * s.cells, st);
    cudaMemsetAsync(s.bin_hi, 0, sizeof(uint32_t) * s.cells, st);
    cudaMemsetAsync(s.lv[0].fluid, 0, sizeof(uint32_t) * s.lv[0].words, st);
    return cudaGetLastError();
}

// Stages before the pressure solve (src/apic.rs:2446-2449).
cudaError_t enqueue_pre_solve(Scene& s) {
    cudaError_t e;
    if ((e = clear_p2g_targets(s)) != cudaSuccess) return e;
    if ((e = launch_p2g(s)) != cudaSuccess) return e;
    if ((e = launch_finalize_faces(s, true, true)) != cudaSuccess) return e;
    if ((e = launch_base_lists(s)) != cudaSuccess) return e;
    if ((e = launch_build_pressure(s)) != cudaSuccess) return e;
    return launch_multilevel(s);
}
// Stages after it (src/apic.rs:2451-2461), without the end-of-substep bookkeeping.
cudaError_t enqueue_post_solve(Scene& s) {
    cudaError_t e;
    if ((e = launch_gradient(s, true)) != cudaSuccess) return e;
    if ((e = launch_extrapolate(s)) != cudaSuccess) return e;
    return launch_g2p(s);
}

// Apic::update as one graph: plan -> IF(sort) -> WHILE(substep due) { stages; advance }.
int ensure_update_graph(Scene& s) {
    if (s.update_exec) return APIC_OK;
    GraphCursor top;
    CK(cudaGraphCreate(&top.g, 0));
    cudaGraphConditionalHandle h_sort, h_loop;
    cudaError_t e = cudaGraphConditionalHandleCreate(&h_sort, top.g, 0, cudaGraphCondAssignDefault);
    if (e == cudaSuccess) e = cudaGraphConditionalHandleCreate(&h_loop, top.g, 0, cudaGraphCondAssignDefault);
    if (e == cudaSuccess)
        e = capture_into(s, top, [&]() {
            k_plan_first_g<<<1, 1, 0, s.stream>>>(s.ctl, h_sort, h_loop);
            return cudaGetLastError();
        });
    GraphCursor sort_body, loop_body;
    if (e == cudaSuccess) e = add_conditional_with(top, cudaGraphCondTypeIf, h_sort, &sort_body);
    if (e == cudaSuccess) e = capture_into(s, sort_body, [&]() { return launch_sort(s); });
    if (e == cudaSuccess) e = add_conditional_with(top, cudaGraphCondTypeWhile, h_loop, &loop_body);
    if (e == cudaSuccess) e = capture_into(s, loop_body, [&]() { return enqueue_pre_solve(s); });
    if (e == cudaSuccess) e = build_solve(s, loop_body);
    if (e == cudaSuccess)
        e = capture_into(s, loop_body, [&]() {
            cudaError_t r = enqueue_post_solve(s);
            if (r != cudaSuccess) return r;
            k_advance_g<<<1, 1, 0, s.stream>>>(s.ctl, h_loop);
            return cudaGetLastError();
        });
    if (e == cudaSuccess) {
        s.kn_top = count_kernel_nodes(top.g);
        s.kn_sort = count_kernel_nodes(sort_body.g);
        s.kn_loop = count_kernel_nodes(loop_body.g);
        e = cudaGraphInstantiate(&s.update_exec, top.g, 0);
    }
    cudaGraphDestroy(top.g);
    if (e != cudaSuccess) return fail(APIC_ERR_CUDA, std::string("update graph: ") + cudaGetErrorString(e));
    return APIC_OK;
}

// One substep launched stage by stage, each bracketed by events when
// profiling (the graph form cannot hold event nodes inside its loops).
int run_substep_eager(Scene& s, bool sort_now) {
    if (sort_now) { StageTimer t(s, APIC_STAGE_SORT); CK(launch_sort(s)); }
    { StageTimer t(s, APIC_STAGE_P2G); CK(clear_p2g_targets(s)); CK(launch_p2g(s)); }
    { StageTimer t(s, APIC_STAGE_FORCES); CK(launch_finalize_faces(s, true, true)); CK(launch_base_lists(s)); }
    { StageTimer t(s, APIC_STAGE_BUILD); CK(launch_build_pressure(s)); }
    { StageTimer t(s, APIC_STAGE_MG); CK(launch_multilevel(s)); }
    { StageTimer t(s, APIC_STAGE_PCG); CK(run_solve_eager(s)); }
    { StageTimer t(s, APIC_STAGE_GRAD); CK(launch_gradient(s, true)); }
    { StageTimer t(s, APIC_STAGE_EXTRAP); CK(launch_extrapolate(s)); }
    { StageTimer t(s, APIC_STAGE_G2P); CK(launch_g2p(s)); }
    k_advance<<<1, 1, 0, s.stream>>>(s.ctl);
    CK(cudaGetLastError());
    return APIC_OK;
}

float bits_to_float(uint32_t b) {
    float f;
    std::memcpy(&f, &b, 4);
    return f;
}

int valid_handle(apic_handle* h) {
    if (!h) return fail(APIC_ERR_INVALID_ARG, "null handle");
    return APIC_OK;
}

}  // namespace

// The stages either side of the pressure solve, for batched updates (batch.cu).
cudaError_t apic::scene_pre_solve(Scene& s) { return enqueue_pre_solve(s); }
cudaError_t apic::scene_post_solve(Scene& s) { return enqueue_post_solve(s); }
Scene& apic::scene_of(apic_handle* h) { return h->s; }

// ---- scene generators live in scene.cpp ----------------------------------

void apic::set_last_error(const char* msg) { g_last_error = msg ? msg : ""; }

// The driver's cuCtxGetCurrent / cuCtxGetId, found through the runtime so the
// library needs no link-time dependency on libcuda.
namespace {
typedef int (*CtxGetCurrentFn)(void**);
typedef int (*CtxGetIdFn)(void*, unsigned long long*);
std::once_flag g_ctx_fns_once;
CtxGetCurrentFn g_ctx_get_current = nullptr;
CtxGetIdFn g_ctx_get_id = nullptr;

cudaError_t context_id_now(unsigned long long* id) {
    void* ctx = nullptr;
    if (g_ctx_get_current(&ctx) != 0) return cudaErrorUnknown;
    if (!ctx) {
        *id = 0;
        return cudaSuccess;
    }
    return g_ctx_get_id(ctx, id) == 0 ? cudaSuccess : cudaErrorUnknown;
}
}  // namespace

cudaError_t apic::current_context_key(unsigned long long* key) {
    std::call_once(g_ctx_fns_once, [] {
        cudaDriverEntryPointQueryResult q;
        void* f = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            g_ctx_get_current = reinterpret_cast<CtxGetCurrentFn>(f);
        f = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            g_ctx_get_id = reinterpret_cast<CtxGetIdFn>(f);
    });
    if (!g_ctx_get_current || !g_ctx_get_id) return cudaErrorNotSupported;
    cudaError_t e = context_id_now(key);
    if (e != cudaSuccess || *key != 0) return e;
    // no context is current on this thread yet: let the runtime make its
    // primary context current, as its first call on this thread would
    if ((e = cudaFree(nullptr)) != cudaSuccess) return e;
    if ((e = context_id_now(key)) != cudaSuccess) return e;
    return *key != 0 ? cudaSuccess : cudaErrorDeviceUninitialized;
}

extern "C" {

const char* apic_last_error(void) { return g_last_error.c_str(); }

int apic_device_count(int* n_out) {
    if (!n_out) return fail(APIC_ERR_INVALID_ARG, "null output");
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess) n = 0;
    *n_out = n;
    return APIC_OK;
}

int apic_create(uint32_t width, uint32_t height, float cell_size, const apic_world_props* props, apic_handle** out) {
    return apic::create_scene(width, height, cell_size, props, true, out);
}

}  // extern "C"

// Apic::new; default_particles false leaves the scene empty (callers that
// set their own particles next, such as the request server, then never hold
// the default block's memory).
int apic::create_scene(uint32_t width, uint32_t height, float cell_size, const apic_world_props* props,
                       bool default_particles, apic_handle** out) {
    if (!out || !props) return fail(APIC_ERR_INVALID_ARG, "null argument");
    *out = nullptr;
    if (width == 0 || height == 0 || !(cell_size > 0.0f) || !std::isfinite(cell_size))
        return fail(APIC_ERR_INVALID_ARG, "width, height and cell_size must be positive");
    if (uint64_t(width) * height > (1ull << 31)) return fail(APIC_ERR_INVALID_ARG, "grid too large");
    // Morton keys interleave 16 bits per axis (src/apic.rs:185-203)
    if (width > 65536u || height > 65536u) return fail(APIC_ERR_INVALID_ARG, "width and height are limited to 65536");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return fail(APIC_ERR_NO_DEVICE, "no CUDA device");

    // the reference's default particles (src/apic.rs:831-849)
    std::vector<float> ix, iy;
    for (uint32_t y = 0; y < height; ++y)
        for (uint32_t x = 0; x < width; ++x) {
            bool border = x == 0 || x == width - 1 || y == 0 || y == height - 1;
            if (default_particles && !border && x > 4 && x < width - 4 && y > 4 && y < height / 2)
                for (int py = 0; py < 3; ++py)
                    for (int px = 0; px < 3; ++px) {
                        ix.push_back((float(x) + (float(px) + 0.5f) / 3.0f) * cell_size);
                        iy.push_back((float(y) + (float(py) + 0.5f) / 3.0f) * cell_size);
                    }
        }

    apic_handle* h = new (std::nothrow) apic_handle();
    if (!h) return fail(APIC_ERR_OOM, "host allocation failed");
    Scene& s = h->s;
    if (cudaGetDevice(&s.device) != cudaSuccess) s.device = 0;
    s.W = width; s.H = height; s.cells = width * height; s.dx = cell_size; s.props = *props;
    s.uf = (width + 1) * height;
    s.vf = width * (height + 1);
    s.u_open_words = even_words(s.uf);
    s.v_open_words = even_words(s.vf);

    // levels: base + halvings (src/apic.rs:900-908)
    s.lv[0].w = width; s.lv[0].h = height;
    s.nlevels = 1;
    {
        uint32_t cw = width, ch = height;
        while (cw % 2 == 0 && ch % 2 == 0 && cw > 4 && ch > 4 && s.nlevels < kMaxLevels) {
            cw /= 2; ch /= 2;
            s.lv[s.nlevels].w = cw; s.lv[s.nlevels].h = ch;
            s.nlevels++;
        }
    }
    if (!ix.empty() && s.nlevels < 2) {
        delete h;
        return fail(APIC_ERR_INVALID_ARG, "grid sides must be even and > 4 (no multigrid level; the reference panics)");
    }

    auto bail = [&](int rc) { free_scene(s); delete h; return rc; };
    cudaError_t e;
#define AL(ptr, count) if ((e = dalloc(&(ptr), (count), s.stream)) != cudaSuccess) return bail(fail(APIC_ERR_OOM, std::string("cudaMalloc: ") + cudaGetErrorString(e)))
    if ((e = cudaStreamCreateWithFlags(&s.stream, cudaStreamNonBlocking)) != cudaSuccess)
        return bail(fail(APIC_ERR_CUDA, cudaGetErrorString(e)));
    if ((e = cudaStreamCreateWithFlags(&s.cap_stream, cudaStreamNonBlocking)) != cudaSuccess)
        return bail(fail(APIC_ERR_CUDA, cudaGetErrorString(e)));
    cudaEventCreate(&s.ev_a);
    cudaEventCreate(&s.ev_b);
    AL(s.pp, 1);
    AL(s.u, s.uf); AL(s.u_alt, s.uf); AL(s.acc_u, s.uf); AL(s.acc_uw, s.uf); AL(s.ext_u, s.uf); AL(s.post_u, s.uf);
    AL(s.v, s.vf); AL(s.v_alt, s.vf); AL(s.acc_v, s.vf); AL(s.acc_vw, s.vf); AL(s.ext_v, s.vf); AL(s.post_v, s.vf);
    AL(s.valid_u, s.uf); AL(s.valid_u_alt, s.uf); AL(s.valid_v, s.vf); AL(s.valid_v_alt, s.vf);
    AL(s.u_open, s.u_open_words); AL(s.v_open, s.v_open_words);
    AL(s.density, s.cells); AL(s.sm_a, s.cells); AL(s.sm_b, s.cells); AL(s.pressure, s.cells);
    AL(s.bin_lo, s.cells); AL(s.bin_hi, s.cells);
    AL(s.obstacle, even_words(s.cells));
    size_t padded0 = (size_t(s.cells) + 2 * size_t(width) + 7) / 8 * 8;
    AL(s.search, padded0); AL(s.ap, padded0); AL(s.corr, padded0);
    AL(s.p64, padded0); AL(s.b64, padded0);
    uint32_t max_words = 0;
    for (int l = 0; l < s.nlevels; ++l) {
        Level& L = s.lv[l];
        L.cells = L.w * L.h;
        L.wshift = -1;
        for (int k = 0; k < 31; ++k)
            if ((1u << k) == L.w) L.wshift = k;
        L.words = even_words(L.cells);
        L.padded = uint32_t((size_t(L.cells) + 2 * size_t(L.w) + 7) / 8 * 8);
        max_words = std::max(max_words, L.words);
        AL(L.fluid, L.words); AL(L.seg, L.words);
        AL(L.diag, L.padded); AL(L.inv_diag, L.padded); AL(L.px, L.padded); AL(L.py, L.padded);
        AL(L.res, L.padded); AL(L.err, L.padded);
    }
    {
        Level& C = s.lv[s.nlevels - 1];
        AL(s.cg_s, C.padded); AL(s.cg_ap, C.padded); AL(s.cg_r, C.padded);
    }
    plan_vcycle(s);
    AL(s.ctl, 1);
    AL(s.partials, kPartialDoubles);
    AL(s.exact_parts, s.cells / 8192 + 1);
    AL(s.seg_pre, s.lv[0].words + 1);
    s.scan_tmp_len = 3 * (div_up(max_words, 1024) + 1);
    AL(s.scan_tmp, s.scan_tmp_len);
#undef AL
    // the buffers are ordered on the scene's stream; the copies below run on
    // the legacy stream
    if ((e = cudaStreamSynchronize(s.stream)) != cudaSuccess) return bail(fail(APIC_ERR_CUDA, cudaGetErrorString(e)));
    if (!(s.ctl_host = ctl_mirror_get())) return bail(fail(APIC_ERR_OOM, "pinned alloc"));
    std::memset(s.ctl_host, 0, sizeof(Ctl));
    s.ctl_host->prev_dt = 1.0f / 60.0f;  // src/apic.rs:824
    s.ctl_host->cfl_cs = props->cfl * cell_size;
    if ((e = cudaMemcpy(s.ctl, s.ctl_host, sizeof(Ctl), cudaMemcpyHostToDevice)) != cudaSuccess)
        return bail(fail(APIC_ERR_CUDA, cudaGetErrorString(e)));

    // solid one-cell border (src/apic.rs:834-836)
    h->obstacle_host.assign(even_words(s.cells), 0);
    for (uint32_t y = 0; y < height; ++y)
        for (uint32_t x = 0; x < width; ++x)
            if (x == 0 || x == width - 1 || y == 0 || y == height - 1) {
                uint32_t i = y * width + x;
                h->obstacle_host[i >> 5] |= 1u << (i & 31);
            }
    int rc = upload_world(h);
    if (rc != APIC_OK) return bail(rc);
    rc = load_particles(h, uint32_t(ix.size()), ix.data(), iy.data(), nullptr, nullptr);
    if (rc != APIC_OK) return bail(rc);
    if ((e = cudaStreamSynchronize(s.stream)) != cudaSuccess) return bail(fail(APIC_ERR_CUDA, cudaGetErrorString(e)));
    *out = h;
    return APIC_OK;
}

extern "C" {

int apic_destroy(apic_handle* h) {
    if (!h) return APIC_OK;
    if (h->s.stream) cudaStreamSynchronize(h->s.stream);
    batch_release_scene(&h->s);
    free_scene(h->s);
    delete h;
    return APIC_OK;
}

int apic_set_particles(apic_handle* h, uint32_t n, const float* px, const float* py, const float* vx,
                       const float* vy) {
    if (valid_handle(h)) return APIC_ERR_INVALID_ARG;
    if (n > 0 && (!px || !py)) return fail(APIC_ERR_INVALID_ARG, "positions required");
    if (n > 0 && h->s.nlevels < 2)
        return fail(APIC_ERR_INVALID_ARG, "grid sides must be even and > 4 (no multigrid level)");
    if (uint64_t(n) + 8 > (1ull << 31)) return fail(APIC_ERR_INVALID_ARG, "too many particles");
    CK(cudaStreamSynchronize(h->s.stream));
    invalidate_graphs(h->s);
    int rc = load_particles(h, n, px, py, vx, vy);
    if (rc == APIC_OK) CK(cudaStreamSynchronize(h->s.stream));
    return rc;
}

int apic_set_solver(apic_handle* h, int mode, float rel_tol, uint32_t max_iterations) {
    if (valid_handle(h)) return APIC_ERR_INVALID_ARG;
    if (mode < APIC_SOLVER_REFERENCE || mode > APIC_SOLVER_REL_MIXED || !(rel_tol > 0.0f) || max_iterations == 0)
        return fail(APIC_ERR_INVALID_ARG, "bad solver configuration");
    if (h->s.stream) cudaStreamSynchronize(h->s.stream);
    h->s.solver_mode = mode;
    h->s.rel_tol = rel_tol;
    h->s.max_iter = max_iterations;
    invalidate_graphs(h->s);
    return APIC_OK;
}

}  // extern "C"

namespace apic {

// What an update enqueues on the scene's stream before its substep loop:
// staged uploads, the control block's reset for the new update, and the max
// speed when no G2P has reduced it yet.
int update_begin(apic_handle* h, uint32_t flags, float frame_dt) {
    if (valid_handle(h)) return APIC_ERR_INVALID_ARG;
    Scene& s = h->s;
    if (!std::isfinite(frame_dt)) return fail(APIC_ERR_INVALID_ARG, "frame_deltatime must be finite");
    cudaStream_t st = s.stream;
    s.stats = apic_step_stats{};
    s.batched = false;
    CK(apply_staged(s));
    k_begin_update<<<1, 1, 0, st>>>(s.ctl, frame_dt, flags, s.has_ext ? 1u : 0u, s.has_post ? 1u : 0u);
    if (!s.vmax_valid) { CK(launch_vmax(s)); s.vmax_valid = true; }
    return APIC_OK;
}

// ... and after it: the force fields of this update are used up, and the
// control block is copied back for update_finish.
int update_end(apic_handle* h) {
    Scene& s = h->s;
    cudaStream_t st = s.stream;
    if (s.has_ext) { CK(cudaMemsetAsync(s.ext_u, 0, sizeof(float) * s.uf, st)); CK(cudaMemsetAsync(s.ext_v, 0, sizeof(float) * s.vf, st)); }
    if (s.has_post) { CK(cudaMemsetAsync(s.post_u, 0, sizeof(float) * s.uf, st)); CK(cudaMemsetAsync(s.post_v, 0, sizeof(float) * s.vf, st)); }
    s.has_ext = s.has_post = false;
    CK(cudaMemcpyAsync(s.ctl_host, s.ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, st));
    return APIC_OK;
}

// First half of Apic::update: everything up to the copy of the control block
// back to the host is enqueued on the scene's stream; nothing waits (except
// in profiling mode, whose host-driven loop reads the device state).
int update_launch(apic_handle* h, uint32_t flags, float frame_dt) {
    int rc0 = update_begin(h, flags, frame_dt);
    if (rc0 != APIC_OK) return rc0;
    Scene& s = h->s;
    cudaStream_t st = s.stream;
    if (s.profiling) {
        // stage-by-stage with host control of the substep loop
        k_plan_first<<<1, 1, 0, st>>>(s.ctl);
        CK(cudaGetLastError());
        bool first = true;
        for (;;) {
            int rc = sync_ctl(s);
            if (rc != APIC_OK) return rc;
            if (!s.ctl_host->go) break;
            rc = run_substep_eager(s, first && !(flags & APIC_UPDATE_DISABLE_SORT));
            if (rc != APIC_OK) return rc;
            first = false;
        }
    } else {
        int rc = ensure_update_graph(s);
        if (rc != APIC_OK) return rc;
        CK(cudaGraphLaunch(s.update_exec, st));
    }
    return update_end(h);
}

// Second half: wait for the scene's stream and publish the step statistics.
int update_finish(apic_handle* h) {
    Scene& s = h->s;
    CK(cudaStreamSynchronize(s.stream));
    const Ctl& c = *s.ctl_host;
    s.stats.substeps = c.substeps;
    s.stats.pcg_iterations = c.pcg_iters;
    s.stats.pcg_iterations_total = c.pcg_iters_total;
    s.stats.refinement_steps = c.refinements;
    s.stats.residual_max = bits_to_float(c.max_r_bits);
    s.stats.residual_rel = c.bnorm2 > 0 ? float(std::sqrt(c.rnorm2 / c.bnorm2)) : 0.0f;
    s.stats.true_residual_rel = c.true_rel;
    s.stats.not_converged = c.not_converged;
    s.stats.nonfinite_lanes = c.nonfinite;
    s.stats.solve_ms = double(c.solve_ns) * 1e-6;
    if (s.batched)  // the scene's own kernels; the batch's solve kernels are counted by the batch
        s.stats.kernel_launches = (c.sorted ? s.kn_bsort : 0u) + uint64_t(c.substeps) * s.kn_bstep;
    else if (!s.profiling)
        s.stats.kernel_launches = uint64_t(s.kn_top) + (c.sorted ? s.kn_sort : 0u) + uint64_t(c.substeps) * s.kn_loop +
                                  uint64_t(c.pcg_iters_total) * s.kn_pcg + uint64_t(c.refinements_total) * s.kn_refine;
    if (c.status & kStatusBounds)
        return fail(APIC_ERR_CUDA, "bounds check: an index left its buffer (build with APIC_BOUNDS_CHECK)");
    if (c.status & kStatusP2gLayout)
        return fail(APIC_ERR_CUDA, "P2G: a particle's stencil left the cells its faces gather from (internal error)");
    if (c.status & kStatusBadStep) return fail(APIC_ERR_NONFINITE, "substep size is not positive (non-finite velocities)");
    return APIC_OK;
}

// Build the update graph before the first update, so that update can launch
// at once (the request server does this on its preparation threads).
int update_prepare(apic_handle* h) {
    if (valid_handle(h)) return APIC_ERR_INVALID_ARG;
    if (h->s.profiling) return APIC_OK;
    return ensure_update_graph(h->s);
}

// The stream of a scene (the request server polls it for completion).
cudaStream_t scene_stream(apic_handle* h) { return h ? h->s.stream : nullptr; }

}  // namespace apic

extern "C" {

int apic_update(apic_handle* h, uint32_t flags, float frame_dt) {
    int rc = update_launch(h, flags, frame_dt);
    if (rc != APIC_OK) return rc;
    return update_finish(h);
}

int apic_update_batch(apic_handle* const* handles, uint32_t count, uint32_t flags, float frame_dt, int* status) {
    if (count && !handles) return fail(APIC_ERR_INVALID_ARG, "null handle array");
    for (uint32_t i = 0; i < count; ++i)
        if (valid_handle(handles[i])) return fail(APIC_ERR_INVALID_ARG, "invalid handle in batch");
    for (uint32_t i = 0; i < count; ++i)
        for (uint32_t j = 0; j < i; ++j)
            if (handles[i] == handles[j]) return fail(APIC_ERR_INVALID_ARG, "a scene appears twice in the batch");
    std::vector<int> rc(count, APIC_OK);
    const uint32_t uflags = flags & ~uint32_t(APIC_UPDATE_BATCH_STREAMS | APIC_UPDATE_BATCH_JOINT);
    // the tuner picks the form (and the joint form's shape) unless told
    const bool tuned = !(flags & APIC_UPDATE_BATCH_STREAMS) && batch_eligible(handles, count);
    const auto t0 = std::chrono::steady_clock::now();
    BatchTicket tk;
    if (tuned) batch_choose(handles, count, (flags & APIC_UPDATE_BATCH_JOINT) != 0, &tk);
    if (tuned && tk.joint) {
        // one graph: every scene's own stages, the pressure solves of all
        // scenes as one launch per phase (batch.cu)
        update_batch_joint(handles, count, uflags, frame_dt, tk.shape, rc.data());
    } else {
        batch_note_streams(count);
        // every scene's update is enqueued on its own stream before any is
        // waited on, so the GPU runs the scenes' kernels side by side
        for (uint32_t i = 0; i < count; ++i) rc[i] = update_launch(handles[i], uflags, frame_dt);
    }
    int first = APIC_OK;
    std::string first_msg;
    uint64_t iterations = 0;
    for (uint32_t i = 0; i < count; ++i) {
        if (rc[i] == APIC_OK) rc[i] = update_finish(handles[i]);
        if (status) status[i] = rc[i];
        if (rc[i] != APIC_OK && first == APIC_OK) {
            first = rc[i];
            first_msg = apic_last_error();
        }
        iterations += handles[i]->s.stats.pcg_iterations_total;
    }
    if (tuned && first == APIC_OK)
        batch_record(tk, std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count(),
                     iterations);
    if (first != APIC_OK) return fail(first, "apic_update_batch: " + first_msg);
    return APIC_OK;
}

int apic_add_radial_force(apic_handle* h, float wx, float wy, float radius, float strength) {
    if (valid_handle(h)) return APIC_ERR_INVALID_ARG;
    Scene& s = h->s;
    uint32_t* box = nullptr;
    CK(cudaMallocHost(&box, 4 * sizeof(uint32_t)));
    uint32_t* dbox = reinterpret_cast<uint32_t*>(s.partials);  // scratch, idle between calls
    k_force_box<<<1, 1, 0, s.stream>>>(wx, wy, radius, s.dx, int(s.W), int(s.H), dbox);
    cudaMemcpyAsync(box, dbox, 4 * sizeof(uint32_t), cudaMemcpyDeviceToHost, s.stream);
    cudaError_t e = cudaStreamSynchronize(s.stream);
    if (e != cudaSuccess) { cudaFreeHost(box); return fail(APIC_ERR_CUDA, cudaGetErrorString(e)); }
    uint32_t x0 = box[0], x1 = box[1], y0 = box[2], y1 = box[3];
    cudaFreeHost(box);
    if (x1 >= x0 && y1 >= y0) {
        uint32_t nx = x1 - x0 + 1, ny = y1 - y0 + 1;
        k_radial_force<<<div_up(uint64_t(nx) * ny, 256), 256, 0, s.stream>>>(
            int(s.W), int(s.H), s.dx, wx, wy, radius, strength, x0, y0, nx, ny, s.ext_u, s.ext_v, s.post_u, s.post_v);
        CK(cudaGetLastError());
        if (strength > 0.0f) s.has_post = true;
        else s.has_ext = true;
    }
    return APIC_OK;
}

int apic_max_particle_velocity(apic_handle* h, float* out) {
    if (valid_handle(h) || !out) return fail(APIC_ERR_INVALID_ARG, "null argument");
    Scene& s = h->s;
    CK(launch_vmax(s));
    int rc = sync_ctl(s);
    if (rc) return rc;
    *out = bits_to_float(s.ctl_host->vmax_bits);
    s.vmax_valid = true;
    return APIC_OK;
}

int apic_is_fluid(apic_handle* h, int32_t i, int32_t j, uint64_t* out) {
    if (valid_handle(h) || !out) return fail(APIC_ERR_INVALID_ARG, "null argument");
    Scene& s = h->s;
    *out = 0;
    if (i < 0 || i >= int32_t(s.W) || j < 0 || j >= int32_t(s.H)) return APIC_OK;
    uint32_t idx = uint32_t(j) * s.W + uint32_t(i), word = 0;
    CK(cudaStreamSynchronize(s.stream));
    CK(cudaMemcpy(&word, s.lv[0].fluid + (idx >> 5), sizeof(uint32_t), cudaMemcpyDeviceToHost));
    *out = (word >> (idx & 31)) & 1u;
    return APIC_OK;
}

int apic_update_world(apic_handle* h) {
    if (valid_handle(h)) return APIC_ERR_INVALID_ARG;
    CK(cudaStreamSynchronize(h->s.stream));
    return upload_world(h);
}

int apic_get_info(apic_handle* h, apic_info* out) {
    if (valid_handle(h) || !out) return fail(APIC_ERR_INVALID_ARG, "null argument");
    Scene& s = h->s;
    int rc = sync_ctl(s);
    if (rc) return rc;
    out->width = s.W; out->height = s.H; out->cells = s.cells; out->cell_size = s.dx;
    out->num_chunks = s.nchunks; out->num_particles = s.n;
    out->fluid_cells = s.ctl_host->fluid_cells;
    out->timestamp = s.ctl_host->timestamp;
    out->prev_deltatime = s.ctl_host->prev_dt;
    out->mg_levels = uint32_t(s.nlevels > 0 ? s.nlevels - 1 : 0);
    return APIC_OK;
}

int apic_get_stats(apic_handle* h, apic_step_stats* out) {
    if (valid_handle(h) || !out) return fail(APIC_ERR_INVALID_ARG, "null argument");
    *out = h->s.stats;
    return APIC_OK;
}

}  // extern "C"

// ---- field access ---------------------------------------------------------
namespace {

enum Kind { kF32, kU8, kU32, kMask };
struct FieldDesc {
    void* dev = nullptr;
    uint64_t count = 0;   // elements as exposed
    uint32_t elem = 0;
    Kind kind = kF32;
    bool ok = false;
};

FieldDesc describe(apic_handle* h, int id, const PartPtrs* pp) {
    Scene& s = h->s;
    FieldDesc d;
    uint64_t padded = uint64_t(s.cells) + 2ull * s.W;
    auto F = [&](void* p, uint64_t n) { d.dev = p; d.count = n; d.elem = 4; d.kind = kF32; d.ok = true; };
    auto M = [&](void* p, uint64_t u32words) { d.dev = p; d.count = u32words / 2; d.elem = 8; d.kind = kMask; d.ok = true; };
    if (id >= APIC_F_POS_X && id <= APIC_F_TRES) { F(pp ? pp->f[id] : nullptr, s.npad); return d; }
    switch (id) {
        case APIC_F_U: F(s.u, s.uf); return d;
        case APIC_F_V: F(s.v, s.vf); return d;
        case APIC_F_VALID_U: d = {s.valid_u, s.uf, 1, kU8, true}; return d;
        case APIC_F_VALID_V: d = {s.valid_v, s.vf, 1, kU8, true}; return d;
        case APIC_F_DENSITY: F(s.density, s.cells); return d;
        case APIC_F_SMOOTHED_DENSITY: F(s.sm_a, s.cells); return d;
        case APIC_F_PRESSURE: F(s.pressure, s.cells); return d;
        case APIC_F_FLUID_BITS: M(s.lv[0].fluid, s.lv[0].words); return d;
        case APIC_F_OBSTACLE_BITS: M(s.obstacle, even_words(s.cells)); return d;
        case APIC_F_U_OPEN_BITS: M(s.u_open, s.u_open_words); return d;
        case APIC_F_V_OPEN_BITS: M(s.v_open, s.v_open_words); return d;
        case APIC_F_RESIDUAL: F(s.lv[0].res, padded); return d;
        case APIC_F_DIAG: F(s.lv[0].diag, padded); return d;
        case APIC_F_INV_DIAG: F(s.lv[0].inv_diag, padded); return d;
        case APIC_F_PLUS_X: F(s.lv[0].px, padded); return d;
        case APIC_F_PLUS_Y: F(s.lv[0].py, padded); return d;
        case APIC_F_ERROR: F(s.lv[0].err, padded); return d;
        case APIC_F_SORT_KEYS: d = {sort_result_in_alt(s) ? s.keys_alt : s.keys, s.n, 4, kU32, true}; return d;
        case APIC_F_SORT_VALS: d = {sort_result_in_alt(s) ? s.vals_alt : s.vals, s.n, 4, kU32, true}; return d;
        case APIC_F_FLUID_LIST: d = {nullptr, 0, 4, kU32, true}; return d;  // derived on read
        case APIC_F_EXT_FORCE_U: F(s.ext_u, s.uf); return d;
        case APIC_F_EXT_FORCE_V: F(s.ext_v, s.vf); return d;
        case APIC_F_POST_FORCE_U: F(s.post_u, s.uf); return d;
        case APIC_F_POST_FORCE_V: F(s.post_v, s.vf); return d;
        default: break;
    }
    if (id >= APIC_F_MG_FLUID_BITS) {
        int l = id / APIC_F_MG_LEVEL_STRIDE + 1;
        int f = id % APIC_F_MG_LEVEL_STRIDE;
        if (l < 1 || l >= s.nlevels) return d;
        Level& L = s.lv[l];
        uint64_t lp = uint64_t(L.cells) + 2ull * L.w;
        switch (f) {
            case APIC_F_MG_FLUID_BITS: M(L.fluid, L.words); return d;
            case APIC_F_MG_DIAG: F(L.diag, lp); return d;
            case APIC_F_MG_INV_DIAG: F(L.inv_diag, lp); return d;
            case APIC_F_MG_PLUS_X: F(L.px, lp); return d;
            case APIC_F_MG_PLUS_Y: F(L.py, lp); return d;
            default: break;
        }
    }
    return d;
}

std::vector<uint32_t> fluid_list(apic_handle* h) {
    Scene& s = h->s;
    std::vector<uint32_t> words(s.lv[0].words), out;
    cudaMemcpy(words.data(), s.lv[0].fluid, sizeof(uint32_t) * words.size(), cudaMemcpyDeviceToHost);
    for (uint32_t w = 0; w < words.size(); ++w) {
        uint32_t m = words[w];
        while (m) {
            uint32_t raw = w * 32 + uint32_t(__builtin_ctz(m));
            if (raw < s.cells) out.push_back(raw + s.W);
            m &= m - 1;
        }
    }
    return out;
}

}  // namespace

extern "C" {

int apic_field_shape(apic_handle* h, int field, uint64_t* count, uint32_t* elem_bytes) {
    if (valid_handle(h) || !count || !elem_bytes) return fail(APIC_ERR_INVALID_ARG, "null argument");
    CK(cudaStreamSynchronize(h->s.stream));
    FieldDesc d = describe(h, field, nullptr);
    if (!d.ok) return fail(APIC_ERR_INVALID_ARG, "unknown field " + std::to_string(field));
    if (field == APIC_F_FLUID_LIST) d.count = fluid_list(h).size();
    *count = d.count;
    *elem_bytes = d.elem;
    return APIC_OK;
}

int apic_read_field(apic_handle* h, int field, void* dst, uint64_t bytes) {
    if (valid_handle(h)) return APIC_ERR_INVALID_ARG;
    Scene& s = h->s;
    CK(cudaStreamSynchronize(s.stream));
    PartPtrs pp = read_ptrs(s);
    FieldDesc d = describe(h, field, &pp);
    if (!d.ok) return fail(APIC_ERR_INVALID_ARG, "unknown field " + std::to_string(field));
    if (field == APIC_F_FLUID_LIST) {
        std::vector<uint32_t> l = fluid_list(h);
        if (bytes != l.size() * 4) return fail(APIC_ERR_INVALID_ARG, "size mismatch");
        if (bytes) std::memcpy(dst, l.data(), bytes);
        return APIC_OK;
    }
    if (bytes != d.count * d.elem) return fail(APIC_ERR_INVALID_ARG, "size mismatch");
    if (bytes == 0) return APIC_OK;
    if (!dst) return fail(APIC_ERR_INVALID_ARG, "null destination");
    if (field == APIC_F_SMOOTHED_DENSITY) {
        float* tmp = s.sm_b;  // free between substeps
        CK(launch_smoothed_view(s, tmp));
        CK(cudaMemcpyAsync(dst, tmp, bytes, cudaMemcpyDeviceToHost, s.stream));
        CK(cudaStreamSynchronize(s.stream));
        return APIC_OK;
    }
    CK(cudaMemcpy(dst, d.dev, bytes, cudaMemcpyDeviceToHost));
    return APIC_OK;
}

int apic_write_field(apic_handle* h, int field, const void* src, uint64_t bytes) {
    if (valid_handle(h)) return APIC_ERR_INVALID_ARG;
    Scene& s = h->s;
    CK(cudaStreamSynchronize(s.stream));
    PartPtrs pp = read_ptrs(s);
    FieldDesc d = describe(h, field, &pp);
    if (!d.ok || field == APIC_F_FLUID_LIST || field == APIC_F_SORT_KEYS || field == APIC_F_SORT_VALS)
        return fail(APIC_ERR_INVALID_ARG, "field not writable: " + std::to_string(field));
    if (bytes != d.count * d.elem) return fail(APIC_ERR_INVALID_ARG, "size mismatch");
    if (bytes == 0) return APIC_OK;
    if (!src) return fail(APIC_ERR_INVALID_ARG, "null source");
    CK(cudaMemcpy(d.dev, src, bytes, cudaMemcpyHostToDevice));
    if (field == APIC_F_VEL_X || field == APIC_F_VEL_Y) s.vmax_valid = false;
    if (field == APIC_F_PRESSURE) s.p64_valid = false;
    if (field == APIC_F_OBSTACLE_BITS) {
        std::memcpy(h->obstacle_host.data(), src, bytes);
        int rc = upload_world(h);
        if (rc) return rc;
    }
    if (field == APIC_F_FLUID_BITS) {
        CK(launch_base_lists(s));
        CK(cudaStreamSynchronize(s.stream));
    }
    if (field >= APIC_F_MG_FLUID_BITS && field % APIC_F_MG_LEVEL_STRIDE == APIC_F_MG_FLUID_BITS) {
        CK(launch_level_lists(s, field / APIC_F_MG_LEVEL_STRIDE + 1));
        CK(cudaStreamSynchronize(s.stream));
    }
    if (field == APIC_F_EXT_FORCE_U || field == APIC_F_EXT_FORCE_V) s.has_ext = true;
    if (field == APIC_F_POST_FORCE_U || field == APIC_F_POST_FORCE_V) s.has_post = true;
    return APIC_OK;
}

int apic_read_vec2x8(apic_handle* h, int which, float* dst, uint64_t floats) {
    if (valid_handle(h) || which < 0 || which > 3) return fail(APIC_ERR_INVALID_ARG, "bad argument");
    Scene& s = h->s;
    if (floats != uint64_t(s.nchunks) * 16) return fail(APIC_ERR_INVALID_ARG, "size mismatch");
    if (floats == 0) return APIC_OK;
    if (!dst) return fail(APIC_ERR_INVALID_ARG, "null destination");
    // per chunk: 8 x lanes then 8 y lanes (ultraviolet::Vec2x8 {x: f32x8, y:
    // f32x8}), interleaved on the device, then one contiguous copy
    if (s.vec_stage_floats < floats) {
        CK(cudaStreamSynchronize(s.stream));
        dfree(s.vec_stage, s.stream);
        s.vec_stage = nullptr;
        s.vec_stage_floats = 0;
        if (dalloc(&s.vec_stage, floats, s.stream) != cudaSuccess)
            return fail(APIC_ERR_OOM, "out of device memory (Vec2x8 staging)");
        s.vec_stage_floats = uint32_t(floats);
    }
    CK(launch_pack_vec2x8(s, which, s.vec_stage));
    CK(cudaMemcpyAsync(dst, s.vec_stage, floats * sizeof(float), cudaMemcpyDeviceToHost, s.stream));
    CK(cudaStreamSynchronize(s.stream));
    return APIC_OK;
}

// ---- pipelined host I/O -------------------------------------------------------
// The stream-ordered forms of apic_update, apic_write_field (force fields)
// and apic_read_vec2x8: the copies run on the handle's upload and download
// streams, so a caller can upload the next update's forces and read back the
// last update's particles while an update runs.

int apic_update_async(apic_handle* h, uint32_t flags, float frame_dt) { return update_launch(h, flags, frame_dt); }

int apic_update_wait(apic_handle* h) {
    if (valid_handle(h)) return APIC_ERR_INVALID_ARG;
    return update_finish(h);
}

int apic_stage_field(apic_handle* h, int field, const void* src, uint64_t bytes) {
    if (valid_handle(h)) return APIC_ERR_INVALID_ARG;
    Scene& s = h->s;
    const int i = field == APIC_F_EXT_FORCE_U ? 0 : field == APIC_F_EXT_FORCE_V ? 1 : field == APIC_F_POST_FORCE_U ? 2
                : field == APIC_F_POST_FORCE_V ? 3 : -1;
    if (i < 0) return fail(APIC_ERR_INVALID_ARG, "only the external and post force fields can be staged");
    const uint64_t n = (i % 2 == 0) ? s.uf : s.vf;
    if (bytes != n * sizeof(float)) return fail(APIC_ERR_INVALID_ARG, "size mismatch");
    if (!src) return fail(APIC_ERR_INVALID_ARG, "null source");
    CK(ensure_pipeline(s));
    const int b = s.stage_next[i];
    if (!s.stage_buf[i][b]) {
        if (dalloc(&s.stage_buf[i][b], n, s.stream) != cudaSuccess)
            return fail(APIC_ERR_OOM, "out of device memory (force staging)");
        CK(cudaStreamSynchronize(s.stream));  // the pool allocation is ordered on the scene's stream
    }
    // the buffer may still be read by the copy of an update staged two calls ago
    CK(cudaStreamWaitEvent(s.up_stream, s.stage_used[i][b], 0));
    CK(cudaMemcpyAsync(s.stage_buf[i][b], src, bytes, cudaMemcpyHostToDevice, s.up_stream));
    CK(cudaEventRecord(s.stage_ready[i][b], s.up_stream));
    s.stage_pending[i] = b;
    s.stage_next[i] = b ^ 1;
    return APIC_OK;
}

int apic_read_vec2x8_async(apic_handle* h, int which, float* dst, uint64_t floats) {
    if (valid_handle(h) || which < 0 || which > 3) return fail(APIC_ERR_INVALID_ARG, "bad argument");
    Scene& s = h->s;
    if (floats != uint64_t(s.nchunks) * 16) return fail(APIC_ERR_INVALID_ARG, "size mismatch");
    if (floats == 0) return APIC_OK;
    if (!dst) return fail(APIC_ERR_INVALID_ARG, "null destination");
    CK(ensure_pipeline(s));
    const int b = s.read_next[which];
    if (s.read_floats[which][b] < floats) {
        CK(cudaStreamSynchronize(s.down_stream));
        CK(cudaStreamSynchronize(s.stream));
        dfree(s.read_buf[which][b], s.stream);
        s.read_buf[which][b] = nullptr;
        s.read_floats[which][b] = 0;
        if (dalloc(&s.read_buf[which][b], floats, s.stream) != cudaSuccess)
            return fail(APIC_ERR_OOM, "out of device memory (Vec2x8 staging)");
        s.read_floats[which][b] = floats;
    }
    // pack after the work already on the scene's stream, once the copy out of
    // this buffer two calls ago finished; copy out on the download stream
    CK(cudaStreamWaitEvent(s.stream, s.read_done[which][b], 0));
    CK(launch_pack_vec2x8(s, which, s.read_buf[which][b]));
    CK(cudaEventRecord(s.read_packed[which][b], s.stream));
    CK(cudaStreamWaitEvent(s.down_stream, s.read_packed[which][b], 0));
    CK(cudaMemcpyAsync(dst, s.read_buf[which][b], floats * sizeof(float), cudaMemcpyDeviceToHost, s.down_stream));
    CK(cudaEventRecord(s.read_done[which][b], s.down_stream));
    s.read_next[which] = b ^ 1;
    return APIC_OK;
}

int apic_read_wait(apic_handle* h) {
    if (valid_handle(h)) return APIC_ERR_INVALID_ARG;
    if (h->s.down_stream) CK(cudaStreamSynchronize(h->s.down_stream));
    return APIC_OK;
}

// ---- snapshot / restore -----------------------------------------------------
// The state a later update reads: the nine particle arrays (all padded lanes),
// the obstacle mask, pending external / post forces, the substep bookkeeping
// (timestamp, prev_deltatime) and the solver settings.  Everything else is
// rebuilt from the particles inside every substep.

namespace {

constexpr uint32_t kSnapMagic = 0x4E535041u;  // "APSN"
constexpr uint32_t kSnapVersion = 1;

struct SnapHeader {
    uint32_t magic, version;
    uint32_t width, height;
    float cell_size;
    apic_world_props props;
    uint32_t num_particles, lanes;
    uint32_t timestamp;
    float prev_deltatime;
    int32_t solver_mode;
    float rel_tol;
    uint32_t max_iterations;
    uint32_t has_ext, has_post;
    uint32_t obstacle_words;  // u64 words
    uint32_t u_faces, v_faces;
    uint32_t p64_words;       // FP64 pressure kept for the next mixed solve's start (0: none)
    uint32_t pad;
    uint64_t bytes;           // whole snapshot
};

uint64_t snap_bytes(uint32_t lanes, uint32_t obstacle_words, uint32_t uf, uint32_t vf, bool ext, bool post,
                    uint32_t p64_words) {
    return sizeof(SnapHeader) + uint64_t(NPF) * lanes * 4 + uint64_t(obstacle_words) * 8 +
           (ext ? uint64_t(uf + vf) * 4 : 0) + (post ? uint64_t(uf + vf) * 4 : 0) + uint64_t(p64_words) * 8;
}

// The warm start of the mixed solve reads the last solve's FP64 pressure.
uint32_t snap_p64_words(const Scene& s) { return warm_start(s) ? s.cells + 2 * s.W : 0u; }

}  // namespace

int apic_snapshot_bytes(apic_handle* h, uint64_t* bytes) {
    if (valid_handle(h) || !bytes) return fail(APIC_ERR_INVALID_ARG, "null argument");
    const Scene& s = h->s;
    *bytes = snap_bytes(s.npad, even_words(s.cells) / 2, s.uf, s.vf, s.has_ext, s.has_post, snap_p64_words(s));
    return APIC_OK;
}

int apic_snapshot(apic_handle* h, void* dst, uint64_t bytes) {
    uint64_t need = 0;
    int rc = apic_snapshot_bytes(h, &need);
    if (rc) return rc;
    if (bytes != need) return fail(APIC_ERR_INVALID_ARG, "size mismatch (apic_snapshot_bytes)");
    if (!dst) return fail(APIC_ERR_INVALID_ARG, "null destination");
    Scene& s = h->s;
    if ((rc = sync_ctl(s))) return rc;
    SnapHeader hd{};
    hd.magic = kSnapMagic;
    hd.version = kSnapVersion;
    hd.width = s.W;
    hd.height = s.H;
    hd.cell_size = s.dx;
    hd.props = s.props;
    hd.num_particles = s.n;
    hd.lanes = s.npad;
    hd.timestamp = s.ctl_host->timestamp;
    hd.prev_deltatime = s.ctl_host->prev_dt;
    hd.solver_mode = s.solver_mode;
    hd.rel_tol = s.rel_tol;
    hd.max_iterations = s.max_iter;
    hd.has_ext = s.has_ext;
    hd.has_post = s.has_post;
    hd.obstacle_words = even_words(s.cells) / 2;
    hd.u_faces = s.uf;
    hd.v_faces = s.vf;
    hd.p64_words = snap_p64_words(s);
    hd.bytes = need;
    uint8_t* out = static_cast<uint8_t*>(dst);
    std::memcpy(out, &hd, sizeof(hd));
    uint64_t off = sizeof(hd);
    auto take = [&](int field, uint64_t n) {
        int r = n ? apic_read_field(h, field, out + off, n) : APIC_OK;
        off += n;
        return r;
    };
    for (int f = APIC_F_POS_X; f <= APIC_F_TRES; ++f)
        if ((rc = take(f, uint64_t(s.npad) * 4))) return rc;
    if ((rc = take(APIC_F_OBSTACLE_BITS, uint64_t(hd.obstacle_words) * 8))) return rc;
    if (s.has_ext && ((rc = take(APIC_F_EXT_FORCE_U, uint64_t(s.uf) * 4)) ||
                      (rc = take(APIC_F_EXT_FORCE_V, uint64_t(s.vf) * 4))))
        return rc;
    if (s.has_post && ((rc = take(APIC_F_POST_FORCE_U, uint64_t(s.uf) * 4)) ||
                       (rc = take(APIC_F_POST_FORCE_V, uint64_t(s.vf) * 4))))
        return rc;
    if (hd.p64_words) CK(cudaMemcpy(out + off, s.p64, uint64_t(hd.p64_words) * 8, cudaMemcpyDeviceToHost));
    return APIC_OK;
}

int apic_restore(apic_handle* h, const void* src, uint64_t bytes) {
    if (valid_handle(h) || !src) return fail(APIC_ERR_INVALID_ARG, "null argument");
    if (bytes < sizeof(SnapHeader)) return fail(APIC_ERR_INVALID_ARG, "not a snapshot");
    Scene& s = h->s;
    SnapHeader hd;
    std::memcpy(&hd, src, sizeof(hd));
    if (hd.magic != kSnapMagic || hd.version != kSnapVersion) return fail(APIC_ERR_INVALID_ARG, "not a snapshot");
    if (hd.bytes != bytes || hd.lanes < hd.num_particles || hd.lanes % 8 != 0 ||
        bytes != snap_bytes(hd.lanes, hd.obstacle_words, hd.u_faces, hd.v_faces, hd.has_ext, hd.has_post,
                            hd.p64_words))
        return fail(APIC_ERR_INVALID_ARG, "snapshot size mismatch");
    if (hd.width != s.W || hd.height != s.H || std::memcmp(&hd.cell_size, &s.dx, 4) != 0 ||
        std::memcmp(&hd.props, &s.props, sizeof(apic_world_props)) != 0 || hd.u_faces != s.uf ||
        hd.v_faces != s.vf || hd.obstacle_words != even_words(s.cells) / 2 ||
        (hd.p64_words != 0 && hd.p64_words != s.cells + 2 * s.W))
        return fail(APIC_ERR_INVALID_ARG, "snapshot of a scene with another grid or world properties");
    const uint8_t* in = static_cast<const uint8_t*>(src) + sizeof(hd);
    const float* f[NPF];
    for (int k = 0; k < NPF; ++k) f[k] = reinterpret_cast<const float*>(in + uint64_t(k) * hd.lanes * 4);
    // particle count and padding first, then every lane exactly as saved
    int rc = apic_set_particles(h, hd.num_particles, f[PX], f[PY], f[VX], f[VY]);
    if (rc) return rc;
    if (s.npad != hd.lanes) return fail(APIC_ERR_INVALID_ARG, "snapshot lane count differs");
    for (int k = 0; k < NPF; ++k)
        if (hd.lanes && (rc = apic_write_field(h, APIC_F_POS_X + k, f[k], uint64_t(hd.lanes) * 4))) return rc;
    uint64_t off = uint64_t(NPF) * hd.lanes * 4;
    if ((rc = apic_write_field(h, APIC_F_OBSTACLE_BITS, in + off, uint64_t(hd.obstacle_words) * 8))) return rc;
    off += uint64_t(hd.obstacle_words) * 8;
    s.has_ext = s.has_post = false;
    if (hd.has_ext) {
        if ((rc = apic_write_field(h, APIC_F_EXT_FORCE_U, in + off, uint64_t(s.uf) * 4))) return rc;
        if ((rc = apic_write_field(h, APIC_F_EXT_FORCE_V, in + off + uint64_t(s.uf) * 4, uint64_t(s.vf) * 4)))
            return rc;
        off += uint64_t(s.uf + s.vf) * 4;
    }
    if (hd.has_post) {
        if ((rc = apic_write_field(h, APIC_F_POST_FORCE_U, in + off, uint64_t(s.uf) * 4))) return rc;
        if ((rc = apic_write_field(h, APIC_F_POST_FORCE_V, in + off + uint64_t(s.uf) * 4, uint64_t(s.vf) * 4)))
            return rc;
        off += uint64_t(s.uf + s.vf) * 4;
    }
    if (hd.p64_words) CK(cudaMemcpy(s.p64, in + off, uint64_t(hd.p64_words) * 8, cudaMemcpyHostToDevice));
    if ((rc = apic_set_solver(h, hd.solver_mode, hd.rel_tol, hd.max_iterations))) return rc;
    CK(cudaMemcpy(&s.ctl->timestamp, &hd.timestamp, sizeof(uint32_t), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(&s.ctl->prev_dt, &hd.prev_deltatime, sizeof(float), cudaMemcpyHostToDevice));
    s.vmax_valid = false;
    return APIC_OK;
}

int apic_render(apic_handle* h, const apic_render_params* rp, apic_render_stats* out) {
    if (valid_handle(h) || !rp) return fail(APIC_ERR_INVALID_ARG, "null argument");
    Scene& s = h->s;
    const apic_render_params& q = *rp;
    if (q.width == 0 || q.height == 0 || q.width > 16384 || q.height > 16384)
        return fail(APIC_ERR_INVALID_ARG, "frame size must be 1..16384 pixels per side");
    if (!(q.scale > 0.0f) || !std::isfinite(q.scale)) return fail(APIC_ERR_INVALID_ARG, "scale must be > 0");
    if (!(q.draw_radius > 0.0f) || q.draw_radius > 7.0f)
        return fail(APIC_ERR_INVALID_ARG, "draw_radius must be in (0, 7]");
    if (!(q.margin >= 0.0f) || q.margin > 65536.0f) return fail(APIC_ERR_INVALID_ARG, "margin must be in [0, 65536]");
    if (!std::isfinite(q.pick_x) || !std::isfinite(q.pick_y) || std::isnan(q.pick_radius))
        return fail(APIC_ERR_INVALID_ARG, "pick centre and radius must be finite");
    if (uint64_t(s.n) * 4 > 0x7FFFFFFFull) return fail(APIC_ERR_INVALID_ARG, "too many particles to render");
    RenderParamsDev p{};
    p.width = q.width;
    p.height = q.height;
    p.ntx = div_up(q.width, 16);
    p.nty = div_up(q.height, 16);
    p.ntiles = p.ntx * p.nty;
    p.fw = float(q.width);
    p.fh = float(q.height);
    p.scale = q.scale;
    p.margin = q.margin;
    p.radius = q.draw_radius;
    p.size = q.draw_radius * 2.0f;
    p.tex_scale = 32.0f / p.size;
    p.pick_x = q.pick_x;
    p.pick_y = q.pick_y;
    p.pick_r2 = q.pick_radius < 0.0f ? -1.0f : q.pick_radius * q.pick_radius;
    p.bg = q.background;
    RenderResult r{};
    cudaError_t e = render_frame(s, p, &r);
    if (e == cudaErrorMemoryAllocation) return fail(APIC_ERR_OOM, "out of device memory (render buffers)");
    if (e != cudaSuccess) return fail(APIC_ERR_CUDA, std::string("render: ") + cudaGetErrorString(e));
    if (out) {
        out->valid = r.valid;
        out->nan = r.nan;
        out->out_of_bounds = r.oob;
        out->fluid_cells = s.ctl_host ? s.ctl_host->fluid_cells : 0u;
        out->picked = r.picked;
        out->volume = float(out->fluid_cells) * (s.dx * s.dx);
        out->kernels = r.kernels;
    }
    return APIC_OK;
}

int apic_read_frame(apic_handle* h, uint8_t* dst, uint64_t bytes) {
    if (valid_handle(h)) return APIC_ERR_INVALID_ARG;
    uint32_t w = 0, ht = 0;
    const uint32_t* f = render_frame_ptr(h->s, &w, &ht);
    if (!f) return fail(APIC_ERR_INVALID_ARG, "no frame rendered yet");
    if (bytes != uint64_t(w) * ht * 4) return fail(APIC_ERR_INVALID_ARG, "size mismatch");
    if (!dst) return fail(APIC_ERR_INVALID_ARG, "null destination");
    CK(cudaMemcpyAsync(dst, f, bytes, cudaMemcpyDeviceToHost, h->s.stream));
    CK(cudaStreamSynchronize(h->s.stream));
    return APIC_OK;
}

int apic_frame_device_ptr(apic_handle* h, void** ptr, uint32_t* width, uint32_t* height) {
    if (valid_handle(h) || !ptr || !width || !height) return fail(APIC_ERR_INVALID_ARG, "null argument");
    uint32_t w = 0, ht = 0;
    const uint32_t* f = render_frame_ptr(h->s, &w, &ht);
    if (!f) return fail(APIC_ERR_INVALID_ARG, "no frame rendered yet");
    *ptr = const_cast<uint32_t*>(f);
    *width = w;
    *height = ht;
    return APIC_OK;
}

int apic_set_option(apic_handle* h, int option, int value) {
    if (valid_handle(h)) return APIC_ERR_INVALID_ARG;
    Scene& s = h->s;
    if (s.stream) cudaStreamSynchronize(s.stream);
    switch (option) {
        case APIC_OPT_PDL:
            s.use_pdl = value != 0;
            invalidate_graphs(s);
            return APIC_OK;
        case APIC_OPT_DSM_VCYCLE:
            s.use_dsm = value != 0;
            invalidate_graphs(s);
            return APIC_OK;
        case APIC_OPT_WARM_START:
            s.warm_start = value != 0;
            invalidate_graphs(s);
            return APIC_OK;
        case APIC_OPT_P2G_ORDER:
            if (value < 0 || value > 2) return fail(APIC_ERR_INVALID_ARG, "P2G order must be 0, 1 or 2");
            s.p2g_order = value;
            invalidate_graphs(s);
            return APIC_OK;
        case APIC_OPT_STREAM_PRIORITY: {
            if (value < 0) return fail(APIC_ERR_INVALID_ARG, "stream priority must be >= 0");
            // the scene's stream is idle (synchronised above): replace it by
            // one of the asked priority; graphs launch into it unchanged
            int least = 0, greatest = 0;
            CK(cudaDeviceGetStreamPriorityRange(&least, &greatest));
            const int prio = std::max(greatest, least - value);
            cudaStream_t ns = nullptr;
            CK(cudaStreamCreateWithPriority(&ns, cudaStreamNonBlocking, prio));
            if (s.stream) cudaStreamDestroy(s.stream);
            s.stream = ns;
            s.priority = least - prio;
            return APIC_OK;
        }
        default: return fail(APIC_ERR_INVALID_ARG, "unknown option");
    }
}

int apic_get_option(apic_handle* h, int option, int* value) {
    if (valid_handle(h) || !value) return fail(APIC_ERR_INVALID_ARG, "null argument");
    switch (option) {
        case APIC_OPT_PDL: *value = h->s.use_pdl ? 1 : 0; return APIC_OK;
        case APIC_OPT_DSM_VCYCLE:
            *value = (h->s.use_dsm && h->s.dsm_first < h->s.dsm_tail) ? 1 : 0;
            return APIC_OK;
        case APIC_OPT_WARM_START: *value = h->s.warm_start ? 1 : 0; return APIC_OK;
        case APIC_OPT_STREAM_PRIORITY: *value = h->s.priority; return APIC_OK;
        case APIC_OPT_P2G_ORDER: *value = p2g_reference_order(h->s) ? 1 : 2; return APIC_OK;
        default: return fail(APIC_ERR_INVALID_ARG, "unknown option");
    }
}

int apic_set_profiling(apic_handle* h, int enabled) {
    if (valid_handle(h)) return APIC_ERR_INVALID_ARG;
    h->s.profiling = enabled != 0;
    return APIC_OK;
}

int apic_get_stage_times(apic_handle* h, double* ms, uint64_t* launches, int n) {
    if (valid_handle(h)) return APIC_ERR_INVALID_ARG;
    for (int i = 0; i < n && i < APIC_STAGE_COUNT; ++i) {
        if (ms) ms[i] = h->s.stage_ms[i];
        if (launches) launches[i] = h->s.stage_launches[i];
    }
    return APIC_OK;
}

int apic_reset_stage_times(apic_handle* h) {
    if (valid_handle(h)) return APIC_ERR_INVALID_ARG;
    for (int i = 0; i < APIC_STAGE_COUNT; ++i) { h->s.stage_ms[i] = 0; h->s.stage_launches[i] = 0; }
    return APIC_OK;
}

int apic_synchronize(apic_handle* h) {
    if (valid_handle(h)) return APIC_ERR_INVALID_ARG;
    CK(cudaStreamSynchronize(h->s.stream));
    return APIC_OK;
}

int apic_get_stream(apic_handle* h, void** stream_out) {
    if (valid_handle(h) || !stream_out) return fail(APIC_ERR_INVALID_ARG, "null argument");
    *stream_out = reinterpret_cast<void*>(h->s.stream);
    return APIC_OK;
}

int apic_debug_run_stage(apic_handle* h, int stage, float dt) {
    if (valid_handle(h)) return APIC_ERR_INVALID_ARG;
    Scene& s = h->s;
    cudaStream_t st = s.stream;
    k_set_dt<<<1, 1, 0, st>>>(s.ctl, dt, s.has_ext ? 1u : 0u, s.has_post ? 1u : 0u);
    switch (stage) {
        case APIC_STAGE_SORT: CK(launch_sort(s)); break;
        case APIC_STAGE_P2G:
            CK(clear_p2g_targets(s));
            CK(launch_p2g(s));
            CK(launch_finalize_faces(s, false, false));
            CK(launch_base_lists(s));
            break;
        case APIC_STAGE_FORCES: CK(launch_external_forces(s)); break;
        case APIC_STAGE_BUILD: CK(launch_base_lists(s)); CK(launch_build_pressure(s)); break;
        case APIC_STAGE_MG: CK(launch_base_lists(s)); CK(launch_multilevel(s)); break;
        case APIC_STAGE_PCG: {
            k_begin_update<<<1, 1, 0, st>>>(s.ctl, 0.0f, 0u, s.has_ext ? 1u : 0u, s.has_post ? 1u : 0u);
            k_set_dt<<<1, 1, 0, st>>>(s.ctl, dt, s.has_ext ? 1u : 0u, s.has_post ? 1u : 0u);
            CK(run_solve_eager(s));
            int rc = sync_ctl(s);
            if (rc) return rc;
            const Ctl& c = *s.ctl_host;
            s.stats.pcg_iterations = c.pcg_iters;
            s.stats.pcg_iterations_total = c.pcg_iters_total;
            s.stats.residual_max = bits_to_float(c.max_r_bits);
            s.stats.true_residual_rel = c.true_rel;
            s.stats.not_converged = c.not_converged;
            s.stats.refinement_steps = c.refinements;
            break;
        }
        case APIC_STAGE_GRAD: CK(launch_gradient(s, false)); break;
        case APIC_STAGE_POST: CK(launch_post_forces(s)); break;
        case APIC_STAGE_EXTRAP: CK(launch_extrapolate(s)); break;
        case APIC_STAGE_G2P: {
            CK(launch_g2p(s));
            break;
        }
        case APIC_STAGE_VMAX: CK(launch_vmax(s)); s.vmax_valid = true; break;
        case APIC_STAGE_VCYCLE:
            k_begin_update<<<1, 1, 0, st>>>(s.ctl, 0.0f, 0u, 0u, 0u);  // clears the solve's done flag
            enqueue_vcycle(s);
            CK(cudaGetLastError());
            break;
        default: return fail(APIC_ERR_INVALID_ARG, "unknown stage");
    }
    CK(cudaStreamSynchronize(st));
    return APIC_OK;
}

// Test hook: end-of-substep bookkeeping (prev_deltatime, timestamp).
int apic_debug_finish_substep(apic_handle* h, float dt) {
    if (valid_handle(h)) return APIC_ERR_INVALID_ARG;
    k_stage_finish<<<1, 1, 0, h->s.stream>>>(h->s.ctl, dt);
    CK(cudaStreamSynchronize(h->s.stream));
    return APIC_OK;
}

}  // extern "C"
