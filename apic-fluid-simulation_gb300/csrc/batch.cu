// batch.cu — apic_update_batch as one CUDA graph with the pressure solves of
// all scenes as one launch per solve phase.
//
// Each scene runs Apic::update (src/apic.rs:2429-2474).  The graph:
//
//   plan every scene's first substep (k_bat_plan_first)
//   per scene, side by side: IF(first substep sorts) { the Morton sort }
//   WHILE(some scene has a substep due) {
//       k_bat_due: per scene, is a substep due
//       per scene, side by side: IF(due) { stages before the solve }
//       the solves of all scenes: one launch per phase over the scene
//           table, each walking the items of the scenes that take part
//           (batch.h)
//       per scene, side by side: IF(due) { stages after the solve }
//       k_bat_advance: end every due scene's substep, plan its next one
//   }
//
// A scene's stages are its own kernels, recorded exactly as in its own
// update graph; the solve phases run the single-scene kernels' bodies with
// each scene's block coordinates.  So every scene computes bit for bit what
// apic_update computes for it, while a batch of small scenes costs one launch
// per solve phase instead of one per scene and phase (the batch of small
// scenes is bound by the rate at which the GPU takes launches).
//
// The V-cycle of a batched solve runs the coarse tail (the levels that fit in
// one CTA's shared memory) as one CTA per scene, and the levels above it with
// the segment kernels; the single-scene form may hold some of those levels
// in a cluster's distributed shared memory instead, which computes the same
// values.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "apic_device.cuh"
#include "apic_graph.h"
#include "apic_internal.h"
#include "batch.h"
#include "substep.cuh"

namespace apic {
namespace {

constexpr int kCtlThreads = 1024;

// ---- substep control over the batch ----------------------------------------
// One block, a thread per scene (the per-scene kernels k_plan_first_g /
// k_advance_g of runtime.cu, with the loop condition the OR over scenes).

__global__ void __launch_bounds__(kCtlThreads) k_bat_plan_first(const BScene* __restrict__ tab, uint32_t n,
                                                               const cudaGraphConditionalHandle* __restrict__ h_sort,
                                                               cudaGraphConditionalHandle h_loop) {
    bool any = false;
    for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) {
        Ctl* c = tab[i].ctl;
        plan(c);
        cudaGraphSetConditional(h_sort[i], (c->go && c->sort_now) ? 1u : 0u);
        any = any || c->go;
    }
    any = __syncthreads_or(any) != 0;
    if (threadIdx.x == 0) cudaGraphSetConditional(h_loop, any ? 1u : 0u);
}

__global__ void __launch_bounds__(kCtlThreads) k_bat_due(const BScene* __restrict__ tab, uint32_t n,
                                                        const cudaGraphConditionalHandle* __restrict__ h_pre,
                                                        const cudaGraphConditionalHandle* __restrict__ h_post,
                                                        BCtl* bc) {
    for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) {
        const uint32_t go = tab[i].ctl->go ? 1u : 0u;
        cudaGraphSetConditional(h_pre[i], go);
        cudaGraphSetConditional(h_post[i], go);
    }
    if (threadIdx.x == 0) bc->substeps++;
}

__global__ void __launch_bounds__(kCtlThreads) k_bat_advance(const BScene* __restrict__ tab, uint32_t n,
                                                            cudaGraphConditionalHandle h_loop) {
    bool any = false;
    for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) {
        Ctl* c = tab[i].ctl;
        if (!c->go) continue;
        advance(c);
        any = any || c->go;
    }
    any = __syncthreads_or(any) != 0;
    if (threadIdx.x == 0) cudaGraphSetConditional(h_loop, any ? 1u : 0u);
}

// ---- the batch -------------------------------------------------------------

struct Batch {
    std::vector<Scene*> scenes;
    std::vector<uint64_t> versions;
    int mode = 0;
    BScene* d_tab = nullptr;
    BCtl* d_bc = nullptr;
    BCtl* h_bc = nullptr;  // pinned copy read after the batch
    uint32_t* d_lists = nullptr;  // the scene lists of gates 1..3
    cudaGraphConditionalHandle* d_handles = nullptr;  // sort, pre, post: n each
    int max_tail = 0;             // deepest first tail level over the scenes
    size_t tail_smem = 0;
    cudaStream_t stream = nullptr, cap = nullptr;
    cudaEvent_t done = nullptr;
    std::vector<cudaEvent_t> ready;
    cudaGraphExec_t exec = nullptr;
    // kernel nodes of the batch's own graph bodies (launch accounting)
    uint32_t kn_top = 0, kn_loop = 0, kn_refine = 0, kn_pcg = 0;
};

void free_batch(Batch& b) {
    if (b.stream) cudaStreamSynchronize(b.stream);
    if (b.exec) cudaGraphExecDestroy(b.exec);
    cudaFree(b.d_tab);
    cudaFree(b.d_bc);
    cudaFree(b.d_lists);
    cudaFree(b.d_handles);
    if (b.h_bc) cudaFreeHost(b.h_bc);
    for (cudaEvent_t e : b.ready) cudaEventDestroy(e);
    if (b.done) cudaEventDestroy(b.done);
    if (b.cap) cudaStreamDestroy(b.cap);
    if (b.stream) cudaStreamDestroy(b.stream);
    b = Batch{};
}

std::mutex g_batch_mu;
Batch g_batch;                 // the graph of the last joint batch (rebuilt when its scene list changes)
apic_batch_info g_last_info{};

// ---- the batch tuner ---------------------------------------------------------
// The first calls for a batch of a given makeup (sides, coarse-tail depth and
// solver mode of every scene, in order) try each way of running it: every
// scene on its own stream, and the joint graph with each shape (segments per
// chunk item, blocks per reduction item), each twice in two interleaved
// sweeps.  A call's cost is its wall time per PCG iteration summed over the
// scenes; the first call of each form (which builds graphs) is not
// measured.  Every way computes the same bits, so the tuning runs on the
// caller's own updates.  Then the way with the lowest mean cost is kept for
// every later batch of that makeup.
struct TuneStep {
    int joint;       // 0: each scene on its own stream
    Shape shape;
    bool measure;
};
struct Tuner {
    std::vector<TuneStep> steps;
    std::vector<double> cost;  // per step, < 0 until measured
    size_t next = 0;           // next step to run
    int best = -1;             // the chosen step once all have run
};
std::map<uint64_t, Tuner> g_tuners;
constexpr size_t kMaxTuners = 256;  // makeups remembered (all are forgotten beyond this)

const std::vector<TuneStep>& tune_steps() {
    static const std::vector<TuneStep> steps = [] {
        std::vector<TuneStep> v;
        v.push_back({0, {64, 4}, false});
        v.push_back({1, {64, 4}, false});
        // every measured form twice, interleaved: a scene's cost drifts from
        // update to update as its flow evolves
        const size_t first = v.size();
        v.push_back({0, {64, 4}, true});
        for (uint32_t cs : {16u, 32u, 64u})
            for (uint32_t bg : {4u, 8u, 16u, 32u}) v.push_back({1, {cs, bg}, true});
        const size_t last = v.size();
        for (size_t i = first; i < last; ++i) v.push_back(v[i]);
        return v;
    }();
    return steps;
}

uint64_t makeup_key(apic_handle* const* handles, uint32_t count) {
    uint64_t h = 1469598103934665603ull;
    auto mix = [&](uint64_t v) { h = (h ^ v) * 1099511628211ull; };
    mix(count);
    for (uint32_t i = 0; i < count; ++i) {
        const Scene& s = scene_of(handles[i]);
        mix(s.W);
        mix(s.H);
        mix(uint64_t(s.tail_first));
        mix(uint64_t(s.solver_mode));
    }
    return h;
}

bool same_batch(const Batch& b, apic_handle* const* handles, uint32_t count) {
    if (!b.exec || b.scenes.size() != count) return false;
    for (uint32_t i = 0; i < count; ++i) {
        Scene& s = scene_of(handles[i]);
        if (b.scenes[i] != &s || b.versions[i] != s.graph_version || s.solver_mode != b.mode) return false;
    }
    return true;
}

BScene make_bscene(Scene& s) {
    BScene t;
    std::memset(&t, 0, sizeof(t));
    for (int l = 0; l < s.nlevels; ++l) {
        t.lv[l] = s.lv[l];
        t.grid[l] = seg_grid(s.lv[l].words);
    }
    t.ctl = s.ctl;
    t.search = s.search;
    t.ap = s.ap;
    t.corr = s.corr;
    t.pressure = s.pressure;
    t.b64 = s.b64;
    t.p64 = s.p64;
    t.partials = s.partials;
    t.nlevels = uint32_t(s.nlevels);
    t.tail_first = uint32_t(s.tail_first);
    t.max_iter = s.max_iter;
    t.warm = warm_start(s);
    t.tol = double(s.rel_tol);
    uint32_t words = 0;
    t.tp = vc::make_tail_params(s, s.tail_first, &words);
    return t;
}

// The V-cycle (enqueue_vcycle's sequence without the distributed levels):
// every scene runs its own levels' kernels in its own order; a launch covers
// the scenes that have that kernel at that point.
void bat_vcycle(const BatchRun& r, int max_tail, int gate, bool in_iteration) {
    if (!in_iteration) {
        bat_smooth(r, 0, gate, 0, 1);
        bat_smooth(r, 0, gate, 1, 1);
    } else {
        bat_smooth_exit(r);  // k_pcg_update ran the red sweep
    }
    for (int l = 1; l <= max_tail; ++l) {
        bat_restrict(r, l, gate);
        if (l < max_tail) bat_smooth(r, l, gate, 1, 1);  // no scene smooths its deepest level here
    }
    bat_tail(r, gate);
    for (int l = max_tail - 1; l >= 1; --l) {
        bat_prolong_black(r, l, gate, 0);
        bat_prolong_red(r, l, gate, 0);
    }
    bat_prolong_black(r, 0, gate, 1);
    if (in_iteration)
        bat_prolong_red_rz(r);
    else
        bat_prolong_red(r, 0, gate, 1);
}

// build_pcg over the batch: setup, then WHILE(some scene's PCG goes on).
cudaError_t bat_pcg(Batch& b, const BatchRun& r, GraphCursor& c, int setup_gate, bool begin, int into_corr) {
    cudaGraphConditionalHandle hp;
    cudaError_t e = cudaGraphConditionalHandleCreate(&hp, c.g, 0, cudaGraphCondAssignDefault);
    if (e != cudaSuccess) return e;
    e = capture_on(r.st, c, [&]() {
        if (begin) bat_pcg_begin(r, setup_gate);
        bat_vcycle(r, b.max_tail, setup_gate, false);
        bat_pcg_start(r, setup_gate);
        bat_pcg_cond(r, hp, setup_gate);
        return cudaGetLastError();
    });
    if (e != cudaSuccess) return e;
    GraphCursor body;
    if ((e = add_conditional_with(c, cudaGraphCondTypeWhile, hp, &body)) != cudaSuccess) return e;
    e = capture_on(r.st, body, [&]() {
        bat_spmv_dot(r);
        bat_sap(r);
        bat_pcg_update(r, into_corr);
        bat_vcycle(r, b.max_tail, kGatePcg, true);
        bat_round_end(r, hp);
        return cudaGetLastError();
    });
    b.kn_pcg = count_kernel_nodes(body.g);
    return e;
}

// build_solve over the batch (relative modes).
cudaError_t bat_solve(Batch& b, const BatchRun& r, GraphCursor& c) {
    const bool mixed = b.mode == APIC_SOLVER_REL_MIXED;
    cudaError_t e = capture_on(r.st, c, [&]() {
        bat_solve_begin(r);
        bat_mixed_init(r, kGateSolve);
        bat_clear_pressure(r, kGateSolve);
        bat_rel_begin(r, mixed ? 1 : 0);
        return cudaGetLastError();
    });
    if (e != cudaSuccess) return e;
    if (!mixed) {
        if ((e = bat_pcg(b, r, c, kGateSolve, true, 0)) != cudaSuccess) return e;
        return capture_on(r.st, c, [&]() {
            bat_finish_solve(r);
            bat_pressure_to64(r, kGateSolve);
            bat_true_residual(r, kGateSolve, 1);
            return cudaGetLastError();
        });
    }
    cudaGraphConditionalHandle hr;
    if ((e = cudaGraphConditionalHandleCreate(&hr, c.g, 0, cudaGraphCondAssignDefault)) != cudaSuccess) return e;
    e = capture_on(r.st, c, [&]() {
        bat_true_residual(r, kGateSolve, 3);
        bat_refine_cond(r, hr, kGateSolve);
        return cudaGetLastError();
    });
    if (e != cudaSuccess) return e;
    GraphCursor body;
    if ((e = add_conditional_with(c, cudaGraphCondTypeWhile, hr, &body)) != cudaSuccess) return e;
    if ((e = bat_pcg(b, r, body, kGateRefine, false, 1)) != cudaSuccess) return e;
    e = capture_on(r.st, body, [&]() {
        bat_mixed_accumulate(r, kGateRefine, 0);
        bat_true_residual(r, kGateRefine, 3);
        bat_refine_cond(r, hr, kGateRefine);
        return cudaGetLastError();
    });
    if (e != cudaSuccess) return e;
    b.kn_refine = count_kernel_nodes(body.g);
    return capture_on(r.st, c, [&]() {
        bat_mixed_accumulate(r, kGateSolve, 1);
        bat_refine_end(r);
        return cudaGetLastError();
    });
}

// One IF node per scene after c.tail, side by side; the cursor then waits on
// all of them.  `enqueue` records the scene's body; kn[i] adds its kernels.
template <class F>
cudaError_t scene_ifs(Batch& b, GraphCursor& c, std::vector<cudaGraphConditionalHandle>& hs, std::vector<uint32_t>& kn,
                      F&& enqueue) {
    const std::vector<cudaGraphNode_t> base = c.tail;
    std::vector<cudaGraphNode_t> tails;
    hs.assign(b.scenes.size(), 0);
    for (size_t i = 0; i < b.scenes.size(); ++i) {
        Scene& s = *b.scenes[i];
        cudaError_t e = cudaGraphConditionalHandleCreate(&hs[i], c.g, 0, cudaGraphCondAssignDefault);
        if (e != cudaSuccess) return e;
        GraphCursor ci;
        ci.g = c.g;
        ci.tail = base;
        GraphCursor body;
        if ((e = add_conditional_with(ci, cudaGraphCondTypeIf, hs[i], &body)) != cudaSuccess) return e;
        if ((e = capture_into(s, body, [&]() { return enqueue(s); })) != cudaSuccess) return e;
        kn[i] += count_kernel_nodes(body.g);
        tails.push_back(ci.tail[0]);
    }
    c.tail = tails;
    return cudaSuccess;
}

#define BCK(call)                                                  \
    do {                                                           \
        cudaError_t e_ = (call);                                   \
        if (e_ != cudaSuccess) return std::string(#call) + ": " + cudaGetErrorString(e_); \
    } while (0)

// Tables, maps and the graph of a new batch.  Returns "" or the failure.
std::string build_batch(Batch& b, apic_handle* const* handles, uint32_t count) {
    b.mode = scene_of(handles[0]).solver_mode;
    for (uint32_t i = 0; i < count; ++i) {
        Scene& s = scene_of(handles[i]);
        b.scenes.push_back(&s);
        b.versions.push_back(s.graph_version);
    }
    const uint32_t n = count;
    // scene table
    std::vector<BScene> tab(n);
    for (uint32_t i = 0; i < n; ++i) {
        tab[i] = make_bscene(*b.scenes[i]);
        uint32_t words = 0;
        vc::make_tail_params(*b.scenes[i], b.scenes[i]->tail_first, &words);
        b.tail_smem = std::max(b.tail_smem, size_t(words) * 4);
        b.max_tail = std::max(b.max_tail, b.scenes[i]->tail_first);
    }
    // the scene lists of gates 1..3 (written by the control kernels)
    BListRef proto;
    proto.N = n;
    proto.K = kinds_for(b.max_tail);
    BCK(cudaMalloc(&b.d_lists, sizeof(uint32_t) * 3 * proto.words()));
    BCK(cudaMemset(b.d_lists, 0, sizeof(uint32_t) * 3 * proto.words()));
    BCK(cudaMalloc(&b.d_tab, sizeof(BScene) * n));
    BCK(cudaMemcpy(b.d_tab, tab.data(), sizeof(BScene) * n, cudaMemcpyHostToDevice));
    BCK(cudaMalloc(&b.d_bc, sizeof(BCtl)));
    BCK(cudaMemset(b.d_bc, 0, sizeof(BCtl)));
    BCK(cudaMallocHost(&b.h_bc, sizeof(BCtl)));
    BCK(cudaMalloc(&b.d_handles, sizeof(cudaGraphConditionalHandle) * 3 * n));
    BCK(cudaStreamCreateWithFlags(&b.stream, cudaStreamNonBlocking));
    BCK(cudaStreamCreateWithFlags(&b.cap, cudaStreamNonBlocking));
    BCK(cudaEventCreateWithFlags(&b.done, cudaEventDisableTiming));
    b.ready.assign(n, nullptr);
    for (uint32_t i = 0; i < n; ++i) BCK(cudaEventCreateWithFlags(&b.ready[i], cudaEventDisableTiming));
    bat_prepare_tail();

    BatchRun r;
    r.tab = b.d_tab;
    r.bc = b.d_bc;
    r.nscenes = n;
    r.st = b.cap;
    r.pdl = true;
    r.tail_smem = b.tail_smem;
    for (int g = 1; g <= 3; ++g) {
        r.list[g] = proto;
        r.list[g].p = b.d_lists + size_t(g - 1) * proto.words();
    }
    // the projection reads the refined FP64 pressure in the mixed mode (as
    // build_solve arranges for a scene's own graph)
    for (Scene* s : b.scenes) s->p64_valid = b.mode == APIC_SOLVER_REL_MIXED;

    std::vector<cudaGraphConditionalHandle> h_sort, h_pre, h_post;
    std::vector<uint32_t> kn_sort(n, 0), kn_step(n, 0);
    GraphCursor top;
    BCK(cudaGraphCreate(&top.g, 0));
    struct GraphGuard {
        cudaGraph_t g;
        ~GraphGuard() { cudaGraphDestroy(g); }
    } guard{top.g};
    cudaGraphConditionalHandle h_loop;
    BCK(cudaGraphConditionalHandleCreate(&h_loop, top.g, 0, cudaGraphCondAssignDefault));
    BCK(capture_on(b.cap, top, [&]() {
        k_bat_plan_first<<<1, kCtlThreads, 0, b.cap>>>(b.d_tab, n, b.d_handles, h_loop);
        return cudaGetLastError();
    }));
    BCK(scene_ifs(b, top, h_sort, kn_sort, [](Scene& s) { return launch_sort(s); }));
    GraphCursor loop;
    BCK(add_conditional_with(top, cudaGraphCondTypeWhile, h_loop, &loop));
    // the IF nodes' handles belong to the loop body, where k_bat_due sets them
    BCK(capture_on(b.cap, loop, [&]() {
        k_bat_due<<<1, kCtlThreads, 0, b.cap>>>(b.d_tab, n, b.d_handles + n, b.d_handles + 2 * n, b.d_bc);
        return cudaGetLastError();
    }));
    BCK(scene_ifs(b, loop, h_pre, kn_step, [](Scene& s) { return scene_pre_solve(s); }));
    BCK(bat_solve(b, r, loop));
    BCK(scene_ifs(b, loop, h_post, kn_step, [](Scene& s) { return scene_post_solve(s); }));
    BCK(capture_on(b.cap, loop, [&]() {
        k_bat_advance<<<1, kCtlThreads, 0, b.cap>>>(b.d_tab, n, h_loop);
        return cudaGetLastError();
    }));
    b.kn_top = count_kernel_nodes(top.g);
    b.kn_loop = count_kernel_nodes(loop.g);
    std::vector<cudaGraphConditionalHandle> hv;
    hv.insert(hv.end(), h_sort.begin(), h_sort.end());
    hv.insert(hv.end(), h_pre.begin(), h_pre.end());
    hv.insert(hv.end(), h_post.begin(), h_post.end());
    BCK(cudaMemcpy(b.d_handles, hv.data(), sizeof(cudaGraphConditionalHandle) * hv.size(), cudaMemcpyHostToDevice));
    BCK(cudaGraphInstantiate(&b.exec, top.g, 0));
    for (uint32_t i = 0; i < n; ++i) {
        b.scenes[i]->kn_bsort = kn_sort[i];
        b.scenes[i]->kn_bstep = kn_step[i];
    }
    return "";
}

}  // namespace

// The joint form applies when every scene solves in the same relative mode,
// has a multigrid level and a shared-memory coarse tail, lives on the
// current device, and is not in profiling mode (whose host-driven loops read
// each scene's state).
bool batch_eligible(apic_handle* const* handles, uint32_t count) {
    if (count < 2 || count > 0xFFFFu) return false;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return false;
    const int mode = scene_of(handles[0]).solver_mode;
    if (mode != APIC_SOLVER_REL_FP32 && mode != APIC_SOLVER_REL_MIXED) return false;
    for (uint32_t i = 0; i < count; ++i) {
        const Scene& s = scene_of(handles[i]);
        if (s.profiling || s.solver_mode != mode || s.nlevels < 2) return false;
        if (s.device != dev) return false;  // one graph runs on one device
        if (s.tail_first < 1 || s.tail_first >= s.nlevels) return false;
        if (s.n == 0) return false;
    }
    return true;
}

void batch_note_streams(uint32_t count) {
    std::lock_guard<std::mutex> lk(g_batch_mu);
    g_last_info = apic_batch_info{};
    g_last_info.scenes = count;
}

// The way to run this call: t->joint (with t->shape) or streams.
// force_joint: joint whatever the tuner's state (its best shape when tuned).
void batch_choose(apic_handle* const* handles, uint32_t count, bool force_joint, BatchTicket* tk) {
    std::lock_guard<std::mutex> lk(g_batch_mu);
    const uint64_t key = makeup_key(handles, count);
    tk->key = key;
    tk->step = -1;
    if (force_joint) {
        auto it = g_tuners.find(key);
        const bool tuned_joint = it != g_tuners.end() && it->second.best >= 0 &&
                                 it->second.steps[size_t(it->second.best)].joint;
        tk->shape = tuned_joint ? it->second.steps[size_t(it->second.best)].shape : Shape{64, 4};
        tk->joint = 1;
        return;
    }
    if (g_tuners.size() >= kMaxTuners && g_tuners.find(key) == g_tuners.end()) g_tuners.clear();
    Tuner& t = g_tuners[key];
    if (t.steps.empty()) {
        t.steps = tune_steps();
        t.cost.assign(t.steps.size(), -1.0);
    }
    if (t.best < 0 && t.next < t.steps.size()) {
        tk->step = int(t.next++);
        tk->shape = t.steps[size_t(tk->step)].shape;
        tk->joint = t.steps[size_t(tk->step)].joint;
        return;
    }
    if (t.best < 0) {  // every step ran: keep the form with the lowest mean cost
        double c = 0.0;
        for (size_t i = 0; i < t.steps.size(); ++i) {
            if (!t.steps[i].measure || t.cost[i] < 0.0) continue;
            double sum = 0.0;
            int k = 0;
            for (size_t j = 0; j < t.steps.size(); ++j)
                if (t.steps[j].measure && t.cost[j] >= 0.0 && t.steps[j].joint == t.steps[i].joint &&
                    t.steps[j].shape.chunk_segs == t.steps[i].shape.chunk_segs &&
                    t.steps[j].shape.block_group == t.steps[i].shape.block_group) {
                    sum += t.cost[j];
                    ++k;
                }
            if (t.best < 0 || sum / k < c) {
                t.best = int(i);
                c = sum / k;
            }
        }
        if (t.best < 0) t.best = 0;
    }
    tk->shape = t.steps[size_t(t.best)].shape;
    tk->joint = t.steps[size_t(t.best)].joint;
}

// Cost of the call that batch_choose planned (wall time, PCG iterations over
// all scenes).
void batch_record(const BatchTicket& tk, double wall_ms, uint64_t iterations) {
    std::lock_guard<std::mutex> lk(g_batch_mu);
    g_last_info.chunk_segs = tk.shape.chunk_segs;
    g_last_info.block_group = tk.shape.block_group;
    auto it = g_tuners.find(tk.key);
    if (tk.step < 0 || it == g_tuners.end() || size_t(tk.step) >= it->second.steps.size()) {
        g_last_info.tuned = 1;
        return;
    }
    Tuner& t = it->second;
    const size_t i = size_t(tk.step);
    if (t.steps[i].measure) t.cost[i] = wall_ms / double(iterations + 1);
    g_last_info.tuned = 0;
}

void batch_release_scene(const Scene* s) {
    std::lock_guard<std::mutex> lk(g_batch_mu);
    if (std::find(g_batch.scenes.begin(), g_batch.scenes.end(), s) != g_batch.scenes.end()) free_batch(g_batch);
}

// Begin every scene's update on its stream, run the batch graph on the
// batch's stream after all of them, end every update on its stream after it.
// rc[i]: per-scene result (apic_update_batch then waits for each scene).
int update_batch_joint(apic_handle* const* handles, uint32_t count, uint32_t flags, float frame_dt, Shape shape,
                       int* rc) {
    std::lock_guard<std::mutex> lk(g_batch_mu);
    auto fail_all = [&](int code, const std::string& msg) {
        set_last_error(("apic_update_batch: " + msg).c_str());
        for (uint32_t i = 0; i < count; ++i)
            if (rc[i] == APIC_OK) rc[i] = code;
        return code;
    };
    for (uint32_t i = 0; i < count; ++i) {
        int r = update_begin(handles[i], flags, frame_dt);
        if (r != APIC_OK) return fail_all(r, apic_last_error());
    }
    if (!same_batch(g_batch, handles, count)) {
        free_batch(g_batch);
        std::string err = build_batch(g_batch, handles, count);
        if (!err.empty()) {
            free_batch(g_batch);
            return fail_all(APIC_ERR_CUDA, "batch graph: " + err);
        }
    }
    Batch& b = g_batch;
    cudaError_t e = cudaSuccess;
    for (uint32_t i = 0; i < count && e == cudaSuccess; ++i) {
        Scene& s = *b.scenes[i];
        e = cudaEventRecord(b.ready[i], s.stream);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(b.stream, b.ready[i], 0);
    }
    if (e == cudaSuccess) {
        *b.h_bc = BCtl{};
        b.h_bc->chunk_segs = shape.chunk_segs;
        b.h_bc->block_group = shape.block_group;
        e = cudaMemcpyAsync(b.d_bc, b.h_bc, sizeof(BCtl), cudaMemcpyHostToDevice, b.stream);
    }
    if (e == cudaSuccess) e = cudaGraphLaunch(b.exec, b.stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(b.h_bc, b.d_bc, sizeof(BCtl), cudaMemcpyDeviceToHost, b.stream);
    if (e == cudaSuccess) e = cudaEventRecord(b.done, b.stream);
    for (uint32_t i = 0; i < count && e == cudaSuccess; ++i) e = cudaStreamWaitEvent(b.scenes[i]->stream, b.done, 0);
    if (e != cudaSuccess) return fail_all(APIC_ERR_CUDA, cudaGetErrorString(e));
    for (uint32_t i = 0; i < count; ++i) {
        b.scenes[i]->batched = true;
        rc[i] = update_end(handles[i]);
    }
    if ((e = cudaStreamSynchronize(b.stream)) != cudaSuccess) return fail_all(APIC_ERR_CUDA, cudaGetErrorString(e));
    g_last_info = apic_batch_info{};
    g_last_info.scenes = count;
    g_last_info.joint = 1;
    g_last_info.substep_rounds = b.h_bc->substeps;
    g_last_info.refine_rounds = b.h_bc->refine_iters;
    g_last_info.pcg_rounds = b.h_bc->pcg_iters;
    g_last_info.batch_kernel_launches = uint64_t(b.kn_top) + uint64_t(b.h_bc->substeps) * b.kn_loop +
                                        uint64_t(b.h_bc->refine_iters) * b.kn_refine +
                                        uint64_t(b.h_bc->pcg_iters) * b.kn_pcg;
    return APIC_OK;
}

}  // namespace apic

extern "C" int apic_batch_last_info(apic_batch_info* out) {
    if (!out) return APIC_ERR_INVALID_ARG;
    std::lock_guard<std::mutex> lk(apic::g_batch_mu);
    *out = apic::g_last_info;
    return APIC_OK;
}
