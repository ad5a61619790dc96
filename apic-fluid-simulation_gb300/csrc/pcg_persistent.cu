// pcg_persistent.cu — the whole pressure solve as ONE persistent cooperative kernel.
//
// Same algorithm and per-cell arithmetic as the graph form (solver.cu,
// vcycle.cu; phases in pcg_common.cuh / vcycle_common.cuh), restating
// Apic::solve_pcg (src/apic.rs:1865-1956) with its V-cycle preconditioner
// (:1788-1821).  One 1024-thread CTA per SM runs every phase of every PCG
// iteration; phases are separated by a grid barrier instead of kernel
// boundaries, so an iteration costs ~20 barriers rather than ~20 dependent
// launches.
//
// * Launched cooperatively (all CTAs co-resident).  The barrier's wait is
//   bounded: after kSpinLimit polls it raises kStatusTimeout in the control
//   block, and every CTA leaves the kernel at its next barrier.
// * Reductions are deterministic and need no broadcast barrier: each CTA
//   publishes its partial, and after the barrier every CTA sums all partials
//   in the same fixed order, so all CTAs take the same branch.  Partial slots
//   alternate so a fast CTA never overwrites a slot another CTA still reads.
// * The coarse tail's masks and coefficients are loaded into CTA 0's shared
//   memory once per solve (they do not change while it runs); per V-cycle
//   CTA 0 copies in the restricted residual and copies out the error.
// * Cells are always visited by the same warp in every base-level phase
//   (warp w owns segments w, w + nwarps, ...), so phases that read only their
//   own cells need no barrier in between.
#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include "apic_device.cuh"
#include "apic_graph.h"
#include "apic_internal.h"
#include "pcg_common.cuh"
#include "vcycle_common.cuh"

namespace apic {
using namespace vc;
namespace {

constexpr int kPThreads = 1024;
constexpr float kSafety = 1e-5f;                     // SAFTY, src/apic.rs:8
constexpr unsigned long long kSpinLimit = 1ull << 25;  // ~2 s of polling, then give up

struct SolveArgs {
    Level lv[kMaxLevels];
    int nlevels;
    int tail_first;
    TailParams tp;
    float *pressure, *search, *ap, *corr, *cg_s, *cg_ap, *cg_r;
    double *b64, *p64, *partials;
    Ctl* ctl;
    GridSync* gs;
    int mode;
    int warm;  // mixed mode starts from the previous solve's FP64 pressure
    float solve_error;
    double tol;
    uint32_t max_iter;
};

// Sense-free generation barrier over all CTAs of the grid, bounded wait.
__device__ __noinline__ bool grid_barrier(GridSync* gs, Ctl* ctl) {
    __shared__ int s_ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        volatile unsigned* vgen = &gs->gen;
        unsigned g = *vgen;
        __threadfence();
        if (atomicAdd(&gs->count, 1u) == gridDim.x - 1) {
            atomicExch(&gs->count, 0u);
            __threadfence();
            atomicAdd(&gs->gen, 1u);
        } else {
            // bounded wait; leave at once if another CTA already gave up
            volatile unsigned* vstatus = &ctl->status;
            unsigned long long spins = 0;
            while (*vgen == g) {
                if ((*vstatus & kStatusTimeout) != 0u) break;
                if (++spins > kSpinLimit) {
                    atomicOr(&ctl->status, kStatusTimeout);
                    break;
                }
                __nanosleep(64);
            }
        }
        __threadfence();
        s_ok = (atomicOr(&ctl->status, 0u) & kStatusTimeout) == 0;
    }
    __syncthreads();
    return s_ok != 0;
}

__device__ __forceinline__ double block_sum_bcast(double v) {
    __shared__ double sh[32];
    __shared__ double res;
    v = warp_sum(v);
    int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) sh[warp] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0;
        for (int w = 0; w < int(blockDim.x / 32); ++w) t += sh[w];
        res = t;
    }
    __syncthreads();
    return res;
}

__device__ __forceinline__ float block_max_bcast(float v) {
    __shared__ float sh[32];
    __shared__ float res;
    v = warp_maxf(v);
    int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) sh[warp] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        float t = 0.0f;
        for (int w = 0; w < int(blockDim.x / 32); ++w) t = fmaxf(t, sh[w]);
        res = t;
    }
    __syncthreads();
    return res;
}

struct Ctx {
    const SolveArgs& a;
    uint32_t* sm;
    const uint32_t* nseg;
    uint32_t warp, nwarps, last_fluid, pad_count;
    int slot;
    bool cluster;  // the grid is one thread-block cluster: hardware barrier
};

// Barrier over every CTA of the solve.  A single cluster uses the hardware
// cluster barrier (all its CTAs are co-scheduled, no polling; its release /
// acquire order covers global memory too); a cooperative grid uses the
// bounded software barrier.
__device__ __forceinline__ bool sync_all(Ctx& c) {
    if (c.cluster) {
        cooperative_groups::this_cluster().sync();
        return true;
    }
    return grid_barrier(c.a.gs, c.a.ctl);
}

// Deterministic grid-wide sum (includes one barrier).
__device__ __forceinline__ bool grid_sum(Ctx& c, double v, double& out) {
    double b = block_sum_bcast(v);
    double* part = c.a.partials + size_t(c.slot) * gridDim.x;
    if (threadIdx.x == 0) part[blockIdx.x] = b;
    if (!sync_all(c)) return false;
    double t = threadIdx.x < gridDim.x ? __ldcg(part + threadIdx.x) : 0.0;
    out = block_sum_bcast(t);
    c.slot ^= 1;
    return true;
}
// Double-float per-thread sums (the phases' dot products) enter as doubles.
__device__ __forceinline__ bool grid_sum(Ctx& c, F2 v, double& out) { return grid_sum(c, f2_value(v), out); }

__device__ __forceinline__ bool grid_max(Ctx& c, float v, float& out) {
    float b = block_max_bcast(v);
    double* part = c.a.partials + size_t(c.slot) * gridDim.x;
    if (threadIdx.x == 0) part[blockIdx.x] = double(b);
    if (!sync_all(c)) return false;
    float t = threadIdx.x < gridDim.x ? float(__ldcg(part + threadIdx.x)) : 0.0f;
    out = block_max_bcast(t);
    c.slot ^= 1;
    return true;
}

#define SYNC_OR_FAIL() \
    if (!sync_all(c)) return false

// One V-cycle (apply_preconditioner, src/apic.rs:1788-1821); z in lv[0].err.
// The last phase writes only base cells that the caller's own-cell phases read.
__device__ bool vcycle(Ctx& c) {
    const Level* L = c.a.lv;
    const int last = c.a.nlevels - 1;
    ph_smooth(L[0], c.nseg[0], c.warp, c.nwarps, 0, 1);
    SYNC_OR_FAIL();
    ph_smooth(L[0], c.nseg[0], c.warp, c.nwarps, 1, 1);
    SYNC_OR_FAIL();
    if (last < 1) {
        ph_smooth(L[0], c.nseg[0], c.warp, c.nwarps, 1, 0);
        SYNC_OR_FAIL();
        ph_smooth(L[0], c.nseg[0], c.warp, c.nwarps, 0, 0);
        return true;
    }
    int deepest_mid = 0;
    for (int l = 1; l <= last; ++l) {
        if (l == c.a.tail_first) {
            ph_restrict(L[l - 1], L[l], c.nseg[l], c.warp, c.nwarps, false);
            SYNC_OR_FAIL();
            if (blockIdx.x == 0) cta_tail(c.a.tp, c.sm, false);
            SYNC_OR_FAIL();
            break;
        }
        if (l == last) {
            ph_restrict(L[l - 1], L[l], c.nseg[l], c.warp, c.nwarps, false);
            SYNC_OR_FAIL();
            if (blockIdx.x == 0)
                cta_coarse_cg(L[l].fluid, L[l].w, L[l].cells, L[l].diag, L[l].px, L[l].py, L[l].res, L[l].err,
                              c.a.cg_s, c.a.cg_ap, c.a.cg_r);
            SYNC_OR_FAIL();
            break;
        }
        ph_restrict(L[l - 1], L[l], c.nseg[l], c.warp, c.nwarps, true);
        SYNC_OR_FAIL();
        ph_smooth(L[l], c.nseg[l], c.warp, c.nwarps, 1, 1);
        SYNC_OR_FAIL();
        deepest_mid = l;
    }
    for (int l = deepest_mid; l >= 1; --l) {
        ph_prolong(L[l + 1], L[l], c.nseg[l], c.warp, c.nwarps, 1, 0xFFFFFFFFu, 0u);
        SYNC_OR_FAIL();
        ph_prolong(L[l + 1], L[l], c.nseg[l], c.warp, c.nwarps, 0, 0xFFFFFFFFu, 0u);
        SYNC_OR_FAIL();
    }
    ph_prolong(L[1], L[0], c.nseg[0], c.warp, c.nwarps, 1, c.last_fluid, c.pad_count);
    SYNC_OR_FAIL();
    ph_prolong(L[1], L[0], c.nseg[0], c.warp, c.nwarps, 0, c.last_fluid, c.pad_count);
    return true;
}

struct LoopOut {
    uint32_t iters = 0;
    bool converged = false;
    float max_r = 0.0f;
    double rn2 = 0.0;
};

// PCG (src/apic.rs:1885-1955) into x.  Reference exits in APIC_SOLVER_REFERENCE,
// otherwise ||r|| <= target_rel * sqrt(bnorm2).
__device__ bool pcg_loop(Ctx& c, int mode, float* x, int x_padded, uint32_t cap, double target_rel, double bnorm2,
                         LoopOut& out) {
    const Level& B = c.a.lv[0];
    const uint32_t n0 = c.nseg[0];
    const bool ref = mode == APIC_SOLVER_REFERENCE;
    if (!vcycle(c)) return false;
    double g64;
    if (!grid_sum(c, pcg::ph_start(B, n0, c.warp, c.nwarps, c.a.search), g64)) return false;
    float gamma = float(g64);
    if (ref ? gamma < kSafety : !(gamma != 0.0f)) {
        out.converged = true;
        return true;
    }
    while (out.iters < cap) {
        double d64;
        if (!grid_sum(c, pcg::ph_spmv(B, n0, c.warp, c.nwarps, c.a.search, c.a.ap), d64)) return false;
        float delta = float(d64);
        out.iters++;
        if (ref ? fabsf(delta) < kSafety : (!(delta != 0.0f) || !isfinite(delta))) {
            out.converged = true;
            break;
        }
        float alpha = gamma / delta;
        float mx;
        F2 r2;
        pcg::ph_update(B, n0, c.warp, c.nwarps, alpha, x, x_padded, c.a.search, c.a.ap, &mx, &r2);
        if (ref) {
            float m;
            if (!grid_max(c, mx, m)) return false;
            out.max_r = m;
            if (m < c.a.solve_error) {
                out.converged = true;
                break;
            }
        } else {
            double t;
            if (!grid_sum(c, r2, t)) return false;
            out.rn2 = t;
            if ((bnorm2 > 0.0 ? sqrt(t / bnorm2) : 0.0) <= target_rel) {
                out.converged = true;
                break;
            }
        }
        if (!vcycle(c)) return false;
        double n64;
        if (!grid_sum(c, pcg::ph_rz(B, n0, c.warp, c.nwarps), n64)) return false;
        float ng = float(n64);
        if (ref ? ng < kSafety : !(ng != 0.0f)) {
            out.converged = true;
            break;
        }
        float beta = ng / gamma;
        gamma = ng;
        pcg::ph_search(B, n0, c.warp, c.nwarps, beta, c.a.search);
        SYNC_OR_FAIL();
    }
    return true;
}

__device__ bool solve(Ctx& c) {
    const SolveArgs& a = c.a;
    const Level& B = a.lv[0];
    const uint32_t n0 = c.nseg[0];
    Ctl* ctl = a.ctl;
    const bool lead = blockIdx.x == 0 && threadIdx.x == 0;
    if (a.mode == APIC_SOLVER_REFERENCE) {
        pcg::ph_clear_pressure(B, n0, c.warp, c.nwarps, a.pressure);
        LoopOut o;
        if (!pcg_loop(c, a.mode, a.pressure, 0, 100, 0.0, 0.0, o)) return false;
        if (lead) {
            ctl->pcg_iters = o.iters;
            ctl->pcg_iters_total += o.iters;
            ctl->max_r_bits = __float_as_uint(o.max_r);
            if (!o.converged) ctl->not_converged++;
        }
        return true;
    }
    double bnorm2;
    if (!grid_sum(c, pcg::ph_mixed_init(B, n0, c.warp, c.nwarps, a.b64, a.p64, a.warm), bnorm2)) return false;
    pcg::ph_clear_pressure(B, n0, c.warp, c.nwarps, a.pressure);
    if (a.mode == APIC_SOLVER_REL_FP32) {
        LoopOut o;
        if (!pcg_loop(c, a.mode, a.pressure, 0, a.max_iter, a.tol, bnorm2, o)) return false;
        pcg::ph_pressure_to64(B, n0, c.warp, c.nwarps, a.pressure, a.p64);
        SYNC_OR_FAIL();
        double rr;
        if (!grid_sum(c, pcg::ph_true_residual(B, n0, c.warp, c.nwarps, a.b64, a.p64, a.corr, 1), rr)) return false;
        if (lead) {
            ctl->pcg_iters = o.iters;
            ctl->pcg_iters_total += o.iters;
            ctl->rnorm2 = o.rn2;
            ctl->bnorm2 = bnorm2;
            ctl->true_rel = bnorm2 > 0.0 ? sqrt(rr / bnorm2) : 0.0;
            if (!o.converged) ctl->not_converged++;
        }
        return true;
    }
    // APIC_SOLVER_REL_MIXED: FP64 iterative refinement around FP32 inner PCG.
    double rr;
    if (!grid_sum(c, pcg::ph_true_residual(B, n0, c.warp, c.nwarps, a.b64, a.p64, a.corr, 3), rr)) return false;
    double tr = bnorm2 > 0.0 ? sqrt(rr / bnorm2) : 0.0;
    uint32_t used = 0, refinements = 0, last_iters = 1;
    double rn2 = 0.0;
    while (tr > a.tol && used < a.max_iter && refinements < 32u && !(refinements > 0u && last_iters == 0u)) {
        refinements++;
        double target = 1e-4 * tr;
        if (target < 0.5 * a.tol) target = 0.5 * a.tol;
        LoopOut o;
        if (!pcg_loop(c, APIC_SOLVER_REL_FP32, a.corr, 1, a.max_iter - used, target, bnorm2, o)) return false;
        used += o.iters;
        last_iters = o.iters;
        rn2 = o.rn2;
        pcg::ph_accumulate(B, n0, c.warp, c.nwarps, a.p64, a.corr, a.pressure, 0);
        SYNC_OR_FAIL();
        if (!grid_sum(c, pcg::ph_true_residual(B, n0, c.warp, c.nwarps, a.b64, a.p64, a.corr, 3), rr)) return false;
        tr = bnorm2 > 0.0 ? sqrt(rr / bnorm2) : 0.0;
    }
    pcg::ph_accumulate(B, n0, c.warp, c.nwarps, a.p64, a.corr, a.pressure, 1);
    if (lead) {
        ctl->pcg_iters = used;
        ctl->pcg_iters_total += used;
        ctl->refinements = refinements;
        ctl->refinements_total += refinements;
        ctl->rnorm2 = rn2;
        ctl->bnorm2 = bnorm2;
        ctl->true_rel = tr;
        if (tr > a.tol) ctl->not_converged++;
    }
    return true;
}

#undef SYNC_OR_FAIL

__global__ void __launch_bounds__(kPThreads, 1) k_solve_persistent(SolveArgs a, int cluster) {
    extern __shared__ uint32_t sm[];
    __shared__ uint32_t nseg[kMaxLevels];
    __shared__ uint32_t s_last, s_pad;
    if (threadIdx.x < uint32_t(a.nlevels)) nseg[threadIdx.x] = a.ctl->seg_count[threadIdx.x];
    if (threadIdx.x == 0) {
        s_last = a.ctl->last_fluid;
        s_pad = a.ctl->pad_count;
    }
    if (blockIdx.x == 0 && a.tail_first < a.nlevels) cta_tail_load_coeffs(a.tp, sm);
    __syncthreads();
    Ctx c{a, sm, nseg, (blockIdx.x * blockDim.x + threadIdx.x) >> 5, (gridDim.x * blockDim.x) >> 5, s_last, s_pad, 0,
          cluster != 0};
    solve(c);
    if (blockIdx.x == 0 && threadIdx.x == 0) a.ctl->pcg_done = 1;
}

}  // namespace

// Grid of the persistent solve: one CTA per SM (0 when a cooperative launch
// of this shape is impossible on the device).
void plan_persistent_solve(Scene& s) {
    s.persist_grid = 0;
    int dev = 0, sms = 0, coop = 0, per_sm = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev);
    if (!coop || sms <= 0) return;
    size_t smem = s.tail_first < s.nlevels ? s.tail_smem : 0;
    // a per-function limit shared by every scene of the process: the largest
    // tail any scene may use, not this scene's
    cudaFuncSetAttribute(k_solve_persistent, cudaFuncAttributeMaxDynamicSharedMemorySize, int(kTailSmemBudget));
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_solve_persistent, kPThreads, smem) != cudaSuccess ||
        per_sm < 1) {
        cudaGetLastError();
        return;
    }
    int grid = sms;  // one CTA per SM
    if (grid > kPThreads || grid > kMaxRedBlocks) grid = kPThreads < kMaxRedBlocks ? kPThreads : kMaxRedBlocks;
    s.persist_grid = grid;
    s.persist_smem = smem;
}

// The whole solve in one thread-block cluster, for scenes small enough that
// 1..16 CTAs cover a base-level phase in about one pass: CTAs = base cells /
// 4096 rounded up to a power of two.  0 when the scene is larger than
// cluster_solve_cells or the GPU cannot hold such a cluster.
void plan_cluster_solve(Scene& s) {
    s.cluster_solve_ctas = 0;
    if (s.cluster_solve_cells == 0 || s.cells > s.cluster_solve_cells || s.nlevels < 2) return;
    int ctas = 1;
    while (ctas < 16 && uint64_t(ctas) * 4096 < s.cells) ctas *= 2;
    size_t smem = s.tail_first < s.nlevels ? s.tail_smem : 0;
    cudaFuncSetAttribute(k_solve_persistent, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
    cudaFuncSetAttribute(k_solve_persistent, cudaFuncAttributeMaxDynamicSharedMemorySize, int(kTailSmemBudget));
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(ctas);
    cfg.blockDim = dim3(kPThreads);
    cfg.dynamicSmemBytes = smem;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = unsigned(ctas);
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    int clusters = 0;
    const bool ok = cudaOccupancyMaxActiveClusters(&clusters, k_solve_persistent, &cfg) == cudaSuccess && clusters > 0;
    cudaGetLastError();
    if (ok) s.cluster_solve_ctas = ctas;
}

static SolveArgs solve_args(Scene& s, uint32_t* words) {
    SolveArgs a;
    for (int l = 0; l < kMaxLevels; ++l) a.lv[l] = s.lv[l];
    a.nlevels = s.nlevels;
    a.tail_first = s.tail_first;
    *words = 0;
    if (s.tail_first < s.nlevels) a.tp = make_tail_params(s, s.tail_first, words);
    else a.tp.n = 0;
    a.pressure = s.pressure; a.search = s.search; a.ap = s.ap; a.corr = s.corr;
    a.cg_s = s.cg_s; a.cg_ap = s.cg_ap; a.cg_r = s.cg_r;
    a.b64 = s.b64; a.p64 = s.p64; a.partials = s.partials;
    a.ctl = s.ctl;
    a.gs = s.gsync;
    a.mode = s.solver_mode;
    a.warm = warm_start(s);
    a.solve_error = s.props.solve_error;
    a.tol = double(s.rel_tol);
    a.max_iter = s.max_iter;
    return a;
}

// Enqueue the whole solve on s.stream as one cluster launch.
cudaError_t enqueue_cluster_solve(Scene& s) {
    uint32_t words = 0;
    SolveArgs a = solve_args(s, &words);
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(s.cluster_solve_ctas);
    cfg.blockDim = dim3(kPThreads);
    cfg.dynamicSmemBytes = size_t(words) * 4;
    cfg.stream = s.stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = unsigned(s.cluster_solve_ctas);
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    s.p64_valid = s.solver_mode == APIC_SOLVER_REL_MIXED;
    return cudaLaunchKernelEx(&cfg, k_solve_persistent, a, 1);
}

// Enqueue the whole solve on s.stream: reset the barrier, launch cooperatively.
cudaError_t enqueue_persistent_solve(Scene& s) {
    SolveArgs a;
    for (int l = 0; l < kMaxLevels; ++l) a.lv[l] = s.lv[l];
    a.nlevels = s.nlevels;
    a.tail_first = s.tail_first;
    uint32_t words = 0;
    if (s.tail_first < s.nlevels) a.tp = make_tail_params(s, s.tail_first, &words);
    else a.tp.n = 0;
    a.pressure = s.pressure; a.search = s.search; a.ap = s.ap; a.corr = s.corr;
    a.cg_s = s.cg_s; a.cg_ap = s.cg_ap; a.cg_r = s.cg_r;
    a.b64 = s.b64; a.p64 = s.p64; a.partials = s.partials;
    a.ctl = s.ctl;
    a.gs = s.gsync;
    a.mode = s.solver_mode;
    a.warm = warm_start(s);
    a.solve_error = s.props.solve_error;
    a.tol = double(s.rel_tol);
    a.max_iter = s.max_iter;
    cudaError_t e = cudaMemsetAsync(s.gsync, 0, sizeof(GridSync), s.stream);
    if (e != cudaSuccess) return e;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(s.persist_grid);
    cfg.blockDim = dim3(kPThreads);
    cfg.dynamicSmemBytes = size_t(words) * 4;
    cfg.stream = s.stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    s.p64_valid = s.solver_mode == APIC_SOLVER_REL_MIXED;
    return cudaLaunchKernelEx(&cfg, k_solve_persistent, a, 0);
}

}  // namespace apic
