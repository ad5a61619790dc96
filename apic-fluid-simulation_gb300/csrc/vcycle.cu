// vcycle.cu — the multigrid V-cycle preconditioner (z = M^-1 r).
//
// Restates Apic::apply_preconditioner (src/apic.rs:1788-1821) and the
// MultiGridLevel methods it calls: red/black SOR with omega = 1.2 and one
// sweep each way (smooth_level, :471-535), restriction of r - A e over the 2x2
// children of each coarse fluid cell (restrict, :537-594), piecewise-constant
// prolongation (prolongate, :596-616) and plain CG on the coarsest level
// (solve_coarse_exact, :618-704).
//
// Launch structure (one CUDA-graph node each), chosen to cut dependent
// launches per PCG iteration while keeping the reference's arithmetic:
//   * the first red sweep after a level's error was zero-filled needs only the
//     level's residual, so it is fused with the restriction that produces
//     that residual (k_restrict_red);
//   * prolongation only adds the coarse error before the reverse sweep, so it
//     is fused into both sweeps: the black sweep reads "error + coarse error"
//     of its red neighbours on the fly, the red sweep then adds its own
//     (k_prolong_black / k_prolong_red) — the same float operations in the
//     same order as the reference, with no cell written twice in one launch;
//   * all levels that fit in shared memory (the coarse tail, including the
//     coarsest CG) run in ONE cooperative CTA: coefficients are loaded from L2
//     once per V-cycle and every sweep is a __syncthreads()-separated phase
//     (k_vcycle_tail);
//   * the middle levels above the tail (a few thousand to some tens of
//     thousands of fluid cells: too small to fill the GPU, so each of their
//     launches costs mostly its latency) live in the distributed shared
//     memory of one thread-block cluster together with the tail
//     (k_vcycle_dsm, vcycle_dsm.cu).
// On the base level the last fluid cell receives the coarse correction once
// more per duplicate that pads the reference's fluid list to a multiple of 8
// (:1487-1494, iterated by prolongate :611-615).
#include <cuda_runtime.h>

#include "apic_device.cuh"
#include "apic_internal.h"
#include "batch.h"
#include "pcg_common.cuh"
#include "vcycle_common.cuh"

namespace apic {
using namespace vc;
namespace {

__device__ __forceinline__ uint32_t gwarp() { return (blockIdx.x * blockDim.x + threadIdx.x) >> 5; }
__device__ __forceinline__ uint32_t gnwarps() { return (gridDim.x * blockDim.x) >> 5; }

// Segment lists and their lengths are written by the multigrid setup, never
// by the kernel just before: each warp loads its first segment word before
// waiting on that kernel (programmatic dependent launch).
__device__ __forceinline__ uint32_t early_word(const uint32_t* seg, uint32_t nseg) {
    const uint32_t s = gwarp();
    return s < nseg ? seg[s] : kNoWord;
}

// The base level's black sweep after k_pcg_update (which ran the red one),
// with the exit test of k_pcg_update's residual and the PCG loop's decision
// in an extra block 0 that runs beside the sweep; later kernels see its
// verdict.
__global__ void __launch_bounds__(kSegBlock) k_smooth_exit(Level L, Ctl* ctl, const float4* part, uint32_t nparts,
                                                           int mode, float solve_error, cudaGraphConditionalHandle h,
                                                           uint32_t cap, int dyn_cap, int set_cond) {
    const uint32_t nseg = ctl->seg_count[0];
    if (blockIdx.x == 0) {
        pdl_wait();
        if (!ctl->pcg_done) pcg::residual_exit(ctl, part, nparts, mode, solve_error);
        if (threadIdx.x == 0) pcg::loop_decision(ctl, mode, h, cap, dyn_cap, set_cond);
        return;
    }
    const uint32_t warp = gwarp() - kSegWarps, nwarps = gnwarps() - kSegWarps;
    const uint32_t w0 = warp < nseg ? L.seg[warp] : kNoWord;
    pdl_wait();
    if (ctl->pcg_done) return;
    ph_smooth(L, nseg, warp, nwarps, 1, 1, w0);
}

__global__ void __launch_bounds__(kSegBlock) k_smooth(Level L, int li, const Ctl* ctl, int color, int init) {
    const uint32_t nseg = ctl->seg_count[li];
    const uint32_t w0 = early_word(L.seg, nseg);
    pdl_wait();
    if (ctl->pcg_done) return;
    ph_smooth(L, nseg, gwarp(), gnwarps(), color, init, w0);
}

// Restriction only (into the first tail level or the coarsest level).
// The transfer kernels come in two register budgets: kMinB 8 (32 registers,
// eight CTAs per SM, a few spilled values) for levels of more than 2 M cells,
// whose launches are bandwidth and occupancy bound (4096^2: 895 vs 983 us per
// PCG iteration), and the unbounded form for the smaller, latency-bound ones.
template <int kMinB>
__global__ void __launch_bounds__(kSegBlock, kMinB) k_restrict(Level f, Level c, int lc, const Ctl* ctl) {
    const uint32_t nseg = ctl->seg_count[lc];
    const uint32_t w0 = early_word(c.seg, nseg);
    pdl_wait();
    if (ctl->pcg_done) return;
    ph_restrict(f, c, nseg, gwarp(), gnwarps(), false, w0);
}

// Restriction fused with the coarse level's first (red) sweep.
template <int kMinB>
__global__ void __launch_bounds__(kSegBlock, kMinB) k_restrict_red(Level f, Level c, int lc, const Ctl* ctl) {
    const uint32_t nseg = ctl->seg_count[lc];
    const uint32_t w0 = early_word(c.seg, nseg);
    pdl_wait();
    if (ctl->pcg_done) return;
    ph_restrict(f, c, nseg, gwarp(), gnwarps(), true, w0);
}

// Prolongation fused with the black sweep.
template <int kMinB>
__global__ void __launch_bounds__(kSegBlock, kMinB) k_prolong_black(Level c, Level f, int lf, const Ctl* ctl, int base) {
    const uint32_t nseg = ctl->seg_count[lf];
    const uint32_t w0 = early_word(f.seg, nseg);
    const uint32_t last = base ? ctl->last_fluid : 0xFFFFFFFFu, extra = base ? ctl->pad_count : 0u;
    pdl_wait();
    if (ctl->pcg_done) return;
    ph_prolong(c, f, nseg, gwarp(), gnwarps(), 1, last, extra, w0);
}

// Base-level prolongation fused with the final red sweep, which also stores
// this block's part of r.z over every fluid cell (red cells' new z, black
// cells' final z): k_dot_rz's work; the next iteration sums the parts.
__global__ void __launch_bounds__(kSegBlock) k_prolong_red_rz(Level c, Level B, const Ctl* ctl, float2* part) {
    const uint32_t nseg = ctl->seg_count[0];
    const uint32_t w0 = early_word(B.seg, nseg);
    const uint32_t last = ctl->last_fluid, extra = ctl->pad_count;
    pdl_wait();
    if (ctl->pcg_done) return;
    const F2 acc = ph_prolong_red_rz(c, B, nseg, gwarp(), gnwarps(), last, extra, w0);
    block_store<kSegBlock>(hw_blk(), acc, part);
}

// Prolongation fused with the final red sweep (black neighbours are final).
__global__ void __launch_bounds__(kSegBlock) k_prolong_red(Level c, Level f, int lf, const Ctl* ctl, int base) {
    const uint32_t nseg = ctl->seg_count[lf];
    const uint32_t w0 = early_word(f.seg, nseg);
    const uint32_t last = base ? ctl->last_fluid : 0xFFFFFFFFu, extra = base ? ctl->pad_count : 0u;
    pdl_wait();
    if (ctl->pcg_done) return;
    ph_prolong(c, f, nseg, gwarp(), gnwarps(), 0, last, extra, w0);
}

__global__ void __launch_bounds__(kTailThreads) k_coarse_solve(Level L, float* __restrict__ cs, float* __restrict__ cap,
                                                               float* __restrict__ cr, const Ctl* __restrict__ ctl,
                                                               int exact) {
    pdl_wait();
    if (ctl->pcg_done) return;
    cta_coarse_cg(L.fluid, L.w, L.cells, L.diag, L.px, L.py, L.res, L.err, cs, cap, cr, exact != 0);
}

__global__ void __launch_bounds__(kTailThreads) k_vcycle_tail(TailParams tp, const Ctl* ctl) {
    pdl_wait();
    if (ctl->pcg_done) return;
    extern __shared__ uint32_t sm[];
    cta_tail(tp, sm, true);
}

size_t tail_level_bytes(const Level& L) { return 4ull * (L.words + 6ull * L.padded); }

// ---- the V-cycle's phases over a batch of scenes (batch.h) ------------------
// Persistent CTAs walk the listed items of their gate; each runs the
// single-scene kernel's work for one block of its scene's own launch.  The
// prolongations run at eight CTAs per SM (32 registers, a few spilled): an
// item is a chain of dependent loads, and more of them in flight beat the
// spills (config 4: 17% per batched update with the reductions of
// solver.cu bounded alike).

// k_smooth_exit: item 0 of each scene takes the scene's exit test and loop
// decision (k_bat_pcg_next then lists the scenes that go on); the others
// are chunks of the base level's black sweep.
__global__ void __launch_bounds__(kSegBlock) k_bat_smooth_exit(const BScene* __restrict__ tab, BListRef L) {
    bat_for_items(L, kKindExit, true, [&](uint32_t sc, uint32_t lb, Shape sh) {
        const BScene& S = tab[sc];
        Ctl* ctl = S.ctl;
        if (!bat_gate(ctl, kGatePcg)) return;
        if (lb == 0) {  // the residual's parts: those of the blocks k_bat_pcg_update ran
            if (!ctl->pcg_done) pcg::residual_exit(ctl, bs_part_res(S), busy_blocks(S), APIC_SOLVER_REL_FP32, 0.0f);
            if (threadIdx.x == 0) ctl->pcg_on = pcg::loop_continue(ctl, APIC_SOLVER_REL_FP32, 0u, 1) ? 1u : 0u;
            return;
        }
        if (ctl->pcg_done) return;
        const Chunk ch = chunk_of(lb - 1, ctl->seg_count[0], sh);
        ph_smooth(S.lv[0], ch.end, ch.warp, ch.nwarps, 1, 1, kNoWord);
    });
}

__global__ void __launch_bounds__(kSegBlock) k_bat_smooth(const BScene* __restrict__ tab, BListRef L, int li,
                                                          int gate, int color, int init) {
    bat_for_items(L, kind_chunk(li), gate == kGatePcg, [&](uint32_t sc, uint32_t lb, Shape sh) {
        const BScene& S = tab[sc];
        const Ctl* ctl = S.ctl;
        if (!bat_gate(ctl, gate) || ctl->pcg_done) return;
        const Chunk ch = chunk_of(lb, ctl->seg_count[li], sh);
        ph_smooth(S.lv[li], ch.end, ch.warp, ch.nwarps, color, init, kNoWord);
    });
}

// Restriction into level lc: fused with the level's first red sweep when the
// level is smoothed by the segment kernels, plain into the first tail level.
__global__ void __launch_bounds__(kSegBlock) k_bat_restrict(const BScene* __restrict__ tab, BListRef L, int lc,
                                                            int gate) {
    bat_for_items(L, kind_rchunk(lc), gate == kGatePcg, [&](uint32_t sc, uint32_t lb, Shape sh) {
        const BScene& S = tab[sc];
        const Ctl* ctl = S.ctl;
        if (!bat_gate(ctl, gate) || ctl->pcg_done) return;
        const Chunk ch = chunk_of(lb, ctl->seg_count[lc], sh);
        ph_restrict(S.lv[lc - 1], S.lv[lc], ch.end, ch.warp, ch.nwarps, uint32_t(lc) < S.tail_first, kNoWord);
    });
}

// Prolongation from level lf + 1 fused with level lf's black (color 1) or
// red (color 0) sweep; base: lf is the base level.
__global__ void __launch_bounds__(kSegBlock, 8) k_bat_prolong(const BScene* __restrict__ tab, BListRef L, int lf,
                                                           int gate, int color, int base) {
    bat_for_items(L, kind_chunk(lf), gate == kGatePcg, [&](uint32_t sc, uint32_t lb, Shape sh) {
        const BScene& S = tab[sc];
        const Ctl* ctl = S.ctl;
        if (!bat_gate(ctl, gate) || ctl->pcg_done) return;
        const uint32_t last = base ? ctl->last_fluid : 0xFFFFFFFFu, extra = base ? ctl->pad_count : 0u;
        const Chunk ch = chunk_of(lb, ctl->seg_count[lf], sh);
        ph_prolong(S.lv[lf + 1], S.lv[lf], ch.end, ch.warp, ch.nwarps, color, last, extra, kNoWord);
    });
}

// The iteration's last V-cycle kernel (k_prolong_red_rz).
__global__ void __launch_bounds__(kSegBlock, 8) k_bat_prolong_red_rz(const BScene* __restrict__ tab, BListRef L) {
    bat_for_items(L, kKindBlocks, true, [&](uint32_t sc, uint32_t item, Shape sh) {
        const BScene& S = tab[sc];
        const Ctl* ctl = S.ctl;
        if (!bat_gate(ctl, kGatePcg) || ctl->pcg_done) return;
        const uint32_t nseg = ctl->seg_count[0], end = group_end(S, item, sh);
        const uint32_t last = ctl->last_fluid, extra = ctl->pad_count;
        for (uint32_t b = item * sh.block_group; b < end; ++b) {
            const Blk bk{b, S.grid[0]};
            const F2 acc = ph_prolong_red_rz(S.lv[1], S.lv[0], nseg, blk_warp(bk), blk_nwarps(bk), last, extra,
                                             kNoWord);
            block_store<kSegBlock>(bk, acc, bs_part_rz(S));
            __syncthreads();  // block_store's shared slots are reused by the next block
        }
    });
}

// The coarse tail (k_vcycle_tail): persistent CTAs take the listed scenes one
// at a time; the scene's tail parameters are copied into shared memory beside
// the levels.
__global__ void __launch_bounds__(kTailThreads) k_bat_tail(const BScene* __restrict__ tab, BListRef L, int gate) {
    __shared__ TailParams s_tp;
    extern __shared__ uint32_t sm[];
    pdl_wait();
    const uint32_t nact = L.p[0];
    for (uint32_t j = blockIdx.x; j < nact; j += gridDim.x) {
        const BScene& S = tab[L.scenes()[j]];
        if (!bat_gate(S.ctl, gate) || S.ctl->pcg_done) continue;
        const uint32_t* src = reinterpret_cast<const uint32_t*>(&S.tp);
        uint32_t* dst = reinterpret_cast<uint32_t*>(&s_tp);
        for (uint32_t i = threadIdx.x; i < sizeof(TailParams) / 4; i += blockDim.x) dst[i] = src[i];
        __syncthreads();
        cta_tail(s_tp, sm, true);
        __syncthreads();
    }
}

}  // namespace

void bat_smooth_exit(const BatchRun& r) {
    static const uint32_t g = persistent_grid(k_bat_smooth_exit, kSegBlock, 0);
    launch(r.pdl, k_bat_smooth_exit, g, kSegBlock, 0, r.st, r.tab, r.list[kGatePcg]);
}
void bat_smooth(const BatchRun& r, int l, int gate, int color, int init) {
    static const uint32_t g = persistent_grid(k_bat_smooth, kSegBlock, 0);
    launch(r.pdl, k_bat_smooth, g, kSegBlock, 0, r.st, r.tab, r.list[gate], l, gate, color, init);
}
void bat_restrict(const BatchRun& r, int l, int gate) {
    static const uint32_t g = persistent_grid(k_bat_restrict, kSegBlock, 0);
    launch(r.pdl, k_bat_restrict, g, kSegBlock, 0, r.st, r.tab, r.list[gate], l, gate);
}
void bat_prolong_black(const BatchRun& r, int l, int gate, int base) {
    static const uint32_t g = persistent_grid(k_bat_prolong, kSegBlock, 0);
    launch(r.pdl, k_bat_prolong, g, kSegBlock, 0, r.st, r.tab, r.list[gate], l, gate, 1, base);
}
void bat_prolong_red(const BatchRun& r, int l, int gate, int base) {
    static const uint32_t g = persistent_grid(k_bat_prolong, kSegBlock, 0);
    launch(r.pdl, k_bat_prolong, g, kSegBlock, 0, r.st, r.tab, r.list[gate], l, gate, 0, base);
}
void bat_prolong_red_rz(const BatchRun& r) {
    static const uint32_t g = persistent_grid(k_bat_prolong_red_rz, kSegBlock, 0);
    launch(r.pdl, k_bat_prolong_red_rz, g, kSegBlock, 0, r.st, r.tab, r.list[kGatePcg]);
}
void bat_tail(const BatchRun& r, int gate) {
    const uint32_t g = r.nscenes < 152u ? r.nscenes : 152u;  // one CTA per SM holds the largest tail
    launch(r.pdl, k_bat_tail, g, kTailThreads, r.tail_smem, r.st, r.tab, r.list[gate], gate);
}
void bat_prepare_tail() {
    cudaFuncSetAttribute(k_bat_tail, cudaFuncAttributeMaxDynamicSharedMemorySize, int(kTailSmemBudget));
}

// Choose the coarse levels that run in one CTA (all of them fit in shared memory).
void plan_vcycle(Scene& s) {
    s.tail_first = s.nlevels;  // none
    s.tail_smem = 0;
    if (s.nlevels < 2) return;
    const Level& C = s.lv[s.nlevels - 1];
    size_t bytes = 3ull * 4 * C.padded;  // coarse CG vectors
    for (int l = s.nlevels - 1; l >= 1; --l) {
        size_t b = bytes + tail_level_bytes(s.lv[l]);
        if (b > kTailSmemBudget) break;
        bytes = b;
        s.tail_first = l;
    }
    if (s.tail_first < s.nlevels) {
        s.tail_smem = bytes;
        cudaFuncSetAttribute(k_vcycle_tail, cudaFuncAttributeMaxDynamicSharedMemorySize, int(kTailSmemBudget));
    }
    plan_vcycle_dsm(s);
}

// One V-cycle on s.stream: z = M^-1 r in lv[0].err.  Two kernels per sweep and
// per transfer on the levels above the distributed-shared-memory cluster or
// the tail (the reference's sequence launch by launch).  Returns false when
// the caller must reduce r.z itself (a grid without multigrid levels).
constexpr uint32_t kBigLevelWords = 65536;  // 2 M cells
bool enqueue_vcycle(Scene& s, bool base_red_done, int rz_mode, bool residual_exit) {
    cudaStream_t st = s.stream;
    Level* L = s.lv;
    auto grid = [&](int l) { return seg_grid(L[l].words); };
    const int last = s.nlevels - 1;
    const bool pdl = s.use_pdl;
    if (!base_red_done) launch(pdl, k_smooth, grid(0), kSegBlock, 0, st, L[0], 0, s.ctl, 0, 1);
    if (residual_exit && base_red_done)
        launch(pdl, k_smooth_exit, grid(0) + 1, kSegBlock, 0, st, L[0], s.ctl,
               static_cast<const float4*>(part_res(s)), grid(0), rz_mode, s.props.solve_error, s.pcg_h, s.pcg_cap,
               s.pcg_dyn_cap, s.pcg_set_cond ? 1 : 0);
    else
        launch(pdl, k_smooth, grid(0), kSegBlock, 0, st, L[0], 0, s.ctl, 1, 1);
    if (last < 1) {
        launch(pdl, k_smooth, grid(0), kSegBlock, 0, st, L[0], 0, s.ctl, 1, 0);
        launch(pdl, k_smooth, grid(0), kSegBlock, 0, st, L[0], 0, s.ctl, 0, 0);
        return rz_mode < 0;
    }
    const bool dsm = s.use_dsm && s.dsm_first < s.dsm_tail && s.dsm_tail < s.nlevels;
    int deepest_mid = 0;  // deepest level smoothed by the global kernels
    auto big = [&](int l) { return L[l].words > kBigLevelWords; };
    auto restrict_red = [&](int l) {
        launch(pdl, big(l) ? k_restrict_red<8> : k_restrict_red<1>, grid(l), kSegBlock, 0, st, L[l - 1], L[l], l,
               s.ctl);
    };
    auto restrict_plain = [&](int l) {
        launch(pdl, big(l) ? k_restrict<8> : k_restrict<1>, grid(l), kSegBlock, 0, st, L[l - 1], L[l], l, s.ctl);
    };
    auto prolong_black = [&](int l, int base) {
        launch(pdl, big(l) ? k_prolong_black<8> : k_prolong_black<1>, grid(l), kSegBlock, 0, st, L[l + 1], L[l], l,
               s.ctl, base);
    };
    for (int l = 1; l <= last; ++l) {
        if (dsm && l == s.dsm_first) {
            restrict_red(l);
            launch_vcycle_dsm(s, st);
            break;
        }
        if (l == s.tail_first) {
            restrict_plain(l);
            uint32_t off = 0;
            TailParams tp = make_tail_params(s, l, &off);
            launch(pdl, k_vcycle_tail, 1, kTailThreads, size_t(off) * 4, st, tp, s.ctl);
            break;
        }
        if (l == last) {
            restrict_plain(l);
            launch(pdl, k_coarse_solve, 1, kTailThreads, 0, st, L[l], s.cg_s, s.cg_ap, s.cg_r, s.ctl,
                   coarse_cg_exact(s) ? 1 : 0);
            break;
        }
        restrict_red(l);
        launch(pdl, k_smooth, grid(l), kSegBlock, 0, st, L[l], l, s.ctl, 1, 1);
        deepest_mid = l;
    }
    for (int l = deepest_mid; l >= 1; --l) {
        prolong_black(l, 0);
        launch(pdl, k_prolong_red, grid(l), kSegBlock, 0, st, L[l + 1], L[l], l, s.ctl, 0);
    }
    prolong_black(0, 1);
    if (rz_mode >= 0)
        launch(pdl, k_prolong_red_rz, grid(0), kSegBlock, 0, st, L[1], L[0], static_cast<const Ctl*>(s.ctl),
               part_rz(s));
    else
        launch(pdl, k_prolong_red, grid(0), kSegBlock, 0, st, L[1], L[0], 0, s.ctl, 1);
    return true;
}

}  // namespace apic
