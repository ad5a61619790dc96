// batch.h — many scenes' pressure solves as one launch per solve phase.
//
// A batched update runs every scene's Apic::update (src/apic.rs:2429-2474).
// The stages before and after the pressure solve are each scene's own
// kernels; the pressure solves of all scenes (solve_pcg :1865-1956 with the
// V-cycle of apply_preconditioner :1788-1821) run as one launch per phase
// over a table of scenes.  A phase with a block reduction runs, as its work
// items, blocks of the launch the scene alone would make (one or a group of
// consecutive ones per item), each with that launch's block index and grid
// size, so the block partials and their sums are the same bit for bit; a
// phase whose cells are independent of each other runs chunks of the level's
// segments.  Only the scenes whose own solve runs the phase take part (a
// substep is due, their refinement and PCG loops go on): the control kernel
// at each of those points lists them, with a prefix of their item counts per
// kind of phase, and the phase kernels are persistent, one wave of CTAs
// walking the listed items (grid-stride), so scenes that have converged cost
// nothing.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "apic_internal.h"
#include "vcycle_common.cuh"

namespace apic {

// A phase runs for a scene while the scene's own update graph would run it.
enum : int {
    kGateSolve = 1,   // a substep is due (ctl->go)
    kGateRefine = 2,  // and its refinement loop goes on (ctl->cond)
    kGatePcg = 3,     // and its PCG loop goes on (ctl->pcg_on)
};

// One scene of a batch, as the phase kernels read it.
struct BScene {
    Level lv[kMaxLevels];
    uint32_t grid[kMaxLevels];  // seg_grid of each level: the scene's own launch size
    Ctl* ctl;
    float *search, *ap, *corr, *pressure;
    double *b64, *p64, *partials;
    uint32_t nlevels, tail_first;
    uint32_t max_iter;
    int warm;
    double tol;
    vc::TailParams tp;  // the coarse tail, levels tail_first..nlevels-1
};

// The batch's own control block.
struct BCtl {
    uint32_t chunk_segs;    // segments per chunk item (a multiple of 8)
    uint32_t pcg_iters;     // executions of the batch's PCG loop body
    uint32_t refine_iters;  // ... of its refinement loop body
    uint32_t substeps;      // ... of its substep loop body
    uint32_t block_group;   // blocks per item of the PCG iteration's reductions
};

// The block partials of the split reductions, at the offsets a single-scene
// solve uses (part_sap, part_res, part_rz).
inline __host__ __device__ float2* bs_part_sap(const BScene& s) {
    return reinterpret_cast<float2*>(s.partials + 2 * kMaxRedBlocks);
}
inline __host__ __device__ float4* bs_part_res(const BScene& s) {
    return reinterpret_cast<float4*>(s.partials + 3 * kMaxRedBlocks);
}
inline __host__ __device__ float2* bs_part_rz(const BScene& s) {
    return reinterpret_cast<float2*>(s.partials + 5 * kMaxRedBlocks);
}

// Kinds of phases by the items a scene contributes.  Phases with a block
// reduction (the partials must come out as the single-scene launch forms
// them) run each block of that launch as it would: kKindBase, one item per
// block, for the reductions whose last block sums the partials; kKindBlocks
// for the PCG iteration's split reductions, whose partials the batch sums
// once per scene (k_bat_round_end, k_bat_sap): only the blocks that hold a
// segment, since the others' partials are zero and a zero adds nothing to
// the sums those partials feed (products and squares; a zero total stops
// the solve whatever its sign), block_group consecutive blocks per item.
// Phases whose every cell is computed independently of the others in the
// launch (sweeps of one colour, restriction, prolongation, copies) take one
// item per chunk of chunk_segs segments of the level: kind_chunk(l) for the
// levels the segment kernels smooth (l = 0, and l < tail_first),
// kind_rchunk(l) for the restriction into level l (l <= tail_first), and
// kKindExit: the base level's chunks after one item for the exit test.  The
// chunk counts follow the segment lists of the substep (ctl->seg_count).
// chunk_segs and block_group are the batch's shape (chosen by its tuner).
using Shape = BatchShape;
enum : int { kKindBase = 0, kKindExit = 1, kKindBlocks = 2 };
inline __host__ __device__ int kind_chunk(int l) { return 3 + 2 * l; }
inline __host__ __device__ int kind_rchunk(int l) { return 4 + 2 * l; }
inline __host__ __device__ uint32_t kinds_for(int max_tail) { return uint32_t(2 * max_tail + 5); }
#ifdef __CUDACC__
// Blocks of the scene's base-level launch that hold a segment (at least one).
__device__ __forceinline__ uint32_t busy_blocks(const BScene& s) {
    const uint32_t b = (s.ctl->seg_count[0] + kSegWarps - 1) / kSegWarps;
    return b < 1u ? 1u : (b < s.grid[0] ? b : s.grid[0]);
}
__device__ __forceinline__ uint32_t kind_items(const BScene& s, int kind, Shape sh) {
    if (kind == kKindBase) return s.grid[0];
    if (kind == kKindBlocks) return (busy_blocks(s) + sh.block_group - 1) / sh.block_group;
    const uint32_t* nseg = s.ctl->seg_count;
    const uint32_t cs = sh.chunk_segs;
    if (kind == kKindExit) return 1u + (nseg[0] + cs - 1) / cs;
    const uint32_t l = uint32_t(kind - 3) >> 1;
    const bool restrict_into = ((kind - 3) & 1) != 0;
    if (restrict_into) return (l >= 1 && l <= s.tail_first) ? (nseg[l] + cs - 1) / cs : 0u;
    if (l == 0) return max(1u, (nseg[0] + cs - 1) / cs);  // chunk 0 always exists
    return l < s.tail_first ? (nseg[l] + cs - 1) / cs : 0u;
}

// A chunk item's segments: [c cs, min(nseg, (c + 1) cs)), warp w of the CTA
// taking every 8th from c cs + w (the phase functions' walk with that first
// segment, stride and end).
struct Chunk {
    uint32_t end, warp, nwarps;
};
__device__ __forceinline__ Chunk chunk_of(uint32_t c, uint32_t nseg, Shape sh) {
    const uint32_t end = min(nseg, (c + 1) * sh.chunk_segs);
    return Chunk{end, c * sh.chunk_segs + (threadIdx.x >> 5), blockDim.x >> 5};
}
// The blocks of a block-group item.
__device__ __forceinline__ uint32_t group_end(const BScene& s, uint32_t item, Shape sh) {
    return min(busy_blocks(s), (item + 1) * sh.block_group);
}
#endif

// A list of the scenes taking part in the phases of one gate, in device
// memory (u32 words): [0] the count n_act, [1] the shape (chunk_segs |
// block_group << 16), [2, 2 + K) the item total of each
// kind, [2 + K, 2 + K + N) the scenes' indices in ascending order, then per
// kind k at 2 + K + N + k (N + 1): the prefix of their item counts (n_act + 1
// entries).  N: scenes in the batch, K: kinds.
struct BListRef {
    uint32_t* p = nullptr;
    uint32_t N = 0, K = 0;
    __host__ __device__ uint32_t words() const { return 2 + K + N + K * (N + 1); }
    __host__ __device__ uint32_t* scenes() const { return p + 2 + K; }
    __host__ __device__ uint32_t* prefix(uint32_t k) const { return p + 2 + K + N + k * (N + 1); }
};

#ifdef __CUDACC__
__device__ __forceinline__ bool bat_gate(const Ctl* c, int g) {
    return (g < kGateSolve || c->go) && (g < kGateRefine || c->cond) && (g < kGatePcg || c->pcg_on);
}

// Exclusive prefix of v over the block's threads (in thread order) and its
// total; every thread of the block calls it.
__device__ __forceinline__ uint32_t block_excl_scan(uint32_t v, uint32_t* total) {
    __shared__ uint32_t s_w[32];
    __shared__ uint32_t s_tot;
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    uint32_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= uint32_t(o)) x += y;
    }
    if (lane == 31) s_w[warp] = x;
    __syncthreads();
    if (warp == 0) {
        uint32_t u = lane < nw ? s_w[lane] : 0u;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, u, o);
            if (lane >= uint32_t(o)) u += y;
        }
        if (lane < nw) s_w[lane] = u;
        if (lane == 31) s_tot = u;
    }
    __syncthreads();
    const uint32_t r = x - v + (warp > 0 ? s_w[warp - 1] : 0u);
    *total = s_tot;
    __syncthreads();  // s_w and s_tot are reused by the next call
    return r;
}

// List the scenes whose gate is open and their items per kind (one block),
// with the batch's current shape.
__device__ __forceinline__ void bat_build_list(const BScene* __restrict__ tab, uint32_t n, int gate, BListRef L,
                                               const BCtl* bc) {
    const Shape sh{bc->chunk_segs, bc->block_group};
    uint32_t* scene = L.scenes();
    uint32_t nact = 0;
    for (uint32_t c0 = 0; c0 < n; c0 += blockDim.x) {
        const uint32_t i = c0 + threadIdx.x;
        const bool act = i < n && bat_gate(tab[i].ctl, gate);
        uint32_t tot;
        const uint32_t pos = block_excl_scan(act ? 1u : 0u, &tot);
        if (act) scene[nact + pos] = i;
        nact += tot;
    }
    __syncthreads();
    for (uint32_t k = 0; k < L.K; ++k) {
        uint32_t* pre = L.prefix(k);
        uint32_t carry = 0;
        for (uint32_t j0 = 0; j0 < nact; j0 += blockDim.x) {
            const uint32_t j = j0 + threadIdx.x;
            const uint32_t v = j < nact ? kind_items(tab[scene[j]], int(k), sh) : 0u;
            uint32_t tot;
            const uint32_t ex = block_excl_scan(v, &tot);
            if (j < nact) pre[j] = carry + ex;
            carry += tot;
        }
        if (threadIdx.x == 0) {
            pre[nact] = carry;
            L.p[2 + k] = carry;
        }
    }
    if (threadIdx.x == 0) {
        L.p[0] = nact;
        L.p[1] = sh.chunk_segs | (sh.block_group << 16);
    }
    __syncthreads();
}

// Walk the listed items of one kind, grid-stride: f(scene, item, shape) with
// the whole CTA, all three uniform across the CTA; the walk waits on the
// previous kernel (pdl_wait) itself.  Warp 0 finds an item's scene with a
// 32-way search of the prefix (two rounds for up to 1024 scenes).  early:
// the list was written two or more launches before this kernel (every phase
// of a PCG iteration after the first), so the header and the first item's
// scene are read while the previous kernel drains, from L2 (a grid that has
// completed has its writes there).
template <bool kL2>
__device__ __forceinline__ uint32_t list_word(const uint32_t* p) {
    return kL2 ? __ldcg(p) : *p;
}
template <bool kL2>
__device__ __forceinline__ void bat_find(const BListRef& L, const uint32_t* pre, uint32_t t, uint32_t nact,
                                         uint32_t* s_sc, uint32_t* s_lb) {
    if (threadIdx.x >= 32) return;
    const uint32_t lane = threadIdx.x & 31;
    uint32_t lo = 0, hi = nact;  // the last listed scene with pre <= t lies in [lo, hi)
    while (hi - lo > 1) {
        const uint32_t step = (hi - lo + 31) >> 5;
        const uint32_t j = lo + lane * step;
        const uint32_t ok = __ballot_sync(0xffffffffu, j < hi && list_word<kL2>(pre + j) <= t);
        lo += (31u - uint32_t(__clz(ok))) * step;  // lane 0 always holds (pre[lo] <= t)
        hi = min(hi, lo + step);
    }
    if (lane == 0) {
        *s_sc = list_word<kL2>(L.scenes() + lo);
        *s_lb = t - list_word<kL2>(pre + lo);
    }
}
template <class F>
__device__ __forceinline__ void bat_for_items(const BListRef L, int kind, bool early, F&& f) {
    __shared__ uint32_t s_sc, s_lb, s_tot, s_nact, s_shape;
    const uint32_t* pre = L.prefix(uint32_t(kind));
    if (early) {
        if (threadIdx.x == 0) {
            s_tot = __ldcg(L.p + 2 + kind);
            s_nact = __ldcg(L.p);
            s_shape = __ldcg(L.p + 1);
        }
        __syncthreads();
        if (blockIdx.x < s_tot) bat_find<true>(L, pre, blockIdx.x, s_nact, &s_sc, &s_lb);
        pdl_wait();
    } else {
        pdl_wait();
        if (threadIdx.x == 0) {
            s_tot = L.p[2 + kind];
            s_nact = L.p[0];
            s_shape = L.p[1];
        }
        __syncthreads();
        if (blockIdx.x < s_tot) bat_find<false>(L, pre, blockIdx.x, s_nact, &s_sc, &s_lb);
    }
    __syncthreads();
    const uint32_t tot = s_tot, nact = s_nact;
    const Shape sh{s_shape & 0xFFFFu, s_shape >> 16};
    for (uint32_t t = blockIdx.x; t < tot; t += gridDim.x) {
        if (t != blockIdx.x) {
            bat_find<false>(L, pre, t, nact, &s_sc, &s_lb);
            __syncthreads();
        }
        f(s_sc, s_lb, sh);
        __syncthreads();
    }
}
#endif

// What the phase launchers need.
struct BatchRun {
    const BScene* tab = nullptr;
    BCtl* bc = nullptr;
    uint32_t nscenes = 0;
    cudaStream_t st = nullptr;
    bool pdl = true;
    size_t tail_smem = 0;   // dynamic shared memory of the tail launch (the largest scene's)
    BListRef list[4];       // index: gate (1..3)
};

// CTAs of a persistent launch of `kernel`: as many as are resident at once.
template <class K> inline uint32_t persistent_grid(K kernel, int threads, size_t smem) {
    int dev = 0, sms = 1, per_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads, smem) != cudaSuccess) per_sm = 1;
    return uint32_t(per_sm > 0 ? per_sm : 1) * uint32_t(sms);
}

// ---- phase launchers (solver.cu) ----
void bat_solve_begin(const BatchRun& r);
void bat_mixed_init(const BatchRun& r, int gate);
void bat_clear_pressure(const BatchRun& r, int gate);
void bat_rel_begin(const BatchRun& r, int mixed);
void bat_true_residual(const BatchRun& r, int gate, int flags);
void bat_refine_cond(const BatchRun& r, cudaGraphConditionalHandle h, int gate);
void bat_pcg_begin(const BatchRun& r, int gate);
void bat_pcg_start(const BatchRun& r, int gate);
void bat_pcg_cond(const BatchRun& r, cudaGraphConditionalHandle h, int gate);
void bat_round_end(const BatchRun& r, cudaGraphConditionalHandle h);
void bat_sap(const BatchRun& r);
void bat_spmv_dot(const BatchRun& r);
void bat_pcg_update(const BatchRun& r, int into_corr);
void bat_mixed_accumulate(const BatchRun& r, int gate, int finalize);
void bat_refine_end(const BatchRun& r);
void bat_finish_solve(const BatchRun& r);
void bat_pressure_to64(const BatchRun& r, int gate);
// ---- V-cycle launchers (vcycle.cu) ----
void bat_smooth_exit(const BatchRun& r);
void bat_smooth(const BatchRun& r, int l, int gate, int color, int init);
void bat_restrict(const BatchRun& r, int l, int gate);
void bat_prolong_black(const BatchRun& r, int l, int gate, int base);
void bat_prolong_red(const BatchRun& r, int l, int gate, int base);
void bat_prolong_red_rz(const BatchRun& r);
void bat_tail(const BatchRun& r, int gate);
void bat_prepare_tail();

}  // namespace apic
