// solver.cu — multigrid-preconditioned CG pressure solve.
//
// Restates Apic::solve_pcg (src/apic.rs:1865-1956) with its preconditioner
// apply_preconditioner (:1788-1821): one V-cycle of red/black SOR (omega 1.2,
// one pre- and one post-sweep, MultiGridLevel::smooth_level :471-535),
// residual restriction over 2x2 children (:537-594), piecewise-constant
// prolongation (:596-616; on the base level the last fluid cell receives the
// correction once more per duplicate that pads the reference's list to a
// multiple of 8, :1487-1494) and plain CG on the coarsest level
// (solve_coarse_exact :618-704, one CTA here).
//
// Every kernel is a grid-stride loop over the level's segment list whose
// length lives in device memory, and returns at once when the device-side
// `pcg_done` flag is set, so an iteration costs no host round trip.  Dot
// products accumulate FP32 products in FP64 and are reduced deterministically
// (per-block partials summed in block order by the last block).  The
// reference's alpha/beta/gamma are FP32 and so are they here: the FP64 sums
// are rounded to float before the reference's FP32 divisions.
//
// Solver modes: APIC_SOLVER_REFERENCE keeps the reference's exits (max|r| <
// solve_error, gamma/delta < 1e-5, 100 iterations).  APIC_SOLVER_REL_FP32
// iterates to ||r||_2 <= tol*||b||_2.  APIC_SOLVER_REL_MIXED wraps FP32 inner
// solves in FP64 iterative refinement on the true residual b - A p.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>

#include "apic_device.cuh"
#include "apic_graph.h"
#include "apic_internal.h"
#include "batch.h"
#include "pcg_common.cuh"

namespace apic {
namespace {

constexpr float kSafety = 1e-5f;  // SAFTY, src/apic.rs:8
constexpr uint32_t kDeltaChunk = 8192;  // apply_matrix_and_dot's par_chunks(8192), src/apic.rs:1857-1859

__device__ __forceinline__ uint32_t gwarp() { return (blockIdx.x * blockDim.x + threadIdx.x) >> 5; }
__device__ __forceinline__ uint32_t gnwarps() { return (gridDim.x * blockDim.x) >> 5; }

// A PCG solve's starting state.
__device__ __forceinline__ void pcg_reset(Ctl* ctl) {
    ctl->pcg_done = 0;
    ctl->pcg_iters = 0;
    ctl->gamma = 0.0f;
    ctl->alpha = 0.0f;
    ctl->beta = 0.0f;
    ctl->beta_valid = 0;
    ctl->delta_stop = 0;
    ctl->rnorm2 = 0.0;
}

__global__ void k_pcg_begin(Ctl* ctl, int stamp) {
    if (stamp) ctl->solve_t0 = global_ns();
    pcg_reset(ctl);
}

// ---- PCG kernels on the base level (phases in pcg_common.cuh) --------------

// Each kernel's work is a body taking the block's coordinates in its scene's
// grid (bk), run by the single-scene kernel with the hardware's and by the
// batch kernel (one launch over many scenes, batch.h) with the scene's.

__global__ void __launch_bounds__(kSegBlock) k_clear_pressure(Level B, float* p, const Ctl* ctl) {
    pcg::ph_clear_pressure(B, ctl->seg_count[0], gwarp(), gnwarps(), p);
}

// s = z and gamma = r.z (src/apic.rs:1887-1892).
// In the reference mode k_gamma_exact forms gamma and the exit instead.
__device__ __forceinline__ void kb_pcg_start(Blk bk, const Level& B, float* s, Ctl* ctl, double* partials, int mode) {
    F2 acc = pcg::ph_start(B, ctl->seg_count[0], blk_warp(bk), blk_nwarps(bk), s);
    if (mode == APIC_SOLVER_REFERENCE) return;
    double tot;
    if (block_sum_last<kSegBlock>(bk, acc, partials, &ctl->red_counter, &tot) && threadIdx.x == 0) {
        float gamma = float(tot);
        ctl->gamma = gamma;
        ctl->dgamma = tot;
        if (mode == APIC_SOLVER_REFERENCE ? (gamma < kSafety) : !(gamma != 0.0f)) ctl->pcg_done = 1;
    }
}
__global__ void __launch_bounds__(kSegBlock) k_pcg_start(Level B, float* s, Ctl* ctl, double* partials, int mode) {
    pdl_wait();
    kb_pcg_start(hw_blk(), B, s, ctl, partials, mode);
}

// s' = z + beta s, Ap = A s' and this block's part of delta = s'.Ap
// (apply_matrix_and_dot, src/apic.rs:1823-1863; the search update
// :1945-1954 is folded in).  k_pcg_update sums the parts.
// In the relative modes the previous iteration's r.z arrives as the parts
// its V-cycle stored (rz): every block sums them into gamma' and forms
// beta = gamma' / gamma (:1934-1943); a zero r.z ends the solve (k_pcg_update
// records it).  Block 0 keeps beta for k_pcg_update.
// (after the dependency wait; w0: this warp's first segment word)
// rz_sum: the parts' sum formed once beforehand (batched solves), else null.
__device__ __forceinline__ void kb_spmv_dot(Blk bk, const Level& B, uint32_t nseg, uint32_t w0, const float* s,
                                            float* ap, Ctl* ctl, float2* part, int mode, const float2* rz,
                                            uint32_t nrz, const float* rz_sum = nullptr) {
    if (ctl->pcg_done) return;
    float beta = ctl->beta;
    const bool bv = ctl->beta_valid != 0;
    if (mode != APIC_SOLVER_REFERENCE && bv) {
        const float ng = rz_sum ? *rz_sum : float(sum_partials<kSegBlock>(rz, nrz));
        if (!(ng != 0.0f)) return;
        beta = ng / ctl->gamma;
        if (bk.id == 0 && threadIdx.x == 0) ctl->beta = beta;
    }
    F2 acc = pcg::ph_spmv_search(B, nseg, blk_warp(bk), blk_nwarps(bk), s, beta, bv, ap, w0);
    block_store<kSegBlock>(bk, acc, part);
}
__global__ void __launch_bounds__(kSegBlock) k_spmv_dot(Level B, const float* s, float* ap, Ctl* ctl, float2* part,
                                                        int mode, const float2* rz, uint32_t nrz) {
    // the base segment list is written by the substep's setup: load this
    // warp's first word before waiting on the previous kernel
    const uint32_t nseg = ctl->seg_count[0];
    const uint32_t w0 = gwarp() < nseg ? B.seg[gwarp()] : 0xFFFFFFFFu;
    pdl_wait();
    kb_spmv_dot(hw_blk(), B, nseg, w0, s, ap, ctl, part, mode, rz, nrz);
}

// delta (the sum of k_spmv_dot's parts, formed by every block) gives alpha or
// the exit (src/apic.rs:1899-1906, applied by the next kernel); then
// p += alpha s', r = fma(-alpha, Ap, r)
// (:1907-1932), s = s', the V-cycle's first red sweep on the base level, and
// this block's part of ||r||^2 and max|r|, whose exit test runs in the next
// kernel (k_smooth_conv).
// rz_sum, sap_sum: the parts' sums formed once beforehand (batched solves).
__device__ __forceinline__ void kb_pcg_update(Blk bk, const Level& B, uint32_t nseg, uint32_t w0, float* p,
                                              int p_padded, float* s, const float* ap, Ctl* ctl, const float2* sap,
                                              uint32_t nsap, float4* part, int mode, const float* exact_parts,
                                              const uint32_t* seg_pre, const float2* rz, uint32_t nrz,
                                              const float* rz_sum = nullptr, const float* sap_sum = nullptr) {
    if (ctl->pcg_done) return;
    // this iteration's gamma: from the solve's start, or (relative modes) the
    // previous iteration's r.z parts, which k_spmv_dot summed the same way
    float gamma = ctl->gamma;
    if (mode != APIC_SOLVER_REFERENCE && ctl->beta_valid) {
        gamma = rz_sum ? *rz_sum : float(sum_partials<kSegBlock>(rz, nrz));
        if (!(gamma != 0.0f)) {
            if (bk.id == 0 && threadIdx.x == 0) ctl->pcg_done = 1;
            return;
        }
    }
    float delta;
    if (mode == APIC_SOLVER_REFERENCE) {
        // the chunk sums of k_delta_exact, added in chunk order from zero
        const uint32_t nchunks = (seg_pre[ctl->seg_count[0]] + kDeltaChunk - 1) / kDeltaChunk;
        delta = 0.0f;
        for (uint32_t c = 0; c < nchunks; ++c) delta = delta + exact_parts[c];
    } else {
        delta = sap_sum ? *sap_sum : float(sum_partials<kSegBlock>(sap, nsap));
    }
    const bool stop = mode == APIC_SOLVER_REFERENCE ? fabsf(delta) < kSafety : (!(delta != 0.0f) || !isfinite(delta));
    const float alpha = gamma / delta;
    // every block reads pcg_done on entry, so the stop is recorded aside and
    // the next kernel turns it into pcg_done
    if (bk.id == 0 && threadIdx.x == 0) {
        ctl->gamma = gamma;
        ctl->pcg_iters++;
        ctl->delta_stop = stop ? 1u : 0u;
        if (!stop) ctl->alpha = alpha;
    }
    if (stop) return;
    float mx;
    F2 acc;
    pcg::ph_update_search(B, nseg, blk_warp(bk), blk_nwarps(bk), alpha, ctl->beta, ctl->beta_valid != 0, p, p_padded,
                          s, ap, &mx, &acc, w0);
    block_store<kSegBlock>(bk, acc, mx, part);
}
__global__ void __launch_bounds__(kSegBlock) k_pcg_update(Level B, float* p, int p_padded, float* s,
                                                          const float* ap, Ctl* ctl, const float2* sap,
                                                          uint32_t nsap, float4* part, int mode,
                                                          const float* exact_parts, const uint32_t* seg_pre,
                                                          const float2* rz, uint32_t nrz) {
    const uint32_t nseg = ctl->seg_count[0];
    const uint32_t w0 = gwarp() < nseg ? B.seg[gwarp()] : 0xFFFFFFFFu;
    pdl_wait();
    kb_pcg_update(hw_blk(), B, nseg, w0, p, p_padded, s, ap, ctl, sap, nsap, part, mode, exact_parts, seg_pre, rz,
                  nrz);
}

// Stand-alone exit test (paths whose V-cycle does not start with the base
// level's black sweep).
__global__ void __launch_bounds__(kSegBlock) k_residual_exit(Ctl* ctl, const float4* part, uint32_t n, int mode,
                                                             float solve_error, cudaGraphConditionalHandle h,
                                                             uint32_t cap, int dyn_cap, int set_cond) {
    pdl_wait();
    if (!ctl->pcg_done) pcg::residual_exit(ctl, part, n, mode, solve_error);
    if (threadIdx.x == 0) pcg::loop_decision(ctl, mode, h, cap, dyn_cap, set_cond);
}

// This block's part of gamma' = r.z (src/apic.rs:1934-1943); the next
// iteration's k_spmv_dot and k_pcg_update sum the parts.
__global__ void __launch_bounds__(kSegBlock) k_dot_rz(Level B, Ctl* ctl, float2* part) {
    pdl_wait();
    if (ctl->pcg_done) return;
    F2 acc = pcg::ph_rz(B, ctl->seg_count[0], gwarp(), gnwarps());
    block_store<kSegBlock>(hw_blk(), acc, part);
}

// ---- the reference's FP32 reduction orders (APIC_SOLVER_REFERENCE) --------
//
// Float addition is not associative, so the reference mode forms its two
// Krylov reductions in exactly the reference's order; the solve is then
// bit-identical to the oracle's.

// gamma = dot_product(residual[W..W+cells], error[W..W+cells]) (:11-29): eight
// lane sums, lane = raw index mod 8, each added in ascending order; then
// wide's reduce_add pairing ((l0 + l2) + (l1 + l3)) + ((l4 + l6) + (l5 + l7));
// then the cells beyond the last full chunk of 8, serially.  The error is
// zero outside the fluid cells (apply_preconditioner zeroes it, :1790-1792,
// and only fluid cells are smoothed or prolonged), and adding a zero product
// leaves a lane sum unchanged (the sums start at +0 and never become -0), so
// only the fluid cells' products count.  One block: warps 1..31 stage the
// products of a batch of segments (32 raw cells each, zero where not fluid)
// in shared memory while threads 0..7 add the previous batch's products of
// their lane in order (two stage buffers); only those eight add chains are
// serial.
// start: the solve's first gamma (sets gamma and the SAFTY exit,
// :1887-1892), else the iteration's new gamma.
constexpr int kGammaThreads = 1024;
constexpr uint32_t kGammaBatch = 512;  // segments staged per round (64 KB)
constexpr size_t kGammaSmem = 2 * size_t(kGammaBatch) * 32 * sizeof(float);
// The iteration's form (start 0) also finishes the iteration (beta, or the
// SAFTY exit) and, when set_cond, sets the loop condition.
__global__ void __launch_bounds__(kGammaThreads) k_gamma_exact(Level B, Ctl* ctl, int start,
                                                               cudaGraphConditionalHandle h, uint32_t cap,
                                                               int dyn_cap, int set_cond) {
    extern __shared__ float stage[];  // two buffers of kGammaBatch segments
    pdl_wait();
    if (ctl->pcg_done) return;
    const uint32_t t = threadIdx.x, lane = t & 31, warp = t >> 5;
    const uint32_t nseg = ctl->seg_count[0];
    const uint32_t full = (B.cells / 8u) * 8u;
    const uint32_t nbatch = (nseg + kGammaBatch - 1) / kGammaBatch;
    // warps 1..31 stage batch b into buffer b % 2
    auto fill = [&](uint32_t b) {
        float* buf = stage + (b & 1u) * kGammaBatch * 32u;
        const uint32_t k0 = b * kGammaBatch, nb = min(kGammaBatch, nseg - k0);
        for (uint32_t q = warp - 1; q < nb; q += kGammaThreads / 32 - 1) {
            const uint32_t w = B.seg[k0 + q];
            const uint32_t raw = w * 32u + lane;
            const bool on = ((B.fluid[w] >> lane) & 1u) && raw < full;
            buf[q * 32u + lane] = on ? B.res[raw + B.w] * B.err[raw + B.w] : 0.0f;
        }
    };
    float acc = 0.0f;
    if (warp != 0 && nbatch > 0) fill(0);
    __syncthreads();
    for (uint32_t b = 0; b < nbatch; ++b) {
        if (warp == 0) {
            if (t < 8) {
                const float* buf = stage + (b & 1u) * kGammaBatch * 32u;
                const uint32_t nb = min(kGammaBatch, nseg - b * kGammaBatch);
                for (uint32_t q = 0; q < nb; ++q) {
                    const float* p = buf + q * 32u + t;
                    acc = acc + p[0];
                    acc = acc + p[8];
                    acc = acc + p[16];
                    acc = acc + p[24];
                }
            }
        } else if (b + 1 < nbatch) {
            fill(b + 1);
        }
        __syncthreads();
    }
    __shared__ float lanes[8];
    if (t < 8) lanes[t] = acc;
    __syncthreads();
    if (t != 0) return;
    float g = ((lanes[0] + lanes[2]) + (lanes[1] + lanes[3])) + ((lanes[4] + lanes[6]) + (lanes[5] + lanes[7]));
    for (uint32_t raw = full; raw < B.cells; ++raw)
        if (bit_at(B.fluid, raw)) g = g + B.res[raw + B.w] * B.err[raw + B.w];
    if (start) {
        ctl->gamma = g;
        ctl->dgamma = double(g);
        if (g < kSafety) ctl->pcg_done = 1;
    } else {
        pcg::finish_rz_reference(ctl, g);
        if (set_cond) {
            const uint32_t c = dyn_cap ? ctl->inner_cap : cap;
            cudaGraphSetConditional(h, (!ctl->pcg_done && ctl->pcg_iters < c) ? 1u : 0u);
        }
    }
}

// Fluid cells before each base segment (seg_pre[k], k <= nseg; seg_pre[nseg]
// = all fluid cells): the position of a segment's cells in the reference's
// ascending fluid list.  One block, once per solve.
__global__ void __launch_bounds__(1024) k_seg_prefix(Level B, const Ctl* ctl, uint32_t* seg_pre) {
    const uint32_t nseg = ctl->seg_count[0];
    __shared__ uint32_t sw[32];
    const uint32_t t = threadIdx.x, lane = t & 31, warp = t >> 5;
    uint32_t carry = 0;
    for (uint32_t k0 = 0; k0 < nseg; k0 += 1024) {
        const uint32_t k = k0 + t;
        const uint32_t v = k < nseg ? uint32_t(__popc(B.fluid[B.seg[k]])) : 0u;
        uint32_t x = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= uint32_t(o)) x += y;
        }
        if (lane == 31) sw[warp] = x;
        __syncthreads();
        if (warp == 0) {
            uint32_t u = sw[lane];
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t y = __shfl_up_sync(0xffffffffu, u, o);
                if (lane >= uint32_t(o)) u += y;
            }
            sw[lane] = u;
        }
        __syncthreads();
        if (k < nseg) seg_pre[k] = carry + (warp > 0 ? sw[warp - 1] : 0u) + x - v;
        const uint32_t tot = sw[31];
        __syncthreads();
        carry += tot;
    }
    if (t == 0) seg_pre[nseg] = carry;
}

// delta = apply_matrix_and_dot's sum (:1823-1863): s'.Ap over the fluid cells
// in ascending order, in chunks of 8192 cells each summed serially from zero
// (rayon's par_chunks(8192)); k_pcg_update then adds the chunk sums in chunk
// order.  s' is the iteration's search direction, z + beta s (k_spmv_dot
// evaluates the same expression).  One block per chunk: its warps stage the
// chunk's products in fluid order in shared memory (positions from
// seg_pre), then one thread adds them in order.
constexpr int kDeltaThreads = 256;
__global__ void __launch_bounds__(kDeltaThreads) k_delta_exact(Level B, const float* __restrict__ s,
                                                               const float* __restrict__ ap,
                                                               const uint32_t* __restrict__ seg_pre, Ctl* ctl,
                                                               float* __restrict__ parts) {
    __shared__ float prod[kDeltaChunk];
    __shared__ uint32_t s_k0, s_k1;
    pdl_wait();
    if (ctl->pcg_done) return;
    const uint32_t nseg = ctl->seg_count[0];
    const uint32_t nfluid = seg_pre[nseg];
    const uint32_t c = blockIdx.x;
    const uint32_t f0 = c * kDeltaChunk;
    if (f0 >= nfluid) return;
    const uint32_t f1 = min(f0 + kDeltaChunk, nfluid);
    if (threadIdx.x == 0) {
        // segments [k0, k1) hold fluid cells f0 .. f1-1 (every segment holds at least one)
        uint32_t lo = 0, hi = nseg;  // last k with seg_pre[k] <= f0
        while (hi - lo > 1) {
            const uint32_t mid = (lo + hi) / 2;
            if (seg_pre[mid] <= f0) lo = mid; else hi = mid;
        }
        s_k0 = lo;
        uint32_t lo2 = lo, hi2 = nseg;  // first k with seg_pre[k] >= f1
        while (lo2 < hi2) {
            const uint32_t mid = (lo2 + hi2) / 2;
            if (seg_pre[mid] < f1) lo2 = mid + 1; else hi2 = mid;
        }
        s_k1 = lo2;
    }
    __syncthreads();
    const float beta = ctl->beta;
    const bool beta_valid = ctl->beta_valid != 0;
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (uint32_t k = s_k0 + warp; k < s_k1; k += kDeltaThreads / 32) {
        const uint32_t w = B.seg[k];
        const uint32_t m = B.fluid[w];
        if (!((m >> lane) & 1u)) continue;
        const uint32_t pos = seg_pre[k] + uint32_t(__popc(m & ((1u << lane) - 1u)));
        if (pos < f0 || pos >= f1) continue;
        const uint32_t cidx = w * 32u + lane + B.w;
        prod[pos - f0] = ap[cidx] * pcg::search_at(B.err, s, beta, beta_valid, cidx);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        float sum = 0.0f;
        for (uint32_t i = 0; i < f1 - f0; ++i) sum = sum + prod[i];
        parts[c] = sum;
    }
}

// ---- FP64 refinement helpers (APIC_SOLVER_REL_MIXED) ----------------------

// b64 = res, p64 = 0 (unless warm) and ||b||^2.
__device__ __forceinline__ void kb_mixed_init(Blk bk, const Level& B, double* b64, double* p64, Ctl* ctl,
                                              double* partials, int warm) {
    if (bk.id == 0 && threadIdx.x == 0) ctl->solve_t0 = global_ns();  // the relative-mode solve starts here
    double bb = pcg::ph_mixed_init(B, ctl->seg_count[0], blk_warp(bk), blk_nwarps(bk), b64, p64, warm);
    double tot;
    if (block_sum_last<kSegBlock>(bk, bb, partials, &ctl->red_counter, &tot) && threadIdx.x == 0) ctl->bnorm2 = tot;
}
__global__ void __launch_bounds__(kSegBlock) k_mixed_init(Level B, double* b64, double* p64, Ctl* ctl,
                                                          double* partials, int warm) {
    kb_mixed_init(hw_blk(), B, b64, p64, ctl, partials, warm);
}

// True relative residual of p64 (flags: see pcg::ph_true_residual).
__device__ __forceinline__ void kb_true_residual(Blk bk, const Level& B, const double* b64, const double* p64,
                                                 float* x, Ctl* ctl, double* partials, int flags) {
    double rr = pcg::ph_true_residual(B, ctl->seg_count[0], blk_warp(bk), blk_nwarps(bk), b64, p64, x, flags);
    double tot;
    if (block_sum_last<kSegBlock>(bk, rr, partials, &ctl->red_counter, &tot) && threadIdx.x == 0)
        ctl->true_rel = ctl->bnorm2 > 0.0 ? sqrt(tot / ctl->bnorm2) : 0.0;
}
__global__ void __launch_bounds__(kSegBlock) k_true_residual(Level B, const double* b64, const double* p64, float* x,
                                                             Ctl* ctl, double* partials, int flags) {
    kb_true_residual(hw_blk(), B, b64, p64, x, ctl, partials, flags);
}

// p64 += x (finalize 0; the refinement also counts the inner solve's
// iterations), or pressure = float(p64) (finalize 1).
__device__ __forceinline__ void kb_mixed_accumulate(Blk bk, const Level& B, double* p64, const float* x,
                                                    float* pressure, Ctl* ctl, int finalize) {
    pcg::ph_accumulate(B, ctl->seg_count[0], blk_warp(bk), blk_nwarps(bk), p64, x, pressure, finalize);
    if (!finalize && bk.id == 0 && threadIdx.x == 0) ctl->used_iters += ctl->pcg_iters;
}
__global__ void __launch_bounds__(kSegBlock) k_mixed_accumulate(Level B, double* p64, const float* x, float* pressure,
                                                                Ctl* ctl, int finalize) {
    kb_mixed_accumulate(hw_blk(), B, p64, x, pressure, ctl, finalize);
}

__global__ void __launch_bounds__(kSegBlock) k_pressure_to64(Level B, const float* pressure, double* p64,
                                                             const Ctl* ctl) {
    pcg::ph_pressure_to64(B, ctl->seg_count[0], gwarp(), gnwarps(), pressure, p64);
}

// ---- loop control (device side; each sets a graph conditional) ------------

// Entry of the PCG loop: go on while not converged and under the iteration
// cap (src/apic.rs:1894-1899); dyn_cap reads the remaining budget of a
// refinement.  Inside the loop the same decision is taken by the kernel that
// runs the residual's exit test (pcg::loop_decision) or, in the reference
// mode, by k_gamma_exact.
__device__ __forceinline__ bool pcg_entry(const Ctl* ctl, uint32_t cap, int dyn_cap) {
    const uint32_t c = dyn_cap ? ctl->inner_cap : cap;
    return !ctl->pcg_done && ctl->pcg_iters < c;
}
__global__ void k_pcg_cond(const Ctl* __restrict__ ctl, cudaGraphConditionalHandle h, uint32_t cap, int dyn_cap) {
    pdl_wait();
    cudaGraphSetConditional(h, pcg_entry(ctl, cap, dyn_cap) ? 1u : 0u);
}

__device__ __forceinline__ void finish_solve(Ctl* ctl, uint32_t cap) {
    ctl->solve_ns += global_ns() - ctl->solve_t0;
    ctl->pcg_iters_total += ctl->pcg_iters;
    if (ctl->pcg_iters >= cap && !ctl->pcg_done) ctl->not_converged++;
}
__global__ void k_finish_solve(Ctl* ctl, uint32_t cap) { finish_solve(ctl, cap); }

__device__ __forceinline__ void rel_begin(Ctl* ctl, double tol, uint32_t cap) {
    ctl->target_rel = tol;
    ctl->inner_cap = cap;
    ctl->refinements = 0;
    ctl->used_iters = 0;
}
__global__ void k_rel_begin(Ctl* ctl, double tol, uint32_t cap) { rel_begin(ctl, tol, cap); }

// Refinement loop: go on while the FP64 true residual is above tol and
// iterations remain.  Each inner FP32 solve reduces its own right-hand side
// (the current true residual) by kInnerReduction, or down to tol / 2 of ||b||
// when that is reached first; FP32 cannot usefully reduce it further.
constexpr double kInnerReduction = 1e-4;
__device__ __forceinline__ bool refine_cond(Ctl* ctl, double tol, uint32_t cap) {
    bool cont = ctl->true_rel > tol && ctl->used_iters < cap && ctl->refinements < 32u;
    // an inner solve that could not take a single step (r.z underflows or is
    // zero) will not make progress on the next round either
    if (ctl->refinements > 0u && ctl->pcg_iters == 0u) cont = false;
    if (cont) {
        ctl->refinements++;
        ctl->inner_cap = cap - ctl->used_iters;
        double t = kInnerReduction * ctl->true_rel;  // target relative to ||b||
        ctl->target_rel = t > 0.5 * tol ? t : 0.5 * tol;
        pcg_reset(ctl);  // the inner solve that follows starts here
    }
    ctl->cond = cont ? 1u : 0u;
    return cont;
}
__global__ void k_refine_cond(Ctl* ctl, cudaGraphConditionalHandle h, double tol, uint32_t cap, int graph) {
    const bool cont = refine_cond(ctl, tol, cap);
    if (graph) cudaGraphSetConditional(h, cont ? 1u : 0u);
}

__device__ __forceinline__ void refine_end(Ctl* ctl, double tol) {
    ctl->solve_ns += global_ns() - ctl->solve_t0;
    ctl->refinements_total += ctl->refinements;
    ctl->pcg_iters = ctl->used_iters;
    ctl->pcg_iters_total += ctl->used_iters;
    if (ctl->true_rel > tol) ctl->not_converged++;
}
__global__ void k_refine_end(Ctl* ctl, double tol) { refine_end(ctl, tol); }

// ---- the same phases over a batch of scenes (batch.h) ----------------------
// Segment phases: persistent CTAs walk the listed items of their gate (each a
// block of a scene's own launch, with that launch's coordinates) and run the
// single-scene body.  Control phases: one CTA, a thread per scene; they list
// the scenes for the phases that follow, and the OR of the scenes' loop
// decisions is the batch loop's condition.  The PCG runs in a relative mode
// (APIC_SOLVER_REL_FP32 arithmetic, as the inner solves of both relative
// modes do).
constexpr int kBatCtlThreads = 1024;
constexpr int kRel = APIC_SOLVER_REL_FP32;

// Start of the batch's solves: list the scenes with a substep due (their
// segment lists are those of this substep's multigrid setup).
__global__ void __launch_bounds__(kBatCtlThreads) k_bat_solve_begin(const BScene* __restrict__ tab, uint32_t n,
                                                                   const BCtl* bc, BListRef l1) {
    bat_build_list(tab, n, kGateSolve, l1, bc);
}

__global__ void __launch_bounds__(kBatCtlThreads) k_bat_rel_begin(const BScene* __restrict__ tab, uint32_t n,
                                                                 int mixed, const BCtl* bc, BListRef l2) {
    for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) {
        Ctl* ctl = tab[i].ctl;
        if (!bat_gate(ctl, kGateSolve)) continue;
        rel_begin(ctl, tab[i].tol, tab[i].max_iter);
        if (!mixed) ctl->cond = 1u;  // no refinement loop: its gate stays open
    }
    if (mixed) return;
    __syncthreads();
    bat_build_list(tab, n, kGateRefine, l2, bc);
}

// gate kGateSolve: the loop's entry (every scene with a substep due decides);
// kGateRefine: the end of a refinement (the scenes still refining decide).
__global__ void __launch_bounds__(kBatCtlThreads) k_bat_refine_cond(const BScene* __restrict__ tab, uint32_t n,
                                                                   BCtl* bc, cudaGraphConditionalHandle h, int gate,
                                                                   BListRef l2) {
    bool any = false;
    for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) {
        Ctl* ctl = tab[i].ctl;
        if (bat_gate(ctl, gate) && refine_cond(ctl, tab[i].tol, tab[i].max_iter)) any = true;
    }
    any = __syncthreads_or(any) != 0;
    if (threadIdx.x == 0) {
        cudaGraphSetConditional(h, any ? 1u : 0u);
        if (any) bc->refine_iters++;
    }
    if (any) bat_build_list(tab, n, kGateRefine, l2, bc);
}

__global__ void __launch_bounds__(kBatCtlThreads) k_bat_refine_end(const BScene* __restrict__ tab, uint32_t n) {
    for (uint32_t i = threadIdx.x; i < n; i += blockDim.x)
        if (bat_gate(tab[i].ctl, kGateSolve)) refine_end(tab[i].ctl, tab[i].tol);
}

__global__ void __launch_bounds__(kBatCtlThreads) k_bat_finish_solve(const BScene* __restrict__ tab, uint32_t n) {
    for (uint32_t i = threadIdx.x; i < n; i += blockDim.x)
        if (bat_gate(tab[i].ctl, kGateSolve)) finish_solve(tab[i].ctl, tab[i].max_iter);
}

__global__ void __launch_bounds__(kBatCtlThreads) k_bat_pcg_begin(const BScene* __restrict__ tab, uint32_t n,
                                                                 int gate) {
    for (uint32_t i = threadIdx.x; i < n; i += blockDim.x)
        if (bat_gate(tab[i].ctl, gate)) pcg_reset(tab[i].ctl);
}

// Entry of the PCG loops (k_pcg_cond with the refinement's dynamic cap).
__global__ void __launch_bounds__(kBatCtlThreads) k_bat_pcg_cond(const BScene* __restrict__ tab, uint32_t n,
                                                                const BCtl* bc, cudaGraphConditionalHandle h,
                                                                int gate, BListRef l3) {
    pdl_wait();
    bool any = false;
    for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) {
        Ctl* ctl = tab[i].ctl;
        if (!bat_gate(ctl, gate)) continue;
        const bool cont = pcg_entry(ctl, 0u, 1);
        ctl->pcg_on = cont ? 1u : 0u;
        any = any || cont;
    }
    any = __syncthreads_or(any) != 0;
    if (threadIdx.x == 0) cudaGraphSetConditional(h, any ? 1u : 0u);
    if (any) bat_build_list(tab, n, kGatePcg, l3, bc);
}

// End of a batch PCG iteration: the exit items have taken every listed
// scene's decision.  CTA 0 lists the scenes that go on and sets the loop
// condition; CTA 1 + i sums scene i's r.z parts (stored by the V-cycle's
// last kernel) for the next iteration, once instead of in every block of
// k_spmv_dot and k_pcg_update (the same function of the same parts).
__global__ void __launch_bounds__(kSegBlock) k_bat_round_end(const BScene* __restrict__ tab, uint32_t n, BCtl* bc,
                                                            cudaGraphConditionalHandle h, BListRef l3) {
    pdl_wait();
    if (blockIdx.x == 0) {
        bat_build_list(tab, n, kGatePcg, l3, bc);
        if (threadIdx.x == 0) {
            cudaGraphSetConditional(h, l3.p[0] ? 1u : 0u);
            bc->pcg_iters++;
        }
        return;
    }
    const BScene& S = tab[blockIdx.x - 1];
    Ctl* ctl = S.ctl;
    if (!bat_gate(ctl, kGatePcg) || ctl->pcg_done) return;
    const float rz = float(sum_partials<kSegBlock>(bs_part_rz(S), busy_blocks(S)));
    if (threadIdx.x == 0) ctl->b_rz = rz;
}

// s.Ap of every listed scene (after k_bat_spmv_dot), once per scene.
__global__ void __launch_bounds__(kSegBlock) k_bat_sap(const BScene* __restrict__ tab, uint32_t n) {
    pdl_wait();
    const BScene& S = tab[blockIdx.x];
    Ctl* ctl = S.ctl;
    if (!bat_gate(ctl, kGatePcg) || ctl->pcg_done) return;
    const float sap = float(sum_partials<kSegBlock>(bs_part_sap(S), busy_blocks(S)));
    if (threadIdx.x == 0) ctl->b_sap = sap;
}

__global__ void __launch_bounds__(kSegBlock) k_bat_mixed_init(const BScene* __restrict__ tab, BListRef L, int gate) {
    bat_for_items(L, kKindBase, false, [&](uint32_t sc, uint32_t lb, Shape sh) {
        const BScene& S = tab[sc];
        if (!bat_gate(S.ctl, gate)) return;
        kb_mixed_init(Blk{lb, S.grid[0]}, S.lv[0], S.b64, S.p64, S.ctl, S.partials, S.warm);
    });
}

__global__ void __launch_bounds__(kSegBlock) k_bat_clear_pressure(const BScene* __restrict__ tab, BListRef L,
                                                                  int gate) {
    bat_for_items(L, kind_chunk(0), false, [&](uint32_t sc, uint32_t lb, Shape sh) {
        const BScene& S = tab[sc];
        if (!bat_gate(S.ctl, gate)) return;
        const Chunk ch = chunk_of(lb, S.ctl->seg_count[0], sh);
        pcg::ph_clear_pressure(S.lv[0], ch.end, ch.warp, ch.nwarps, S.pressure);
    });
}

__global__ void __launch_bounds__(kSegBlock) k_bat_true_residual(const BScene* __restrict__ tab, BListRef L, int gate,
                                                                 int flags) {
    bat_for_items(L, kKindBase, false, [&](uint32_t sc, uint32_t lb, Shape sh) {
        const BScene& S = tab[sc];
        if (!bat_gate(S.ctl, gate)) return;
        kb_true_residual(Blk{lb, S.grid[0]}, S.lv[0], S.b64, S.p64, S.corr, S.ctl, S.partials, flags);
    });
}

__global__ void __launch_bounds__(kSegBlock) k_bat_pcg_start(const BScene* __restrict__ tab, BListRef L, int gate) {
    bat_for_items(L, kKindBase, false, [&](uint32_t sc, uint32_t lb, Shape sh) {
        const BScene& S = tab[sc];
        if (!bat_gate(S.ctl, gate)) return;
        kb_pcg_start(Blk{lb, S.grid[0]}, S.lv[0], S.search, S.ctl, S.partials, kRel);
    });
}

__global__ void __launch_bounds__(kSegBlock, 8) k_bat_spmv_dot(const BScene* __restrict__ tab, BListRef L) {
    bat_for_items(L, kKindBlocks, false, [&](uint32_t sc, uint32_t item, Shape sh) {
        const BScene& S = tab[sc];
        Ctl* ctl = S.ctl;
        if (!bat_gate(ctl, kGatePcg)) return;
        const uint32_t nseg = ctl->seg_count[0], end = group_end(S, item, sh);
        for (uint32_t b = item * sh.block_group; b < end; ++b) {
            kb_spmv_dot(Blk{b, S.grid[0]}, S.lv[0], nseg, 0xFFFFFFFFu, S.search, S.ap, ctl, bs_part_sap(S), kRel,
                        bs_part_rz(S), S.grid[0], &ctl->b_rz);
            __syncthreads();  // block_store's shared slots are reused by the next block
        }
    });
}

__global__ void __launch_bounds__(kSegBlock, 8) k_bat_pcg_update(const BScene* __restrict__ tab, BListRef L,
                                                              int into_corr) {
    bat_for_items(L, kKindBlocks, true, [&](uint32_t sc, uint32_t item, Shape sh) {
        const BScene& S = tab[sc];
        Ctl* ctl = S.ctl;
        if (!bat_gate(ctl, kGatePcg)) return;
        const uint32_t nseg = ctl->seg_count[0], end = group_end(S, item, sh);
        for (uint32_t b = item * sh.block_group; b < end; ++b) {
            kb_pcg_update(Blk{b, S.grid[0]}, S.lv[0], nseg, 0xFFFFFFFFu, into_corr ? S.corr : S.pressure, into_corr,
                          S.search, S.ap, ctl, bs_part_sap(S), S.grid[0], bs_part_res(S), kRel, nullptr, nullptr,
                          bs_part_rz(S), S.grid[0], &ctl->b_rz, &ctl->b_sap);
            __syncthreads();
        }
    });
}

// (k_mixed_accumulate: chunk 0 also counts the inner solve's iterations)
__global__ void __launch_bounds__(kSegBlock) k_bat_mixed_accumulate(const BScene* __restrict__ tab, BListRef L,
                                                                    int gate, int finalize) {
    bat_for_items(L, kind_chunk(0), false, [&](uint32_t sc, uint32_t lb, Shape sh) {
        const BScene& S = tab[sc];
        Ctl* ctl = S.ctl;
        if (!bat_gate(ctl, gate)) return;
        const Chunk ch = chunk_of(lb, ctl->seg_count[0], sh);
        pcg::ph_accumulate(S.lv[0], ch.end, ch.warp, ch.nwarps, S.p64, S.corr, S.pressure, finalize);
        if (!finalize && lb == 0 && threadIdx.x == 0) ctl->used_iters += ctl->pcg_iters;
    });
}

__global__ void __launch_bounds__(kSegBlock) k_bat_pressure_to64(const BScene* __restrict__ tab, BListRef L,
                                                                 int gate) {
    bat_for_items(L, kind_chunk(0), false, [&](uint32_t sc, uint32_t lb, Shape sh) {
        const BScene& S = tab[sc];
        if (!bat_gate(S.ctl, gate)) return;
        const Chunk ch = chunk_of(lb, S.ctl->seg_count[0], sh);
        pcg::ph_pressure_to64(S.lv[0], ch.end, ch.warp, ch.nwarps, S.pressure, S.p64);
    });
}

}  // namespace

// ---- batch phase launchers (batch.h); launch kinds as in the single-scene
// graph: programmatic dependent launch where the predecessor is a kernel of
// the PCG setup or loop, plain launches elsewhere ----
#define APIC_PGRID(kern) static const uint32_t g = persistent_grid(kern, kSegBlock, 0)
void bat_solve_begin(const BatchRun& r) {
    k_bat_solve_begin<<<1, kBatCtlThreads, 0, r.st>>>(r.tab, r.nscenes, r.bc, r.list[kGateSolve]);
}
void bat_mixed_init(const BatchRun& r, int gate) {
    APIC_PGRID(k_bat_mixed_init);
    launch(false, k_bat_mixed_init, g, kSegBlock, 0, r.st, r.tab, r.list[gate], gate);
}
void bat_clear_pressure(const BatchRun& r, int gate) {
    APIC_PGRID(k_bat_clear_pressure);
    launch(false, k_bat_clear_pressure, g, kSegBlock, 0, r.st, r.tab, r.list[gate], gate);
}
void bat_rel_begin(const BatchRun& r, int mixed) {
    k_bat_rel_begin<<<1, kBatCtlThreads, 0, r.st>>>(r.tab, r.nscenes, mixed, r.bc, r.list[kGateRefine]);
}
void bat_true_residual(const BatchRun& r, int gate, int flags) {
    APIC_PGRID(k_bat_true_residual);
    launch(false, k_bat_true_residual, g, kSegBlock, 0, r.st, r.tab, r.list[gate], gate, flags);
}
void bat_refine_cond(const BatchRun& r, cudaGraphConditionalHandle h, int gate) {
    k_bat_refine_cond<<<1, kBatCtlThreads, 0, r.st>>>(r.tab, r.nscenes, r.bc, h, gate, r.list[kGateRefine]);
}
void bat_pcg_begin(const BatchRun& r, int gate) {
    k_bat_pcg_begin<<<1, kBatCtlThreads, 0, r.st>>>(r.tab, r.nscenes, gate);
}
void bat_pcg_start(const BatchRun& r, int gate) {
    APIC_PGRID(k_bat_pcg_start);
    launch(r.pdl, k_bat_pcg_start, g, kSegBlock, 0, r.st, r.tab, r.list[gate], gate);
}
void bat_pcg_cond(const BatchRun& r, cudaGraphConditionalHandle h, int gate) {
    launch(r.pdl, k_bat_pcg_cond, 1, kBatCtlThreads, 0, r.st, r.tab, r.nscenes, static_cast<const BCtl*>(r.bc), h,
           gate, r.list[kGatePcg]);
}
void bat_round_end(const BatchRun& r, cudaGraphConditionalHandle h) {
    launch(r.pdl, k_bat_round_end, r.nscenes + 1, kSegBlock, 0, r.st, r.tab, r.nscenes, r.bc, h, r.list[kGatePcg]);
}
void bat_sap(const BatchRun& r) { launch(r.pdl, k_bat_sap, r.nscenes, kSegBlock, 0, r.st, r.tab, r.nscenes); }
void bat_spmv_dot(const BatchRun& r) {
    APIC_PGRID(k_bat_spmv_dot);
    k_bat_spmv_dot<<<g, kSegBlock, 0, r.st>>>(r.tab, r.list[kGatePcg]);
}
void bat_pcg_update(const BatchRun& r, int into_corr) {
    APIC_PGRID(k_bat_pcg_update);
    launch(r.pdl, k_bat_pcg_update, g, kSegBlock, 0, r.st, r.tab, r.list[kGatePcg], into_corr);
}
void bat_mixed_accumulate(const BatchRun& r, int gate, int finalize) {
    APIC_PGRID(k_bat_mixed_accumulate);
    launch(false, k_bat_mixed_accumulate, g, kSegBlock, 0, r.st, r.tab, r.list[gate], gate, finalize);
}
void bat_refine_end(const BatchRun& r) { k_bat_refine_end<<<1, kBatCtlThreads, 0, r.st>>>(r.tab, r.nscenes); }
void bat_finish_solve(const BatchRun& r) { k_bat_finish_solve<<<1, kBatCtlThreads, 0, r.st>>>(r.tab, r.nscenes); }
void bat_pressure_to64(const BatchRun& r, int gate) {
    APIC_PGRID(k_bat_pressure_to64);
    launch(false, k_bat_pressure_to64, g, kSegBlock, 0, r.st, r.tab, r.list[gate], gate);
}
#undef APIC_PGRID

// One PCG iteration (src/apic.rs:1899-1955); x receives alpha * s.  The
// search update that ends the reference's iteration happens at the start of
// the next one (inside k_spmv_dot / k_pcg_update), and k_pcg_update also
// runs the V-cycle's first base-level sweep.
static void pcg_iteration(Scene& s, int mode, float* x, int p_padded) {
    const Level& B = s.lv[0];
    uint32_t g = seg_grid(B.words);
    cudaStream_t st = s.stream;
    const bool pdl = s.use_pdl;
    k_spmv_dot<<<g, kSegBlock, 0, st>>>(B, s.search, s.ap, s.ctl, part_sap(s), mode,
                                         static_cast<const float2*>(part_rz(s)), g);
    if (mode == APIC_SOLVER_REFERENCE)
        launch(pdl, k_delta_exact, div_up(B.cells, kDeltaChunk), kDeltaThreads, 0, st, B,
               static_cast<const float*>(s.search), static_cast<const float*>(s.ap),
               static_cast<const uint32_t*>(s.seg_pre), s.ctl, s.exact_parts);
    launch(pdl, k_pcg_update, g, kSegBlock, 0, st, B, x, p_padded, s.search, s.ap, s.ctl,
           static_cast<const float2*>(part_sap(s)), g, part_res(s), mode, static_cast<const float*>(s.exact_parts),
           static_cast<const uint32_t*>(s.seg_pre), static_cast<const float2*>(part_rz(s)), g);
    // the residual's exit test runs inside the V-cycle's first kernel when
    // that is the base level's black sweep, else on its own
    const bool exit_in_vcycle = s.nlevels >= 2;
    if (!exit_in_vcycle)
        launch(pdl, k_residual_exit, 1, kSegBlock, 0, st, s.ctl, static_cast<const float4*>(part_res(s)), g, mode,
               s.props.solve_error, s.pcg_h, s.pcg_cap, s.pcg_dyn_cap, s.pcg_set_cond ? 1 : 0);
    // the V-cycle's last kernel also stores the parts of r.z (k_dot_rz's work)
    if (!enqueue_vcycle(s, true, mode, exit_in_vcycle)) launch(pdl, k_dot_rz, g, kSegBlock, 0, st, B, s.ctl, part_rz(s));
    if (mode == APIC_SOLVER_REFERENCE)
        launch(pdl, k_gamma_exact, 1, kGammaThreads, kGammaSmem, st, B, s.ctl, 0, s.pcg_h, s.pcg_cap, s.pcg_dyn_cap,
               s.pcg_set_cond ? 1 : 0);
}

// PCG setup (src/apic.rs:1885-1892) followed by a device-controlled WHILE
// loop over iterations.
// begin: reset the PCG state first (the refinement loop's k_refine_cond has
// already done so for its inner solves).
static cudaError_t build_pcg(Scene& s, GraphCursor& c, int mode, float* x, int p_padded, uint32_t cap, int dyn_cap,
                             bool clear_pressure, bool begin = true) {
    const Level& B = s.lv[0];
    uint32_t g = seg_grid(B.words);
    cudaGraphConditionalHandle h;
    cudaError_t e = cudaGraphConditionalHandleCreate(&h, c.g, 0, cudaGraphCondAssignDefault);
    if (e != cudaSuccess) return e;
    e = capture_into(s, c, [&]() {
        cudaStream_t st = s.stream;
        // only the reference-mode solve clears the pressure, and it starts here
        if (begin) k_pcg_begin<<<1, 1, 0, st>>>(s.ctl, clear_pressure ? 1 : 0);
        if (clear_pressure) k_clear_pressure<<<g, kSegBlock, 0, st>>>(B, s.pressure, s.ctl);
        if (mode == APIC_SOLVER_REFERENCE) k_seg_prefix<<<1, 1024, 0, st>>>(B, s.ctl, s.seg_pre);
        enqueue_vcycle(s);
        launch(s.use_pdl, k_pcg_start, g, kSegBlock, 0, st, B, s.search, s.ctl, s.partials, mode);
        if (mode == APIC_SOLVER_REFERENCE)
            launch(s.use_pdl, k_gamma_exact, 1, kGammaThreads, kGammaSmem, st, B, s.ctl, 1,
                   cudaGraphConditionalHandle(0), 0u, 0, 0);
        launch(s.use_pdl, k_pcg_cond, 1, 1, 0, st, static_cast<const Ctl*>(s.ctl), h, cap, dyn_cap);
        return cudaGetLastError();
    });
    if (e != cudaSuccess) return e;
    GraphCursor body;
    e = add_conditional_with(c, cudaGraphCondTypeWhile, h, &body);
    if (e != cudaSuccess) return e;
    // the loop condition is set inside the iteration (the residual's exit test,
    // or k_gamma_exact in the reference mode): no kernel of its own
    s.pcg_h = h;
    s.pcg_cap = cap;
    s.pcg_dyn_cap = dyn_cap;
    s.pcg_set_cond = true;
    e = capture_into(s, body, [&]() {
        pcg_iteration(s, mode, x, p_padded);
        return cudaGetLastError();
    });
    s.pcg_set_cond = false;
    s.kn_pcg = count_kernel_nodes(body.g);
    return e;
}

cudaError_t build_solve(Scene& s, GraphCursor& c) {
    s.kn_pcg = s.kn_refine = 0;
    cudaFuncSetAttribute(k_gamma_exact, cudaFuncAttributeMaxDynamicSharedMemorySize, int(kGammaSmem));
    const Level& B = s.lv[0];
    uint32_t g = seg_grid(B.words);
    int mode = s.solver_mode;
    s.p64_valid = false;
    cudaError_t e;
    if (mode == APIC_SOLVER_REFERENCE) {
        e = build_pcg(s, c, mode, s.pressure, 0, 100, 0, true);
        if (e != cudaSuccess) return e;
        return capture_into(s, c, [&]() {
            k_finish_solve<<<1, 1, 0, s.stream>>>(s.ctl, 100);
            return cudaGetLastError();
        });
    }
    const double tol = double(s.rel_tol);
    e = capture_into(s, c, [&]() {
        cudaStream_t st = s.stream;
        k_mixed_init<<<g, kSegBlock, 0, st>>>(B, s.b64, s.p64, s.ctl, s.partials, warm_start(s));
        k_clear_pressure<<<g, kSegBlock, 0, st>>>(B, s.pressure, s.ctl);
        k_rel_begin<<<1, 1, 0, st>>>(s.ctl, tol, s.max_iter);
        return cudaGetLastError();
    });
    if (e != cudaSuccess) return e;
    if (mode == APIC_SOLVER_REL_FP32) {
        e = build_pcg(s, c, APIC_SOLVER_REL_FP32, s.pressure, 0, s.max_iter, 1, false);
        if (e != cudaSuccess) return e;
        // true residual of the FP32 pressure that the projection will use
        return capture_into(s, c, [&]() {
            cudaStream_t st = s.stream;
            k_finish_solve<<<1, 1, 0, st>>>(s.ctl, s.max_iter);
            k_pressure_to64<<<g, kSegBlock, 0, st>>>(B, s.pressure, s.p64, s.ctl);
            k_true_residual<<<g, kSegBlock, 0, st>>>(B, s.b64, s.p64, s.corr, s.ctl, s.partials, 1);
            return cudaGetLastError();
        });
    }
    // APIC_SOLVER_REL_MIXED: r = b - A p in FP64, FP32 PCG on A d = r, p += d.
    cudaGraphConditionalHandle hr;
    e = cudaGraphConditionalHandleCreate(&hr, c.g, 0, cudaGraphCondAssignDefault);
    if (e != cudaSuccess) return e;
    e = capture_into(s, c, [&]() {
        cudaStream_t st = s.stream;
        k_true_residual<<<g, kSegBlock, 0, st>>>(B, s.b64, s.p64, s.corr, s.ctl, s.partials, 3);
        k_refine_cond<<<1, 1, 0, st>>>(s.ctl, hr, tol, s.max_iter, 1);
        return cudaGetLastError();
    });
    if (e != cudaSuccess) return e;
    GraphCursor body;
    e = add_conditional_with(c, cudaGraphCondTypeWhile, hr, &body);
    if (e != cudaSuccess) return e;
    e = build_pcg(s, body, APIC_SOLVER_REL_FP32, s.corr, 1, s.max_iter, 1, false, false);
    if (e != cudaSuccess) return e;
    e = capture_into(s, body, [&]() {
        cudaStream_t st = s.stream;
        k_mixed_accumulate<<<g, kSegBlock, 0, st>>>(B, s.p64, s.corr, s.pressure, s.ctl, 0);
        k_true_residual<<<g, kSegBlock, 0, st>>>(B, s.b64, s.p64, s.corr, s.ctl, s.partials, 3);
        k_refine_cond<<<1, 1, 0, st>>>(s.ctl, hr, tol, s.max_iter, 1);
        return cudaGetLastError();
    });
    if (e != cudaSuccess) return e;
    s.kn_refine = count_kernel_nodes(body.g);
    // the projection uses the FP64 pressure; its true residual is the one reported
    s.p64_valid = true;
    return capture_into(s, c, [&]() {
        cudaStream_t st = s.stream;
        k_mixed_accumulate<<<g, kSegBlock, 0, st>>>(B, s.p64, s.corr, s.pressure, s.ctl, 1);
        k_refine_end<<<1, 1, 0, st>>>(s.ctl, tol);
        return cudaGetLastError();
    });
}

// ---- eager form (profiling): same kernels, host-side loop control ----------

static cudaError_t read_ctl(Scene& s) {
    cudaError_t e = cudaMemcpyAsync(s.ctl_host, s.ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, s.stream);
    if (e != cudaSuccess) return e;
    return cudaStreamSynchronize(s.stream);
}

// PCG setup and iterations until the device flags convergence or the cap.
static cudaError_t eager_pcg(Scene& s, int mode, float* x, int p_padded, uint32_t cap, bool clear_pressure) {
    const Level& B = s.lv[0];
    uint32_t g = seg_grid(B.words);
    cudaStream_t st = s.stream;
    k_pcg_begin<<<1, 1, 0, st>>>(s.ctl, clear_pressure ? 1 : 0);
    if (clear_pressure) k_clear_pressure<<<g, kSegBlock, 0, st>>>(B, s.pressure, s.ctl);
    if (mode == APIC_SOLVER_REFERENCE) k_seg_prefix<<<1, 1024, 0, st>>>(B, s.ctl, s.seg_pre);
    enqueue_vcycle(s);
    k_pcg_start<<<g, kSegBlock, 0, st>>>(B, s.search, s.ctl, s.partials, mode);
    if (mode == APIC_SOLVER_REFERENCE)
        k_gamma_exact<<<1, kGammaThreads, kGammaSmem, st>>>(B, s.ctl, 1, cudaGraphConditionalHandle(0), 0u, 0, 0);
    s.pcg_set_cond = false;
    s.pcg_cap = cap;
    s.pcg_dyn_cap = 0;
    for (;;) {
        cudaError_t e = read_ctl(s);
        if (e != cudaSuccess) return e;
        if (s.ctl_host->pcg_done || s.ctl_host->pcg_iters >= cap) break;
        pcg_iteration(s, mode, x, p_padded);
    }
    return cudaGetLastError();
}

cudaError_t run_solve_eager(Scene& s) {
    cudaFuncSetAttribute(k_gamma_exact, cudaFuncAttributeMaxDynamicSharedMemorySize, int(kGammaSmem));
    const Level& B = s.lv[0];
    uint32_t g = seg_grid(B.words);
    cudaStream_t st = s.stream;
    int mode = s.solver_mode;
    s.p64_valid = false;
    cudaError_t e;
    if (mode == APIC_SOLVER_REFERENCE) {
        if ((e = eager_pcg(s, mode, s.pressure, 0, 100, true)) != cudaSuccess) return e;
        k_finish_solve<<<1, 1, 0, st>>>(s.ctl, 100);
        return cudaGetLastError();
    }
    const double tol = double(s.rel_tol);
    k_mixed_init<<<g, kSegBlock, 0, st>>>(B, s.b64, s.p64, s.ctl, s.partials, warm_start(s));
    k_clear_pressure<<<g, kSegBlock, 0, st>>>(B, s.pressure, s.ctl);
    k_rel_begin<<<1, 1, 0, st>>>(s.ctl, tol, s.max_iter);
    if (mode == APIC_SOLVER_REL_FP32) {
        if ((e = eager_pcg(s, mode, s.pressure, 0, s.max_iter, false)) != cudaSuccess) return e;
        k_finish_solve<<<1, 1, 0, st>>>(s.ctl, s.max_iter);
        k_pressure_to64<<<g, kSegBlock, 0, st>>>(B, s.pressure, s.p64, s.ctl);
        k_true_residual<<<g, kSegBlock, 0, st>>>(B, s.b64, s.p64, s.corr, s.ctl, s.partials, 1);
        return cudaGetLastError();
    }
    k_true_residual<<<g, kSegBlock, 0, st>>>(B, s.b64, s.p64, s.corr, s.ctl, s.partials, 3);
    k_refine_cond<<<1, 1, 0, st>>>(s.ctl, 0, tol, s.max_iter, 0);
    for (;;) {
        if ((e = read_ctl(s)) != cudaSuccess) return e;
        if (!s.ctl_host->cond) break;
        if ((e = eager_pcg(s, APIC_SOLVER_REL_FP32, s.corr, 1, s.ctl_host->inner_cap, false)) != cudaSuccess) return e;
        k_mixed_accumulate<<<g, kSegBlock, 0, st>>>(B, s.p64, s.corr, s.pressure, s.ctl, 0);
        k_true_residual<<<g, kSegBlock, 0, st>>>(B, s.b64, s.p64, s.corr, s.ctl, s.partials, 3);
        k_refine_cond<<<1, 1, 0, st>>>(s.ctl, 0, tol, s.max_iter, 0);
    }
    s.p64_valid = true;
    k_mixed_accumulate<<<g, kSegBlock, 0, st>>>(B, s.p64, s.corr, s.pressure, s.ctl, 1);
    k_refine_end<<<1, 1, 0, st>>>(s.ctl, tol);
    return cudaGetLastError();
}

}  // namespace apic
