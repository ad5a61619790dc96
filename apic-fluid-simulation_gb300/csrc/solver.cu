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

namespace apic {
namespace {

constexpr float kSafety = 1e-5f;  // SAFTY, src/apic.rs:8

#define SEG_LOOP(level_idx)                                                        \
    const uint32_t nseg = ctl->seg_count[level_idx];                               \
    const int lane = threadIdx.x & 31;                                             \
    const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;                         \
    for (uint32_t s_ = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; s_ < nseg; s_ += nwarps)

__global__ void k_pcg_begin(Ctl* ctl) {
    ctl->pcg_done = 0;
    ctl->pcg_iters = 0;
    ctl->gamma = 0.0f;
    ctl->alpha = 0.0f;
    ctl->beta = 0.0f;
    ctl->rnorm2 = 0.0;
}

// ---- PCG kernels on the base level ---------------------------------------

__global__ void __launch_bounds__(kSegBlock) k_clear_pressure(Level B, float* __restrict__ p, const Ctl* __restrict__ ctl) {
    SEG_LOOP(0) {
        uint32_t word = B.seg[s_];
        if ((B.fluid[word] >> lane) & 1u) p[word * 32 + lane] = 0.0f;
    }
}

// s = z and gamma = r.z (src/apic.rs:1887-1892).
__global__ void __launch_bounds__(kSegBlock) k_pcg_start(Level B, float* __restrict__ s, Ctl* __restrict__ ctl,
                                                         double* __restrict__ partials, int mode) {
    double acc = 0;
    SEG_LOOP(0) {
        uint32_t word = B.seg[s_];
        if (!((B.fluid[word] >> lane) & 1u)) continue;
        uint32_t c = word * 32 + lane + B.w;
        float z = B.err[c], r = B.res[c];
        s[c] = z;
        acc += double(r * z);
    }
    double tot;
    if (block_sum_last<kSegBlock>(acc, partials, &ctl->red_counter, &tot) && threadIdx.x == 0) {
        float gamma = float(tot);
        ctl->gamma = gamma;
        ctl->dgamma = tot;
        if (mode == APIC_SOLVER_REFERENCE ? (gamma < kSafety) : !(gamma != 0.0f)) ctl->pcg_done = 1;
    }
}

// Ap = A s and delta = s.Ap (apply_matrix_and_dot, src/apic.rs:1823-1863).
__global__ void __launch_bounds__(kSegBlock) k_spmv_dot(Level B, const float* __restrict__ s, float* __restrict__ ap,
                                                        Ctl* __restrict__ ctl, double* __restrict__ partials,
                                                        int mode) {
    if (ctl->pcg_done) return;
    double acc = 0;
    const long long W = B.w;
    SEG_LOOP(0) {
        uint32_t word = B.seg[s_];
        if (!((B.fluid[word] >> lane) & 1u)) continue;
        long long raw = (long long)word * 32 + lane;
        uint32_t c = uint32_t(raw) + B.w;
        float sc = s[c];
        float v = B.diag[c] * sc;
        if (fluid_raw(B.fluid, raw + 1, B.cells)) v = __fmaf_rn(B.px[c], s[c + 1], v);
        if (fluid_raw(B.fluid, raw - 1, B.cells)) v = __fmaf_rn(B.px[c - 1], s[c - 1], v);
        if (fluid_raw(B.fluid, raw + W, B.cells)) v = __fmaf_rn(B.py[c], s[c + W], v);
        if (fluid_raw(B.fluid, raw - W, B.cells)) v = __fmaf_rn(B.py[c - W], s[c - W], v);
        ap[c] = v;
        acc += double(v * sc);
    }
    double tot;
    if (block_sum_last<kSegBlock>(acc, partials, &ctl->red_counter, &tot) && threadIdx.x == 0) {
        float delta = float(tot);
        ctl->pcg_iters++;
        if (mode == APIC_SOLVER_REFERENCE) {
            if (fabsf(delta) < kSafety) { ctl->pcg_done = 1; return; }
            ctl->alpha = ctl->gamma / delta;
        } else {
            if (!(delta != 0.0f) || !isfinite(delta)) { ctl->pcg_done = 1; return; }
            ctl->alpha = ctl->gamma / delta;
        }
    }
}

// p += alpha s, r = fma(-alpha, Ap, r), max|r| (src/apic.rs:1907-1932);
// relative modes reduce ||r||^2 instead.  Relative modes accumulate into x.
__global__ void __launch_bounds__(kSegBlock) k_pcg_update(Level B, float* __restrict__ p, int p_padded,
                                                          const float* __restrict__ s, const float* __restrict__ ap,
                                                          Ctl* __restrict__ ctl, double* __restrict__ partials,
                                                          int mode, float solve_error) {
    if (ctl->pcg_done) return;
    const float alpha = ctl->alpha;
    double acc = 0;
    float mx = 0.0f;
    SEG_LOOP(0) {
        uint32_t word = B.seg[s_];
        if (!((B.fluid[word] >> lane) & 1u)) continue;
        uint32_t raw = word * 32 + lane;
        uint32_t c = raw + B.w;
        uint32_t pi = p_padded ? c : raw;
        p[pi] = p[pi] + alpha * s[c];
        float nr = __fmaf_rn(-alpha, ap[c], B.res[c]);
        B.res[c] = nr;
        mx = fmaxf(mx, fabsf(nr));
        acc += double(nr) * double(nr);
    }
    if (mode == APIC_SOLVER_REFERENCE) {
        float t;
        if (block_max_last<kSegBlock>(mx, partials, &ctl->red_counter, &t) && threadIdx.x == 0) {
            ctl->max_r_bits = __float_as_uint(t);
            if (t < solve_error) ctl->pcg_done = 1;
        }
    } else {
        double tot;
        if (block_sum_last<kSegBlock>(acc, partials, &ctl->red_counter, &tot) && threadIdx.x == 0) {
            ctl->rnorm2 = tot;
            double rel = ctl->bnorm2 > 0.0 ? sqrt(tot / ctl->bnorm2) : 0.0;
            if (rel <= ctl->target_rel) ctl->pcg_done = 1;
        }
    }
}

// gamma' = r.z, beta (src/apic.rs:1934-1943).
__global__ void __launch_bounds__(kSegBlock) k_dot_rz(Level B, Ctl* __restrict__ ctl, double* __restrict__ partials,
                                                      int mode) {
    if (ctl->pcg_done) return;
    double acc = 0;
    SEG_LOOP(0) {
        uint32_t word = B.seg[s_];
        if (!((B.fluid[word] >> lane) & 1u)) continue;
        uint32_t c = word * 32 + lane + B.w;
        acc += double(B.res[c] * B.err[c]);
    }
    double tot;
    if (block_sum_last<kSegBlock>(acc, partials, &ctl->red_counter, &tot) && threadIdx.x == 0) {
        float ng = float(tot);
        if (mode == APIC_SOLVER_REFERENCE ? (ng < kSafety) : !(ng != 0.0f)) { ctl->pcg_done = 1; return; }
        ctl->beta = ng / ctl->gamma;
        ctl->gamma = ng;
    }
}

// s = z + beta s (src/apic.rs:1945-1954); counts the iteration cap.
__global__ void __launch_bounds__(kSegBlock) k_search(Level B, float* __restrict__ s, const Ctl* __restrict__ ctl) {
    if (ctl->pcg_done) return;
    const float beta = ctl->beta;
    SEG_LOOP(0) {
        uint32_t word = B.seg[s_];
        if (!((B.fluid[word] >> lane) & 1u)) continue;
        uint32_t c = word * 32 + lane + B.w;
        s[c] = B.err[c] + (beta * s[c]);
    }
}

// ---- FP64 refinement helpers (APIC_SOLVER_REL_MIXED) ----------------------

// b64 = res (FP64 copy of the right-hand side), p64 = 0.
__global__ void __launch_bounds__(kSegBlock) k_mixed_init(Level B, double* __restrict__ b64, double* __restrict__ p64,
                                                          const Ctl* __restrict__ ctl) {
    SEG_LOOP(0) {
        uint32_t word = B.seg[s_];
        if (!((B.fluid[word] >> lane) & 1u)) continue;
        uint32_t c = word * 32 + lane + B.w;
        b64[c] = double(B.res[c]);
        p64[c] = 0.0;
    }
}

// r64 = b64 - A p64 in FP64 and the true relative residual; flags bit 0:
// res = float(r64), bit 1: x = 0 (start of an inner correction solve).
__global__ void __launch_bounds__(kSegBlock) k_true_residual(Level B, const double* __restrict__ b64,
                                                             const double* __restrict__ p64, float* __restrict__ x,
                                                             Ctl* __restrict__ ctl, double* __restrict__ partials,
                                                             int flags) {
    double rr = 0;
    const long long W = B.w;
    SEG_LOOP(0) {
        uint32_t word = B.seg[s_];
        if (!((B.fluid[word] >> lane) & 1u)) continue;
        long long raw = (long long)word * 32 + lane;
        uint32_t c = uint32_t(raw) + B.w;
        double v = double(B.diag[c]) * p64[c];
        if (fluid_raw(B.fluid, raw + 1, B.cells)) v += double(B.px[c]) * p64[c + 1];
        if (fluid_raw(B.fluid, raw - 1, B.cells)) v += double(B.px[c - 1]) * p64[c - 1];
        if (fluid_raw(B.fluid, raw + W, B.cells)) v += double(B.py[c]) * p64[c + W];
        if (fluid_raw(B.fluid, raw - W, B.cells)) v += double(B.py[c - W]) * p64[c - W];
        double r = b64[c] - v;
        rr += r * r;
        if (flags & 1) B.res[c] = float(r);
        if (flags & 2) x[c] = 0.0f;
    }
    double tot;
    if (block_sum_last<kSegBlock>(rr, partials, &ctl->red_counter, &tot) && threadIdx.x == 0) {
        ctl->true_rel = ctl->bnorm2 > 0.0 ? sqrt(tot / ctl->bnorm2) : 0.0;
    }
}

__global__ void __launch_bounds__(kSegBlock) k_bnorm(Level B, const double* __restrict__ b64, Ctl* __restrict__ ctl,
                                                     double* __restrict__ partials) {
    double bb = 0;
    SEG_LOOP(0) {
        uint32_t word = B.seg[s_];
        if (!((B.fluid[word] >> lane) & 1u)) continue;
        uint32_t c = word * 32 + lane + B.w;
        bb += b64[c] * b64[c];
    }
    double tot;
    if (block_sum_last<kSegBlock>(bb, partials, &ctl->red_counter, &tot) && threadIdx.x == 0) ctl->bnorm2 = tot;
}

// p64 += x; optionally pressure = float(p64) at the end.
__global__ void __launch_bounds__(kSegBlock) k_mixed_accumulate(Level B, double* __restrict__ p64,
                                                                const float* __restrict__ x,
                                                                float* __restrict__ pressure,
                                                                const Ctl* __restrict__ ctl, int finalize) {
    SEG_LOOP(0) {
        uint32_t word = B.seg[s_];
        if (!((B.fluid[word] >> lane) & 1u)) continue;
        uint32_t raw = word * 32 + lane;
        uint32_t c = raw + B.w;
        if (!finalize) p64[c] += double(x[c]);
        else pressure[raw] = float(p64[c]);
    }
}

// Pressure as FP64 field (for the true residual of modes 1 and 2).
__global__ void __launch_bounds__(kSegBlock) k_pressure_to64(Level B, const float* __restrict__ pressure,
                                                             double* __restrict__ p64, const Ctl* __restrict__ ctl) {
    SEG_LOOP(0) {
        uint32_t word = B.seg[s_];
        if (!((B.fluid[word] >> lane) & 1u)) continue;
        uint32_t raw = word * 32 + lane;
        p64[raw + B.w] = double(pressure[raw]);
    }
}

// ---- loop control (device side; each sets a graph conditional) ------------

// Continue the PCG loop while not converged and under the iteration cap
// (src/apic.rs:1894-1899); dyn_cap reads the remaining budget of a refinement.
__global__ void k_pcg_cond(const Ctl* __restrict__ ctl, cudaGraphConditionalHandle h, uint32_t cap, int dyn_cap) {
    uint32_t c = dyn_cap ? ctl->inner_cap : cap;
    cudaGraphSetConditional(h, (!ctl->pcg_done && ctl->pcg_iters < c) ? 1u : 0u);
}

__global__ void k_finish_solve(Ctl* ctl, uint32_t cap) {
    ctl->pcg_iters_total += ctl->pcg_iters;
    if (ctl->pcg_iters >= cap && !ctl->pcg_done) ctl->not_converged++;
}

__global__ void k_rel_begin(Ctl* ctl, double tol, uint32_t cap) {
    ctl->target_rel = tol;
    ctl->inner_cap = cap;
    ctl->refinements = 0;
    ctl->used_iters = 0;
}

// Refinement loop: go on while the FP64 true residual is above tol and
// iterations remain.  Each inner FP32 solve reduces its own right-hand side
// (the current true residual) by kInnerReduction, or down to tol / 2 of ||b||
// when that is reached first; FP32 cannot usefully reduce it further.
constexpr double kInnerReduction = 1e-4;
__global__ void k_refine_cond(Ctl* ctl, cudaGraphConditionalHandle h, double tol, uint32_t cap) {
    bool cont = ctl->true_rel > tol && ctl->used_iters < cap && ctl->refinements < 32u;
    // an inner solve that could not take a single step (r.z underflows or is
    // zero) will not make progress on the next round either
    if (ctl->refinements > 0u && ctl->pcg_iters == 0u) cont = false;
    if (cont) {
        ctl->refinements++;
        ctl->inner_cap = cap - ctl->used_iters;
        double t = kInnerReduction * ctl->true_rel;  // target relative to ||b||
        ctl->target_rel = t > 0.5 * tol ? t : 0.5 * tol;
    }
    cudaGraphSetConditional(h, cont ? 1u : 0u);
}

__global__ void k_refine_post(Ctl* ctl) { ctl->used_iters += ctl->pcg_iters; }

__global__ void k_refine_end(Ctl* ctl, double tol) {
    ctl->pcg_iters = ctl->used_iters;
    ctl->pcg_iters_total += ctl->used_iters;
    if (ctl->true_rel > tol) ctl->not_converged++;
}

#undef SEG_LOOP

}  // namespace

// One PCG iteration (src/apic.rs:1899-1955); x receives alpha * s.
static void pcg_iteration(Scene& s, int mode, float* x, int p_padded) {
    const Level& B = s.lv[0];
    uint32_t g = seg_grid(B.words);
    cudaStream_t st = s.stream;
    k_spmv_dot<<<g, kSegBlock, 0, st>>>(B, s.search, s.ap, s.ctl, s.partials, mode);
    k_pcg_update<<<g, kSegBlock, 0, st>>>(B, x, p_padded, s.search, s.ap, s.ctl, s.partials, mode, s.props.solve_error);
    enqueue_vcycle(s);
    k_dot_rz<<<g, kSegBlock, 0, st>>>(B, s.ctl, s.partials, mode);
    k_search<<<g, kSegBlock, 0, st>>>(B, s.search, s.ctl);
}

// PCG setup (src/apic.rs:1885-1892) followed by a device-controlled WHILE
// loop over iterations.
static cudaError_t build_pcg(Scene& s, GraphCursor& c, int mode, float* x, int p_padded, uint32_t cap, int dyn_cap,
                             bool clear_pressure) {
    const Level& B = s.lv[0];
    uint32_t g = seg_grid(B.words);
    cudaGraphConditionalHandle h;
    cudaError_t e = cudaGraphConditionalHandleCreate(&h, c.g, 0, cudaGraphCondAssignDefault);
    if (e != cudaSuccess) return e;
    e = capture_into(s, c, [&]() {
        cudaStream_t st = s.stream;
        k_pcg_begin<<<1, 1, 0, st>>>(s.ctl);
        if (clear_pressure) k_clear_pressure<<<g, kSegBlock, 0, st>>>(B, s.pressure, s.ctl);
        enqueue_vcycle(s);
        k_pcg_start<<<g, kSegBlock, 0, st>>>(B, s.search, s.ctl, s.partials, mode);
        k_pcg_cond<<<1, 1, 0, st>>>(s.ctl, h, cap, dyn_cap);
        return cudaGetLastError();
    });
    if (e != cudaSuccess) return e;
    GraphCursor body;
    e = add_conditional_with(c, cudaGraphCondTypeWhile, h, &body);
    if (e != cudaSuccess) return e;
    return capture_into(s, body, [&]() {
        pcg_iteration(s, mode, x, p_padded);
        k_pcg_cond<<<1, 1, 0, s.stream>>>(s.ctl, h, cap, dyn_cap);
        return cudaGetLastError();
    });
}

cudaError_t build_solve(Scene& s, GraphCursor& c) {
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
        k_mixed_init<<<g, kSegBlock, 0, st>>>(B, s.b64, s.p64, s.ctl);
        k_bnorm<<<g, kSegBlock, 0, st>>>(B, s.b64, s.ctl, s.partials);
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
        k_refine_cond<<<1, 1, 0, st>>>(s.ctl, hr, tol, s.max_iter);
        return cudaGetLastError();
    });
    if (e != cudaSuccess) return e;
    GraphCursor body;
    e = add_conditional_with(c, cudaGraphCondTypeWhile, hr, &body);
    if (e != cudaSuccess) return e;
    e = build_pcg(s, body, APIC_SOLVER_REL_FP32, s.corr, 1, s.max_iter, 1, false);
    if (e != cudaSuccess) return e;
    e = capture_into(s, body, [&]() {
        cudaStream_t st = s.stream;
        k_mixed_accumulate<<<g, kSegBlock, 0, st>>>(B, s.p64, s.corr, s.pressure, s.ctl, 0);
        k_refine_post<<<1, 1, 0, st>>>(s.ctl);
        k_true_residual<<<g, kSegBlock, 0, st>>>(B, s.b64, s.p64, s.corr, s.ctl, s.partials, 3);
        k_refine_cond<<<1, 1, 0, st>>>(s.ctl, hr, tol, s.max_iter);
        return cudaGetLastError();
    });
    if (e != cudaSuccess) return e;
    // the projection uses the FP64 pressure; its true residual is the one reported
    s.p64_valid = true;
    return capture_into(s, c, [&]() {
        cudaStream_t st = s.stream;
        k_mixed_accumulate<<<g, kSegBlock, 0, st>>>(B, s.p64, s.corr, s.pressure, s.ctl, 1);
        k_refine_end<<<1, 1, 0, st>>>(s.ctl, tol);
        return cudaGetLastError();
    });
}

}  // namespace apic
