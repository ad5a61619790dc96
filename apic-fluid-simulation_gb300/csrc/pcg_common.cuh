// pcg_common.cuh — per-cell PCG phases on the base level, shared by the graph
// kernels (solver.cu) and the V-cycle (vcycle.cu).
//
// Restates Apic::solve_pcg (src/apic.rs:1865-1956) and apply_matrix_and_dot
// (:1823-1863).  Each phase visits the base fluid cells through the segment
// list (one warp per non-zero 32-cell mask word) and returns this thread's
// contribution to the phase's reduction; callers reduce deterministically.
#pragma once

#include <cuda_runtime.h>

#include "apic_device.cuh"
#include "apic_internal.h"

namespace apic {
namespace pcg {

#define APIC_BASE_LOOP(B, nseg, warp, nwarps)                                                          \
    const uint32_t lane_ = threadIdx.x & 31;                                                           \
    for (uint32_t s_ = (warp), nxt_ = seg_first((B).seg, (nseg), (warp), 0xFFFFFFFFu); s_ < (nseg);    \
         s_ += (nwarps))                                                                               \
        if (uint32_t word_ = seg_step((B).seg, (nseg), s_ + (nwarps), nxt_); ((B).fluid[word_] >> lane_) & 1u)

// The same loop over every lane of a segment inside the grid: the body runs
// without waiting for the mask word, so its loads issue at once, and tests
// fluid_ before it stores or accumulates.  All reads of a cell in [0, cells)
// and of its neighbours stay inside the padded arrays.
#define APIC_BASE_ALL(B, nseg, warp, nwarps) APIC_BASE_ALL_W0(B, nseg, warp, nwarps, 0xFFFFFFFFu)
// w0: the warp's first segment word when the caller loaded it early (before
// waiting on the previous kernel), else 0xFFFFFFFF.
#define APIC_BASE_ALL_W0(B, nseg, warp, nwarps, w0)                                                  \
    const uint32_t lane_ = threadIdx.x & 31;                                                         \
    for (uint32_t s_ = (warp), nxt_ = seg_first((B).seg, (nseg), (warp), (w0)); s_ < (nseg);        \
         s_ += (nwarps))                                                                             \
        if (const uint32_t word_ = seg_step((B).seg, (nseg), s_ + (nwarps), nxt_),                   \
            raw_ = word_ * 32 + lane_;                                                               \
            raw_ < (B).cells)                                                                        \
            if (const bool fluid_ = (((B).fluid[word_] >> lane_) & 1u) != 0u; true)

// pressure = 0 at fluid cells (src/apic.rs:1872-1883).
__device__ __forceinline__ void ph_clear_pressure(const Level& B, uint32_t nseg, uint32_t warp, uint32_t nwarps,
                                                  float* p) {
    APIC_BASE_LOOP(B, nseg, warp, nwarps) { p[word_ * 32 + lane_] = 0.0f; }
}

// s = z; returns r.z (src/apic.rs:1887-1888).  Dot products sum the FP32
// products in double-float (F2, apic_device.cuh).
__device__ __forceinline__ F2 ph_start(const Level& B, uint32_t nseg, uint32_t warp, uint32_t nwarps, float* s) {
    F2 acc{0.0f, 0.0f};
    APIC_BASE_ALL(B, nseg, warp, nwarps) {
        const uint32_t c = raw_ + B.w;
        const float z = B.err[c], r = B.res[c];
        if (!fluid_) continue;
        s[c] = z;
        acc = f2_add(acc, r * z);
    }
    return acc;
}

// Ap = A s (FMA chain of :1833-1846); returns s.Ap.
__device__ __forceinline__ F2 ph_spmv(const Level& B, uint32_t nseg, uint32_t warp, uint32_t nwarps,
                                      const float* s, float* ap) {
    F2 acc{0.0f, 0.0f};
    const long long W = B.w;
    APIC_BASE_ALL(B, nseg, warp, nwarps) {
        const long long raw = raw_;
        const uint32_t c = raw_ + B.w;
        const bool fr = fluid_raw(B.fluid, raw + 1, B.cells), fl = fluid_raw(B.fluid, raw - 1, B.cells);
        const bool fu = fluid_raw(B.fluid, raw + W, B.cells), fd = fluid_raw(B.fluid, raw - W, B.cells);
        const float sc = s[c], sr = s[c + 1], sl = s[c - 1], su = s[c + W], sd = s[c - W];
        const float pxc = B.px[c], pxl = B.px[c - 1], pyc = B.py[c], pyd = B.py[c - W];
        float v = B.diag[c] * sc;
        float t = __fmaf_rn(pxc, sr, v);
        v = fr ? t : v;
        t = __fmaf_rn(pxl, sl, v);
        v = fl ? t : v;
        t = __fmaf_rn(pyc, su, v);
        v = fu ? t : v;
        t = __fmaf_rn(pyd, sd, v);
        v = fd ? t : v;
        if (!fluid_) continue;
        ap[c] = v;
        acc = f2_add(acc, v * sc);
    }
    return acc;
}

// x += alpha s (x = pressure in cell layout, or a padded vector);
// r = fma(-alpha, Ap, r) (:1910-1928).  Returns max|r| and sum r^2 (each
// square exact, summed in double-float).
__device__ __forceinline__ void ph_update(const Level& B, uint32_t nseg, uint32_t warp, uint32_t nwarps, float alpha,
                                          float* x, int x_padded, const float* s, const float* ap, float* max_r,
                                          F2* r2) {
    float mx = 0.0f;
    F2 acc{0.0f, 0.0f};
    APIC_BASE_ALL(B, nseg, warp, nwarps) {
        const uint32_t c = raw_ + B.w;
        const uint32_t xi = x_padded ? c : raw_;
        const float nx = x[xi] + alpha * s[c];
        const float nr = __fmaf_rn(-alpha, ap[c], B.res[c]);
        if (!fluid_) continue;
        x[xi] = nx;
        B.res[c] = nr;
        mx = fmaxf(mx, fabsf(nr));
        acc = f2_add(acc, f2_square(nr));
    }
    *max_r = mx;
    *r2 = acc;
}

// ---- graph-path forms with the search update folded in -----------------------
// The search direction of an iteration, s' = z + beta s (:1945-1954), is not
// written by a kernel of its own: the SpMV evaluates it at the five stencil
// points from z and the previous s, and the update kernel, the last to read
// the previous s, stores it.  Both round exactly as the separate update would.
// With beta_valid == 0 (first iteration of a solve) s already holds z.

// s' at padded index q.
__device__ __forceinline__ float search_at(const float* z, const float* s, float beta, bool beta_valid, uint32_t q) {
    return beta_valid ? z[q] + (beta * s[q]) : s[q];
}

// Ap' = A s' (the FMA chain of :1833-1846); returns s'.Ap'.
__device__ __forceinline__ F2 ph_spmv_search(const Level& B, uint32_t nseg, uint32_t warp, uint32_t nwarps,
                                             const float* s, float beta, bool beta_valid, float* ap,
                                             uint32_t w0 = 0xFFFFFFFFu) {
    F2 acc{0.0f, 0.0f};
    const long long W = B.w;
    const float* z = B.err;
    APIC_BASE_ALL_W0(B, nseg, warp, nwarps, w0) {
        const long long raw = raw_;
        const uint32_t c = raw_ + B.w;
        const bool fr = fluid_raw(B.fluid, raw + 1, B.cells), fl = fluid_raw(B.fluid, raw - 1, B.cells);
        const bool fu = fluid_raw(B.fluid, raw + W, B.cells), fd = fluid_raw(B.fluid, raw - W, B.cells);
        const float sc = search_at(z, s, beta, beta_valid, c);
        const float sr = search_at(z, s, beta, beta_valid, c + 1), sl = search_at(z, s, beta, beta_valid, c - 1);
        const float su = search_at(z, s, beta, beta_valid, c + uint32_t(W));
        const float sd = search_at(z, s, beta, beta_valid, c - uint32_t(W));
        const float pxc = B.px[c], pxl = B.px[c - 1], pyc = B.py[c], pyd = B.py[c - W];
        float v = B.diag[c] * sc;
        float t = __fmaf_rn(pxc, sr, v);
        v = fr ? t : v;
        t = __fmaf_rn(pxl, sl, v);
        v = fl ? t : v;
        t = __fmaf_rn(pyc, su, v);
        v = fu ? t : v;
        t = __fmaf_rn(pyd, sd, v);
        v = fd ? t : v;
        if (!fluid_) continue;
        ap[c] = v;
        acc = f2_add(acc, v * sc);
    }
    return acc;
}

// x += alpha s', r = fma(-alpha, Ap, r) (:1910-1928), s = s'; and on red
// cells the preconditioner's first sweep from zero error, which needs only
// the cell's new residual: z = 0 + omega (r / diag - 0) (smooth_level
// :487-507 with every neighbour still zero).  Returns max|r| and sum r^2.
__device__ __forceinline__ void ph_update_search(const Level& B, uint32_t nseg, uint32_t warp, uint32_t nwarps,
                                                 float alpha, float beta, bool beta_valid, float* x, int x_padded,
                                                 float* s, const float* ap, float* max_r, F2* r2,
                                                 uint32_t w0 = 0xFFFFFFFFu) {
    constexpr float kOmegaSor = 1.2f;
    float mx = 0.0f;
    F2 acc{0.0f, 0.0f};
    APIC_BASE_ALL_W0(B, nseg, warp, nwarps, w0) {
        const uint32_t c = raw_ + B.w;
        const uint32_t xi = x_padded ? c : raw_;
        const float sc = search_at(B.err, s, beta, beta_valid, c);
        const float nx = x[xi] + alpha * sc;
        const float nr = __fmaf_rn(-alpha, ap[c], B.res[c]);
        const float inv = B.inv_diag[c];
        if (!fluid_) continue;
        s[c] = sc;
        x[xi] = nx;
        B.res[c] = nr;
        if (red_at(raw_, B.w, B.wshift))
            B.err[c] = inv != 0.0f ? 0.0f + (kOmegaSor * (nr * inv - 0.0f)) : 0.0f;
        mx = fmaxf(mx, fabsf(nr));
        acc = f2_add(acc, f2_square(nr));
    }
    *max_r = mx;
    *r2 = acc;
}

// gamma' = r.z ends the reference mode's iteration (:1934-1943): beta, or
// the exit when r.z is below SAFTY.  Run by one thread.  (The relative modes
// form beta at the start of the next iteration, where a zero r.z ends the
// solve.)
__device__ __forceinline__ void finish_rz_reference(Ctl* ctl, float ng) {
    constexpr float kSafetyRz = 1e-5f;  // SAFTY, src/apic.rs:8
    if (ng < kSafetyRz) {
        ctl->pcg_done = 1;
        return;
    }
    ctl->beta = ng / ctl->gamma;
    ctl->beta_valid = 1;
    ctl->gamma = ng;
}

// After the residual's exit test: whether the PCG loop goes on (not
// converged, under the iteration cap; dyn_cap reads the remaining budget of a
// refinement).  In the relative modes a continuing loop's next iteration
// forms beta from the r.z parts that this iteration's V-cycle stores
// (beta_valid); the reference mode's k_gamma_exact does that itself.  Run by
// thread 0 of one block; loop_decision sets the graph's loop condition when
// set_cond.
__device__ __forceinline__ bool loop_continue(Ctl* ctl, int mode, uint32_t cap, int dyn_cap) {
    const uint32_t c = dyn_cap ? ctl->inner_cap : cap;
    const bool cont = !ctl->pcg_done && ctl->pcg_iters < c;
    if (cont && mode != APIC_SOLVER_REFERENCE) ctl->beta_valid = 1;
    return cont;
}
__device__ __forceinline__ void loop_decision(Ctl* ctl, int mode, cudaGraphConditionalHandle h, uint32_t cap,
                                              int dyn_cap, int set_cond) {
    const bool cont = loop_continue(ctl, mode, cap, dyn_cap);
    if (set_cond) cudaGraphSetConditional(h, cont ? 1u : 0u);
}

// The exits that k_pcg_update leaves to the next kernel: its delta stop, or
// the residual test on its block parts, max|r| < solve_error (reference
// mode, src/apic.rs:1929-1932) or ||r|| <= target * ||b||.  Run by one
// block, after the caller's dependency wait.
__device__ __forceinline__ void residual_exit(Ctl* ctl, const float4* part, uint32_t n, int mode, float solve_error) {
    if (ctl->delta_stop) {  // s.Ap was unusable: no update, no residual parts
        if (threadIdx.x == 0) ctl->pcg_done = 1;
        return;
    }
    double tot;
    float t;
    sum_max_partials<kSegBlock>(part, n, &tot, &t);
    if (threadIdx.x == 0) {
        if (mode == APIC_SOLVER_REFERENCE) {
            ctl->max_r_bits = __float_as_uint(t);
            if (t < solve_error) ctl->pcg_done = 1;
        } else {
            ctl->rnorm2 = tot;
            const double rel = ctl->bnorm2 > 0.0 ? sqrt(tot / ctl->bnorm2) : 0.0;
            if (rel <= ctl->target_rel) ctl->pcg_done = 1;
        }
    }
}

// r.z after the preconditioner (:1936).
__device__ __forceinline__ F2 ph_rz(const Level& B, uint32_t nseg, uint32_t warp, uint32_t nwarps) {
    F2 acc{0.0f, 0.0f};
    APIC_BASE_ALL(B, nseg, warp, nwarps) {
        const uint32_t c = raw_ + B.w;
        const float rz = B.res[c] * B.err[c];
        if (fluid_) acc = f2_add(acc, rz);
    }
    return acc;
}

// s = z + beta s (:1945-1954).
__device__ __forceinline__ void ph_search(const Level& B, uint32_t nseg, uint32_t warp, uint32_t nwarps, float beta,
                                          float* s) {
    APIC_BASE_ALL(B, nseg, warp, nwarps) {
        const uint32_t c = raw_ + B.w;
        const float v = B.err[c] + (beta * s[c]);
        if (fluid_) s[c] = v;
    }
}

// ---- FP64 refinement (APIC_SOLVER_REL_MIXED) ---------------------------------

// b64 = res, p64 = 0; returns ||b||^2.
// warm: keep p64 as the previous solve left it (the initial guess of the
// refinement), else start from zero.
__device__ __forceinline__ double ph_mixed_init(const Level& B, uint32_t nseg, uint32_t warp, uint32_t nwarps,
                                                double* b64, double* p64, int warm) {
    double bb = 0;
    APIC_BASE_ALL(B, nseg, warp, nwarps) {
        const uint32_t c = raw_ + B.w;
        const double b = double(B.res[c]);
        if (!fluid_) continue;
        b64[c] = b;
        if (!warm) p64[c] = 0.0;
        bb += b * b;
    }
    return bb;
}

// r64 = b64 - A p64 in FP64; flags bit 0: res = float(r64), bit 1: x = 0.
// Returns ||r64||^2.
__device__ __forceinline__ double ph_true_residual(const Level& B, uint32_t nseg, uint32_t warp, uint32_t nwarps,
                                                   const double* b64, const double* p64, float* x, int flags) {
    double rr = 0;
    const uint32_t W = B.w;
    // every load is issued before the fluid tests (all neighbours of a cell
    // inside the grid lie inside the padded arrays); non-fluid neighbours
    // are dropped by selects, which adds exactly what skipping them adds
    APIC_BASE_ALL(B, nseg, warp, nwarps) {
        const uint32_t c = raw_ + W;
        const long long raw = raw_;
        const float dg = B.diag[c], pxc = B.px[c], pxl = B.px[c - 1], pyc = B.py[c], pyd = B.py[c - W];
        const double pc = p64[c], pr = p64[c + 1], pl = p64[c - 1], pu = p64[c + W], pd = p64[c - W], bc = b64[c];
        const bool fr = fluid_raw(B.fluid, raw + 1, B.cells), fl = fluid_raw(B.fluid, raw - 1, B.cells);
        const bool fu = fluid_raw(B.fluid, raw + W, B.cells), fd = fluid_raw(B.fluid, raw - (long long)W, B.cells);
        double v = double(dg) * pc;
        double t = v + double(pxc) * pr;
        v = fr ? t : v;
        t = v + double(pxl) * pl;
        v = fl ? t : v;
        t = v + double(pyc) * pu;
        v = fu ? t : v;
        t = v + double(pyd) * pd;
        v = fd ? t : v;
        if (!fluid_) continue;
        const double r = bc - v;
        rr += r * r;
        if (flags & 1) B.res[c] = float(r);
        if (flags & 2) x[c] = 0.0f;
    }
    return rr;
}

// p64 += x, or (finalize) pressure = float(p64).
__device__ __forceinline__ void ph_accumulate(const Level& B, uint32_t nseg, uint32_t warp, uint32_t nwarps,
                                              double* p64, const float* x, float* pressure, int finalize) {
    APIC_BASE_ALL(B, nseg, warp, nwarps) {
        const uint32_t c = raw_ + B.w;
        const double p = p64[c];
        const float xv = finalize ? 0.0f : x[c];
        if (!fluid_) continue;
        if (!finalize) p64[c] = p + double(xv);
        else pressure[raw_] = float(p);
    }
}

// p64 = pressure (the FP32 pressure the projection uses, for its true residual).
__device__ __forceinline__ void ph_pressure_to64(const Level& B, uint32_t nseg, uint32_t warp, uint32_t nwarps,
                                                 const float* pressure, double* p64) {
    APIC_BASE_LOOP(B, nseg, warp, nwarps) {
        uint32_t raw = word_ * 32 + lane_;
        p64[raw + B.w] = double(pressure[raw]);
    }
}

#undef APIC_BASE_LOOP

}  // namespace pcg
}  // namespace apic
