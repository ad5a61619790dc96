// vcycle_common.cuh — per-cell V-cycle arithmetic shared by the graph kernels
// (vcycle.cu) and the distributed-shared-memory V-cycle (vcycle_dsm.cu).
//
// Restates MultiGridLevel::smooth_level (src/apic.rs:471-535), restrict
// (:537-594), prolongate (:596-616) and solve_coarse_exact (:618-704).
#pragma once

#include <cuda_runtime.h>

#include "apic_device.cuh"
#include "apic_internal.h"

namespace apic {
namespace vc {

constexpr float kOmega = 1.2f;
// "no preloaded segment word" (phases load seg[warp] themselves)
constexpr uint32_t kNoWord = 0xFFFFFFFFu;
constexpr int kTailThreads = 1024;
constexpr size_t kTailSmemBudget = 200 * 1024;

// ---- per-cell arithmetic shared by the global and the shared-memory kernels

// One SOR update (src/apic.rs:487-507) of padded cell c with raw index raw.
// nb(padded, raw) returns a neighbour's current error; neighbours that are not
// fluid are skipped (their reference contribution is zero).
template <class NB>
__device__ __forceinline__ float sor_cell(const uint32_t* bits, uint32_t w, uint32_t cells, const float* inv_d,
                                          const float* px, const float* py, const float* res, long long raw,
                                          uint32_t c, float old, bool neighbours, NB nb) {
    float inv = inv_d[c];
    if (inv == 0.0f) return old;
    float sum = res[c];
    if (neighbours) {
        const long long W = w;
        if (fluid_raw(bits, raw + 1, cells)) sum = __fmaf_rn(-px[c], nb(c + 1, raw + 1), sum);
        if (fluid_raw(bits, raw + W, cells)) sum = __fmaf_rn(-py[c], nb(c + w, raw + W), sum);
        if (fluid_raw(bits, raw - 1, cells)) sum = __fmaf_rn(-px[c - 1], nb(c - 1, raw - 1), sum);
        if (fluid_raw(bits, raw - W, cells)) sum = __fmaf_rn(-py[c - w], nb(c - w, raw - W), sum);
    }
    float gs = sum * inv;
    return old + (kOmega * (gs - old));
}

// Coarse residual of coarse cell (cx, cy) from its fine children (:549-583).
// E(padded, raw) gives the fine error of a fluid cell.
template <class E>
__device__ __forceinline__ float restrict_cell_fn(const uint32_t* fb, uint32_t fw, uint32_t fcells, const float* fd,
                                                  const float* fpx, const float* fpy, const float* fr, E fe,
                                                  uint32_t cx, uint32_t cy) {
    float sum = 0.0f;
    const long long W = fw;
    for (uint32_t dy = 0; dy < 2; ++dy)
        for (uint32_t dx = 0; dx < 2; ++dx) {
            long long rf = (long long)(cy * 2 + dy) * fw + (cx * 2 + dx);
            if (!fluid_raw(fb, rf, fcells)) continue;
            uint32_t pf = uint32_t(rf) + fw;
            float b = fr[pf];
            float ax = fd[pf] * fe(pf, rf);
            if (fluid_raw(fb, rf + 1, fcells)) ax += fpx[pf] * fe(pf + 1, rf + 1);
            if (fluid_raw(fb, rf + W, fcells)) ax += fpy[pf] * fe(pf + fw, rf + W);
            if (fluid_raw(fb, rf - 1, fcells)) ax += fpx[pf - 1] * fe(pf - 1, rf - 1);
            if (fluid_raw(fb, rf - W, fcells)) ax += fpy[pf - fw] * fe(pf - fw, rf - W);
            sum += b - ax;
        }
    return sum;
}

__device__ __forceinline__ float restrict_cell(const uint32_t* fb, uint32_t fw, uint32_t fcells, const float* fd,
                                               const float* fpx, const float* fpy, const float* fr, const float* fe,
                                               uint32_t cx, uint32_t cy) {
    return restrict_cell_fn(fb, fw, fcells, fd, fpx, fpy, fr, [fe](uint32_t p, long long) { return fe[p]; }, cx, cy);
}

// Branch-free forms of sor_cell / restrict_cell for the sweeps whose
// neighbour values are plain loads.  Every load is issued up front, without
// waiting for the fluid tests: all neighbours of a cell with raw index in
// [0, cells) have padded indices inside [0, cells + 2w), the extent of every
// level array.  Non-fluid neighbours (and children) are then dropped by
// selects, which yields the same floats as skipping them.  nb / fe must be
// safe to call for any such neighbour.
template <class NB>
__device__ __forceinline__ float sor_cell_all(const uint32_t* bits, uint32_t w, uint32_t cells, const float* inv_d,
                                              const float* px, const float* py, const float* res, long long raw,
                                              uint32_t c, float old, bool neighbours, NB nb) {
    const float inv = inv_d[c];
    float sum = res[c];
    if (neighbours) {
        const long long W = w;
        const bool fr = fluid_raw(bits, raw + 1, cells), fu = fluid_raw(bits, raw + W, cells);
        const bool fl = fluid_raw(bits, raw - 1, cells), fd = fluid_raw(bits, raw - W, cells);
        const float pxc = px[c], pyc = py[c], pxl = px[c - 1], pyd = py[c - w];
        const float er = nb(c + 1, raw + 1), eu = nb(c + w, raw + W), el = nb(c - 1, raw - 1), ed = nb(c - w, raw - W);
        float t = __fmaf_rn(-pxc, er, sum);
        sum = fr ? t : sum;
        t = __fmaf_rn(-pyc, eu, sum);
        sum = fu ? t : sum;
        t = __fmaf_rn(-pxl, el, sum);
        sum = fl ? t : sum;
        t = __fmaf_rn(-pyd, ed, sum);
        sum = fd ? t : sum;
    }
    const float gs = sum * inv;
    const float nv = old + (kOmega * (gs - old));
    return inv == 0.0f ? old : nv;
}

// Coarse residual of coarse cell (cx, cy) (any cell of the coarse grid).
__device__ __forceinline__ float restrict_cell_all(const uint32_t* fb, uint32_t fw, uint32_t fcells, const float* fd,
                                                   const float* fpx, const float* fpy, const float* fr,
                                                   const float* fe, uint32_t cx, uint32_t cy) {
    float sum = 0.0f;
    const long long W = fw;
#pragma unroll
    for (uint32_t dy = 0; dy < 2; ++dy)
#pragma unroll
        for (uint32_t dx = 0; dx < 2; ++dx) {
            const long long rf = (long long)(cy * 2 + dy) * fw + (cx * 2 + dx);
            const uint32_t pf = uint32_t(rf) + fw;
            const bool f0 = fluid_raw(fb, rf, fcells);
            const bool fr_ = fluid_raw(fb, rf + 1, fcells), fu = fluid_raw(fb, rf + W, fcells);
            const bool fl = fluid_raw(fb, rf - 1, fcells), fdn = fluid_raw(fb, rf - W, fcells);
            const float b = fr[pf];
            float ax = fd[pf] * fe[pf];
            float t = ax + fpx[pf] * fe[pf + 1];
            ax = fr_ ? t : ax;
            t = ax + fpy[pf] * fe[pf + fw];
            ax = fu ? t : ax;
            t = ax + fpx[pf - 1] * fe[pf - 1];
            ax = fl ? t : ax;
            t = ax + fpy[pf - fw] * fe[pf - fw];
            ax = fdn ? t : ax;
            t = sum + (b - ax);
            sum = f0 ? t : sum;
        }
    return sum;
}


// e + ec, plus ec again `reps` times (the padded base list, :611-615).
__device__ __forceinline__ float prolonged(float e, float ec, uint32_t reps) {
    e = e + ec;
    for (uint32_t k = 0; k < reps; ++k) e = e + ec;
    return e;
}

// ---- CTA-wide helpers -------------------------------------------------------
__device__ __forceinline__ double cta_sum(double v, double* sh) {
    v = warp_sum(v);
    int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) sh[warp] = v;
    __syncthreads();
    double t = 0;
    for (int w = 0; w < int(blockDim.x / 32); ++w) t += sh[w];
    return t;
}
__device__ __forceinline__ float cta_max(float v, float* sh) {
    v = warp_maxf(v);
    int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) sh[warp] = v;
    __syncthreads();
    float t = 0.0f;
    for (int w = 0; w < int(blockDim.x / 32); ++w) t = fmaxf(t, sh[w]);
    return t;
}

// solve_coarse_exact's FP32 sums (:627-629, :660, :681-687): a[c] * b[c]
// added one fluid cell after another in ascending order, by one thread.
__device__ __forceinline__ float serial_dot(const uint32_t* bits, uint32_t w, uint32_t cells, const float* a,
                                            const float* b) {
    float s = 0.0f;
    for (uint32_t r = 0; r < cells; ++r)
        if (bit_at(bits, r)) s = s + a[r + w] * b[r + w];
    return s;
}
// Sum of a CTA: FP64 over the threads' parts (fast), or the serial FP32 sum
// in the reference's order by thread 0 (exact; the vectors must be written
// and visible to the CTA).
__device__ __forceinline__ float cta_dot(bool exact, double part, const uint32_t* bits, uint32_t w, uint32_t cells,
                                         const float* a, const float* b, double* shd) {
    if (!exact) return float(cta_sum(part, shd));
    __shared__ float s_dot;
    __syncthreads();
    if (threadIdx.x == 0) s_dot = serial_dot(bits, w, cells, a, b);
    __syncthreads();
    return s_dot;
}

// Plain CG on the coarsest level (solve_coarse_exact, :618-704) by one CTA.
// Arrays may live in global or shared memory.  exact: the dot products are
// the reference's serial FP32 sums (reference solver mode); otherwise FP64
// sums over the threads.
static __device__ __noinline__ void cta_coarse_cg(const uint32_t* bits, uint32_t w, uint32_t cells, const float* diag, const float* px,
                              const float* py, const float* res, float* err, float* cs, float* cap, float* cr,
                              bool exact) {
    __shared__ double shd[32];
    __shared__ float shf[32];
    const long long W = w;
    uint32_t nf = 0;
    double g = 0;
    for (uint32_t r = threadIdx.x; r < cells; r += blockDim.x) {
        if (!bit_at(bits, r)) continue;
        uint32_t c = r + w;
        float rv = res[c];
        err[c] = 0.0f;
        cr[c] = rv;
        cs[c] = rv;
        g += double(rv * rv);
        nf++;
    }
    float gamma = cta_dot(exact, g, bits, w, cells, cr, cr, shd);
    uint32_t nfl = uint32_t(cta_sum(double(nf), shd));
    if (gamma < 1e-12f) return;
    uint32_t max_it = min(nfl, 100u);
    for (uint32_t it = 0; it < max_it; ++it) {
        __syncthreads();
        double d = 0;
        for (uint32_t r = threadIdx.x; r < cells; r += blockDim.x) {
            if (!bit_at(bits, r)) continue;
            uint32_t c = r + w;
            float v = diag[c] * cs[c];
            if (fluid_raw(bits, (long long)r + 1, cells)) v = __fmaf_rn(px[c], cs[c + 1], v);
            if (fluid_raw(bits, (long long)r - 1, cells)) v = __fmaf_rn(px[c - 1], cs[c - 1], v);
            if (fluid_raw(bits, (long long)r + W, cells)) v = __fmaf_rn(py[c], cs[c + w], v);
            if (fluid_raw(bits, (long long)r - W, cells)) v = __fmaf_rn(py[c - w], cs[c - w], v);
            cap[c] = v;
            d += double(cs[c] * v);
        }
        float delta = cta_dot(exact, d, bits, w, cells, cs, cap, shd);
        if (fabsf(delta) < 1e-5f) break;
        float alpha = gamma / delta;
        float me = 0.0f;
        for (uint32_t r = threadIdx.x; r < cells; r += blockDim.x) {
            if (!bit_at(bits, r)) continue;
            uint32_t c = r + w;
            err[c] = err[c] + alpha * cs[c];
            float nr = cr[c] - alpha * cap[c];
            cr[c] = nr;
            me = fmaxf(me, fabsf(nr));
        }
        if (cta_max(me, shf) < 1e-6f) break;
        double ng = 0;
        for (uint32_t r = threadIdx.x; r < cells; r += blockDim.x) {
            if (!bit_at(bits, r)) continue;
            uint32_t c = r + w;
            ng += double(cr[c] * cr[c]);
        }
        float new_gamma = cta_dot(exact, ng, bits, w, cells, cr, cr, shd);
        float beta = new_gamma / gamma;
        gamma = new_gamma;
        for (uint32_t r = threadIdx.x; r < cells; r += blockDim.x) {
            if (!bit_at(bits, r)) continue;
            uint32_t c = r + w;
            cs[c] = cr[c] + (beta * cs[c]);
        }
    }
    __syncthreads();
}

// The same CG run by one warp (shuffles only, no block barriers) for a
// coarsest level of at most 32 * kWarpCgCells cells; the other warps wait.
constexpr uint32_t kWarpCgCells = 8;
static __device__ __noinline__ void warp_coarse_cg(const uint32_t* bits, uint32_t w, uint32_t cells, const float* diag, const float* px,
                               const float* py, const float* res, float* err, float* cs, float* cap, float* cr,
                               bool exact) {
    if (threadIdx.x < 32) {
        const long long W = w;
        const uint32_t lane = threadIdx.x;
        auto wsum = [](double v) {
            for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
            return v;
        };
        // FP64 over the lanes, or the reference's serial FP32 sum by lane 0
        auto wdot = [&](double part, const float* a, const float* b) {
            if (!exact) return float(wsum(part));
            __syncwarp();
            float v = lane == 0 ? serial_dot(bits, w, cells, a, b) : 0.0f;
            return __shfl_sync(0xffffffffu, v, 0);
        };
        double g = 0, nf = 0;
        for (uint32_t r = lane; r < cells; r += 32) {
            if (!bit_at(bits, r)) continue;
            uint32_t c = r + w;
            float rv = res[c];
            err[c] = 0.0f;
            cr[c] = rv;
            cs[c] = rv;
            g += double(rv * rv);
            nf += 1.0;
        }
        float gamma = wdot(g, cr, cr);
        uint32_t nfl = uint32_t(wsum(nf));
        if (!(gamma < 1e-12f)) {
            uint32_t max_it = min(nfl, 100u);
            for (uint32_t it = 0; it < max_it; ++it) {
                __syncwarp();
                double d = 0;
                for (uint32_t r = lane; r < cells; r += 32) {
                    if (!bit_at(bits, r)) continue;
                    uint32_t c = r + w;
                    float v = diag[c] * cs[c];
                    if (fluid_raw(bits, (long long)r + 1, cells)) v = __fmaf_rn(px[c], cs[c + 1], v);
                    if (fluid_raw(bits, (long long)r - 1, cells)) v = __fmaf_rn(px[c - 1], cs[c - 1], v);
                    if (fluid_raw(bits, (long long)r + W, cells)) v = __fmaf_rn(py[c], cs[c + w], v);
                    if (fluid_raw(bits, (long long)r - W, cells)) v = __fmaf_rn(py[c - w], cs[c - w], v);
                    cap[c] = v;
                    d += double(cs[c] * v);
                }
                float delta = wdot(d, cs, cap);
                if (fabsf(delta) < 1e-5f) break;
                float alpha = gamma / delta;
                float me = 0.0f;
                for (uint32_t r = lane; r < cells; r += 32) {
                    if (!bit_at(bits, r)) continue;
                    uint32_t c = r + w;
                    err[c] = err[c] + alpha * cs[c];
                    float nr = cr[c] - alpha * cap[c];
                    cr[c] = nr;
                    me = fmaxf(me, fabsf(nr));
                }
                if (warp_maxf(me) < 1e-6f) break;
                double ng = 0;
                for (uint32_t r = lane; r < cells; r += 32) {
                    if (!bit_at(bits, r)) continue;
                    uint32_t c = r + w;
                    ng += double(cr[c] * cr[c]);
                }
                float new_gamma = wdot(ng, cr, cr);
                float beta = new_gamma / gamma;
                gamma = new_gamma;
                __syncwarp();
                for (uint32_t r = lane; r < cells; r += 32) {
                    if (!bit_at(bits, r)) continue;
                    uint32_t c = r + w;
                    cs[c] = cr[c] + (beta * cs[c]);
                }
            }
        }
    }
    __syncthreads();
}

// ---- the coarse tail in shared memory ----------------------------------------
struct TailLevel {
    uint32_t w, h, cells, words, padded;
    int wshift;   // log2 w, or -1 when w is not a power of two
    const uint32_t* fluid;
    const float *diag, *inv, *px, *py;
    float* res;   // global residual (read for the first tail level)
    float* err;   // global error (written back for the first tail level)
    uint32_t o_bits, o_diag, o_inv, o_px, o_py, o_res, o_err;  // shared offsets, 4-byte units
};
struct TailParams {
    int n;                      // tail levels; lv[n - 1] is the coarsest
    int exact;                  // coarsest CG with the reference's serial FP32 sums
    uint32_t o_cs, o_cap, o_cr;  // coarse CG vectors
    TailLevel lv[kMaxLevels];
};

struct SmemLevel {
    uint32_t w, h, cells;
    int wshift;
    uint32_t* bits;
    float *diag, *inv, *px, *py, *res, *err;
};

__device__ __forceinline__ SmemLevel smem_level(uint32_t* sm, const TailLevel& t) {
    float* f = reinterpret_cast<float*>(sm);
    return SmemLevel{t.w,          t.h,          t.cells,      t.wshift,     sm + t.o_bits, f + t.o_diag,
                     f + t.o_inv,  f + t.o_px,   f + t.o_py,   f + t.o_res,  f + t.o_err};
}

// One colour sweep of a shared-memory level (w even: every level that is
// swept has a coarser one).  Thread t visits the colour's cells k = t,
// t + blockDim.x, ... directly, row by row, and skips the cells outside the
// fluid mask (their result is never stored).
__device__ __forceinline__ void cta_sweep(const SmemLevel& L, int color, int init) {
    const float* e = L.err;
    const uint32_t half = L.w >> 1;
    const int hs = L.wshift > 0 ? L.wshift - 1 : -1;
    const uint32_t n = L.h * half;
    for (uint32_t k = threadIdx.x; k < n; k += blockDim.x) {
        uint32_t kk, row;
        raw_xy(k, half, hs, kk, row);
        const uint32_t r = row * L.w + 2u * kk + ((row + uint32_t(color)) & 1u);
        if (!bit_at(L.bits, r)) continue;
        const uint32_t c = r + L.w;
        const float old = init ? 0.0f : e[c];
        L.err[c] = sor_cell_all(L.bits, L.w, L.cells, L.inv, L.px, L.py, L.res, r, c, old, !(init && color == 0),
                                [e](uint32_t p, long long) { return e[p]; });
    }
    __syncthreads();
}



// ---- sweep phases over a level's segment list -------------------------------
// `warp` / `nwarps`: this warp's index in the grid and the grid's warp count.
// Each phase visits every fluid cell of the level once (one warp per segment).

// One colour sweep; init: first sweep after the level's error was zero-filled.
// Every lane of the colour computes (its loads do not wait for the mask word)
// and only fluid cells store.
// w0: this warp's first segment word if the caller loaded it early
// (before waiting on the previous kernel), else kNoWord.
__device__ __forceinline__ void ph_smooth(const Level& L, uint32_t nseg, uint32_t warp, uint32_t nwarps, int color,
                                          int init, uint32_t w0 = kNoWord) {
    const uint32_t lane = threadIdx.x & 31;
    const float* e = L.err;
    for (uint32_t s = warp, nxt = seg_first(L.seg, nseg, warp, w0); s < nseg; s += nwarps) {
        const uint32_t word = nxt;
        nxt = seg_next(L.seg, nseg, s + nwarps);
        const uint32_t raw = word * 32 + lane;
        if (raw >= L.cells || int(!red_at(raw, L.w, L.wshift)) != color) continue;
        const bool fluid = (L.fluid[word] >> lane) & 1u;
        const uint32_t c = raw + L.w;
        const float old = init ? 0.0f : e[c];
        const float v = sor_cell_all(L.fluid, L.w, L.cells, L.inv_diag, L.px, L.py, L.res, raw, c, old,
                                     !(init && color == 0), [e](uint32_t p, long long) { return e[p]; });
        if (fluid) L.err[c] = v;
    }
}

// Restriction into coarse level c; with_red also runs c's first (red) sweep.
__device__ __forceinline__ void ph_restrict(const Level& f, const Level& c, uint32_t nseg_c, uint32_t warp,
                                            uint32_t nwarps, bool with_red, uint32_t w0 = kNoWord) {
    const uint32_t lane = threadIdx.x & 31;
    for (uint32_t s = warp, nxt = seg_first(c.seg, nseg_c, warp, w0); s < nseg_c; s += nwarps) {
        const uint32_t word = nxt;
        nxt = seg_next(c.seg, nseg_c, s + nwarps);
        const uint32_t rc = word * 32 + lane;
        if (rc >= c.cells) continue;
        const bool fluid = (c.fluid[word] >> lane) & 1u;
        const uint32_t cp = rc + c.w;
        uint32_t cx, cy;
        raw_xy(rc, c.w, c.wshift, cx, cy);
        const float r = restrict_cell_all(f.fluid, f.w, f.cells, f.diag, f.px, f.py, f.res, f.err, cx, cy);
        const float inv = c.inv_diag[cp];
        if (!fluid) continue;
        c.res[cp] = r;
        if (with_red && ((cx + cy) & 1u) == 0u) c.err[cp] = inv != 0.0f ? 0.0f + (kOmega * (r * inv - 0.0f)) : 0.0f;
    }
}

// Prolongation from c fused with f's reverse sweep of one colour: black (1)
// reads red neighbours as prolonged values, red (0) reads final black ones.
// last / extra: the base level's duplicated last fluid cell (else ~0u / 0).
__device__ __forceinline__ void ph_prolong(const Level& c, const Level& f, uint32_t nseg_f, uint32_t warp,
                                           uint32_t nwarps, int color, uint32_t last, uint32_t extra,
                                           uint32_t w0 = kNoWord) {
    const uint32_t lane = threadIdx.x & 31;
    const float* fe = f.err;
    const float* ce = c.err;
    const uint32_t fw = f.w, cw = c.w;
    const long long fcells = f.cells;
    const int fs = f.wshift;
    // coarse error under fine raw index rf; rf outside the grid (a neighbour
    // whose value a select drops) is clamped so the load stays in bounds
    auto coarse_e = [=](long long rf) {
        const uint32_t r = uint32_t(rf < 0 ? 0 : (rf >= fcells ? fcells - 1 : rf));
        uint32_t x, y;
        raw_xy(r, fw, fs, x, y);
        return ce[(y >> 1) * cw + (x >> 1) + cw];
    };
    for (uint32_t s = warp, nxt = seg_first(f.seg, nseg_f, warp, w0); s < nseg_f; s += nwarps) {
        const uint32_t word = nxt;
        nxt = seg_next(f.seg, nseg_f, s + nwarps);
        const uint32_t raw = word * 32 + lane;
        if (raw >= f.cells || int(!red_at(raw, fw, fs)) != color) continue;
        const bool fluid = (f.fluid[word] >> lane) & 1u;
        const uint32_t p = raw + fw;
        const float old = prolonged(fe[p], coarse_e(raw), p == last ? extra : 0u);
        float v;
        if (color == 1)
            v = sor_cell_all(f.fluid, fw, f.cells, f.inv_diag, f.px, f.py, f.res, raw, p, old, true,
                             [=](uint32_t q, long long rq) {
                                 return prolonged(fe[q], coarse_e(rq), q == last ? extra : 0u);
                             });
        else
            v = sor_cell_all(f.fluid, fw, f.cells, f.inv_diag, f.px, f.py, f.res, raw, p, old, true,
                             [fe](uint32_t q, long long) { return fe[q]; });
        if (fluid) f.err[p] = v;
    }
}

// ph_prolong's red pass on the base level, also returning this thread's share
// of r.z over every fluid cell: red cells' new z, black cells' z as the
// black pass left it (final).  The products are those of pcg::ph_rz.
__device__ __forceinline__ F2 ph_prolong_red_rz(const Level& c, const Level& f, uint32_t nseg_f, uint32_t warp,
                                                uint32_t nwarps, uint32_t last, uint32_t extra,
                                                uint32_t w0 = kNoWord) {
    const uint32_t lane = threadIdx.x & 31;
    const float* fe = f.err;
    const float* ce = c.err;
    const uint32_t fw = f.w, cw = c.w;
    F2 acc{0.0f, 0.0f};
    for (uint32_t s = warp, nxt = seg_first(f.seg, nseg_f, warp, w0); s < nseg_f; s += nwarps) {
        const uint32_t word = nxt;
        nxt = seg_next(f.seg, nseg_f, s + nwarps);
        const uint32_t raw = word * 32 + lane;
        if (raw >= f.cells) continue;
        const bool fluid = (f.fluid[word] >> lane) & 1u;
        const uint32_t p = raw + fw;
        float z;
        uint32_t x, y;
        raw_xy(raw, fw, f.wshift, x, y);
        if (((x + y) & 1u) == 0u) {
            const float ec = ce[(y >> 1) * cw + (x >> 1) + cw];
            const float old = prolonged(fe[p], ec, p == last ? extra : 0u);
            z = sor_cell_all(f.fluid, fw, f.cells, f.inv_diag, f.px, f.py, f.res, raw, p, old, true,
                             [fe](uint32_t q, long long) { return fe[q]; });
            if (fluid) f.err[p] = z;
        } else {
            z = fe[p];
        }
        const float rz = f.res[p] * z;
        if (fluid) acc = f2_add(acc, rz);
    }
    return acc;
}

// Asynchronous 4-byte copy global -> shared (cp.async, sm_80+): the copies
// of a whole array set are issued back to back and complete together at
// cp_async_wait_all, so loading costs about one L2 round trip instead of one
// per loop iteration.
__device__ __forceinline__ void cp_async4(void* smem, const void* gmem) {
    const uint32_t sa = static_cast<uint32_t>(__cvta_generic_to_shared(smem));
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(sa), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }
// 16-byte form (both addresses 16-byte aligned), through L2 only.
__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
    const uint32_t sa = static_cast<uint32_t>(__cvta_generic_to_shared(smem));
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(sa), "l"(gmem) : "memory");
}

// Start copying every tail level's mask and coefficients into shared memory
// (complete after cp_async_wait_all).  The whole tail region is zeroed first:
// cells outside the fluid mask are never written, and with the stale shared
// memory of earlier kernels left in place the cluster-launched solve reached
// NaN (after other scenes had run in the process; the read that carried it
// was not located), while zeroed memory gives the same results as before.
__device__ __forceinline__ void cta_tail_issue_coeffs(const TailParams& tp, uint32_t* sm) {
    if (tp.n > 0) {
        const uint32_t words = tp.o_cr + tp.lv[tp.n - 1].padded;
        for (uint32_t i = threadIdx.x; i < words; i += blockDim.x) sm[i] = 0u;
        __syncthreads();  // zeroes land before any copy into the same words
    }
    for (int l = 0; l < tp.n; ++l) {
        const TailLevel& t = tp.lv[l];
        SmemLevel L = smem_level(sm, t);
        for (uint32_t i = threadIdx.x; i < t.words; i += blockDim.x) cp_async4(L.bits + i, t.fluid + i);
        for (uint32_t i = threadIdx.x; i < t.padded; i += blockDim.x) {
            cp_async4(L.diag + i, t.diag + i);
            cp_async4(L.inv + i, t.inv + i);
            cp_async4(L.px + i, t.px + i);
            cp_async4(L.py + i, t.py + i);
        }
    }
}

// Copy every tail level's mask and coefficients into shared memory.
__device__ __forceinline__ void cta_tail_load_coeffs(const TailParams& tp, uint32_t* sm) {
    cta_tail_issue_coeffs(tp, sm);
    cp_async_wait_all();
    __syncthreads();
}

// The coarse tail (levels held in shared memory) by one CTA.  load_coeffs:
// copy masks and coefficients first (otherwise they are already resident);
// the first level's residual is always copied in and its error copied out.
// load_coeffs false: the coefficients are resident or their copies were
// issued earlier by this CTA (cta_tail_issue_coeffs); the wait below covers
// those too.  global_io false: the first level's residual is already in
// shared memory and its error stays there (a cluster's other CTAs exchange
// them through distributed shared memory).
__device__ __forceinline__ void cta_tail(const TailParams& tp, uint32_t* sm, bool load_coeffs,
                                         bool global_io = true) {
    if (load_coeffs) cta_tail_issue_coeffs(tp, sm);
    if (global_io) {
        const TailLevel& t = tp.lv[0];
        SmemLevel L = smem_level(sm, t);
        for (uint32_t i = threadIdx.x; i < t.padded; i += blockDim.x) cp_async4(L.res + i, t.res + i);
    }
    cp_async_wait_all();
    __syncthreads();
    for (int l = 0; l + 1 < tp.n; ++l) {
        SmemLevel f = smem_level(sm, tp.lv[l]);
        SmemLevel c = smem_level(sm, tp.lv[l + 1]);
        cta_sweep(f, 0, 1);
        cta_sweep(f, 1, 1);
        for (uint32_t rc = threadIdx.x; rc < c.cells; rc += blockDim.x) {
            if (!bit_at(c.bits, rc)) continue;
            uint32_t cx, cy;
            raw_xy(rc, c.w, c.wshift, cx, cy);
            c.res[rc + c.w] = restrict_cell_all(f.bits, f.w, f.cells, f.diag, f.px, f.py, f.res, f.err, cx, cy);
        }
        __syncthreads();
    }
    {
        SmemLevel L = smem_level(sm, tp.lv[tp.n - 1]);
        float* fs = reinterpret_cast<float*>(sm);
        if (L.cells <= 32 * kWarpCgCells)
            warp_coarse_cg(L.bits, L.w, L.cells, L.diag, L.px, L.py, L.res, L.err, fs + tp.o_cs, fs + tp.o_cap,
                           fs + tp.o_cr, tp.exact != 0);
        else
            cta_coarse_cg(L.bits, L.w, L.cells, L.diag, L.px, L.py, L.res, L.err, fs + tp.o_cs, fs + tp.o_cap,
                          fs + tp.o_cr, tp.exact != 0);
    }
    for (int l = tp.n - 2; l >= 0; --l) {
        SmemLevel f = smem_level(sm, tp.lv[l]);
        SmemLevel c = smem_level(sm, tp.lv[l + 1]);
        for (uint32_t r = threadIdx.x; r < f.cells; r += blockDim.x)
            if (bit_at(f.bits, r)) {
                uint32_t x, y;
                raw_xy(r, f.w, f.wshift, x, y);
                f.err[r + f.w] = f.err[r + f.w] + c.err[(y >> 1) * c.w + (x >> 1) + c.w];
            }
        __syncthreads();
        cta_sweep(f, 1, 0);
        cta_sweep(f, 0, 0);
    }
    if (!global_io) {
        __syncthreads();
        return;
    }
    const TailLevel& t = tp.lv[0];
    SmemLevel L = smem_level(sm, t);
    for (uint32_t r = threadIdx.x; r < t.cells; r += blockDim.x)
        if (bit_at(L.bits, r)) t.err[r + t.w] = L.err[r + t.w];
}

// Host: tail parameters for levels [first, s.nlevels) laid out in shared memory.
inline TailParams make_tail_params(const Scene& s, int first, uint32_t* words_out) {
    TailParams tp;
    tp.n = s.nlevels - first;
    tp.exact = coarse_cg_exact(s) ? 1 : 0;
    uint32_t off = 0;
    for (int k = 0; k < tp.n; ++k) {
        const Level& v = s.lv[first + k];
        TailLevel& t = tp.lv[k];
        t.w = v.w; t.h = v.h; t.cells = v.cells; t.words = v.words; t.padded = v.padded;
        t.wshift = -1;
        for (int k = 0; k < 31; ++k)
            if ((1u << k) == v.w) t.wshift = k;
        t.fluid = v.fluid; t.diag = v.diag; t.inv = v.inv_diag; t.px = v.px; t.py = v.py;
        t.res = v.res; t.err = v.err;
        t.o_bits = off; off += v.words;
        t.o_diag = off; off += v.padded;
        t.o_inv = off; off += v.padded;
        t.o_px = off; off += v.padded;
        t.o_py = off; off += v.padded;
        t.o_res = off; off += v.padded;
        t.o_err = off; off += v.padded;
    }
    uint32_t cp = s.lv[s.nlevels - 1].padded;
    tp.o_cs = off; off += cp;
    tp.o_cap = off; off += cp;
    tp.o_cr = off; off += cp;
    *words_out = off;
    return tp;
}

}  // namespace vc
}  // namespace apic
