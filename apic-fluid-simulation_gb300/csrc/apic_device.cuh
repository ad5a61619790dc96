// apic_device.cuh — device helpers that restate the reference's scalar rules.
//
// Compiled with -fmad=false: no multiply-add is contracted unless written as
// __fmaf_rn, which is used exactly where src/apic.rs calls mul_add.  Division
// and sqrt are IEEE (-prec-div=true -prec-sqrt=true, the nvcc defaults).
#pragma once

#include <climits>
#include <cstdint>

#include "apic_internal.h"

namespace apic {

// wide::f32x8::fast_max / fast_min (x86 maxps/minps operand rule).
__device__ __forceinline__ float fmax_x86(float a, float b) { return a > b ? a : b; }
__device__ __forceinline__ float fmin_x86(float a, float b) { return a < b ? a : b; }
// wide::f32x8::fast_trunc_int (cvttps2dq: out of range or NaN -> INT_MIN).
__device__ __forceinline__ int trunc_x86(float x) {
    return (x >= -2147483648.0f && x < 2147483648.0f) ? __float2int_rz(x) : INT_MIN;
}
// Rust f32::clamp.
__device__ __forceinline__ float rclamp(float x, float lo, float hi) {
    if (x < lo) x = lo;
    if (x > hi) x = hi;
    return x;
}

// temporal_kernel_w_t, src/apic.rs:31-46.
__device__ __forceinline__ float temporal_w(float tau) {
    float ts = tau - 0.5f;
    float tsq = ts * ts;
    float inner = fmax_x86(1.0f - tsq, 0.0f);
    float w = inner * inner * inner;
    float wt = w * 2.1875f;
    return fmax_x86(wt, 1e-5f);
}

// Apic::random_simd for one lane, src/apic.rs:946-975.
__device__ __forceinline__ float random_lane(uint32_t slot, uint32_t seed) {
    uint32_t m = slot ^ seed;
    m ^= m >> 16;
    m *= 0x7feb352du;
    m ^= m >> 15;
    m *= 0x846ca68bu;
    m ^= m >> 16;
    return __uint_as_float((m & 0x007FFFFFu) | 0x3F800000u) - 1.5f;
}

// expand_bits / morton_code, src/apic.rs:185-203.
__device__ __forceinline__ uint32_t expand_bits(uint32_t v) {
    v &= 0x0000FFFFu;
    v = (v | (v << 8)) & 0x00FF00FFu;
    v = (v | (v << 4)) & 0x0F0F0F0Fu;
    v = (v | (v << 2)) & 0x33333333u;
    v = (v | (v << 1)) & 0x55555555u;
    return v;
}
__device__ __forceinline__ uint32_t morton(uint32_t x, uint32_t y) { return expand_bits(x) | (expand_bits(y) << 1); }

// calculate_theta, src/apic.rs:1628-1638.
__device__ __forceinline__ float theta(float rho, float rho_center, float target) {
    float threshold = target * 0.5f;
    float diff = rho_center - rho;
    if (fabsf(diff) <= 1e-5f) return 1.0f;
    return rclamp((rho_center - threshold) / diff, 0.1f, 1.0f);
}

// u_index_simd / v_index_simd, src/apic.rs:1029-1041.
__device__ __forceinline__ uint32_t u_index(int i, int j, int W, int H) {
    uint32_t ci = uint32_t(max(min(i, W), 0));
    uint32_t cj = uint32_t(max(min(j, H - 1), 0));
    return cj * uint32_t(W + 1) + ci;
}
__device__ __forceinline__ uint32_t v_index(int i, int j, int W, int H) {
    uint32_t ci = uint32_t(max(min(i, W - 1), 0));
    uint32_t cj = uint32_t(max(min(j, H), 0));
    return cj * uint32_t(W) + ci;
}

// Staggered bilinear stencil (get_u_grid / get_v_grid / get_grid_distances,
// src/apic.rs:1113-1216): node indices bl, br, tl, tr, weights, node offsets.
struct Stencil {
    uint32_t idx[4];
    float w[4];
    float ox[4], oy[4];
    float tx, ty;
};

__device__ __forceinline__ void stencil_weights(Stencil& s) {
    float itx = 1.0f - s.tx, ity = 1.0f - s.ty;
    s.w[0] = itx * ity;
    s.w[1] = s.tx * ity;
    s.w[2] = itx * s.ty;
    s.w[3] = s.tx * s.ty;
}
__device__ __forceinline__ void stencil_offsets(Stencil& s, float dx) {
    float itx = 1.0f - s.tx, ity = 1.0f - s.ty;
    s.ox[0] = -s.tx * dx; s.oy[0] = -s.ty * dx;
    s.ox[1] = itx * dx;   s.oy[1] = -s.ty * dx;
    s.ox[2] = -s.tx * dx; s.oy[2] = ity * dx;
    s.ox[3] = itx * dx;   s.oy[3] = ity * dx;
}
__device__ __forceinline__ void u_stencil(float gx, float gy, int W, int H, float dx, Stencil& s) {
    float ugx = gx, ugy = gy - 0.5f;
    float bx = floorf(ugx), by = floorf(ugy);
    int ix = trunc_x86(bx), iy = trunc_x86(by);
    s.idx[0] = u_index(ix, iy, W, H);
    s.idx[1] = u_index(ix + 1, iy, W, H);
    s.idx[2] = u_index(ix, iy + 1, W, H);
    s.idx[3] = u_index(ix + 1, iy + 1, W, H);
    s.tx = ugx - bx;
    s.ty = ugy - by;
    stencil_weights(s);
    stencil_offsets(s, dx);
}
__device__ __forceinline__ void v_stencil(float gx, float gy, int W, int H, float dx, Stencil& s) {
    float vgx = gx - 0.5f, vgy = gy;
    float bx = floorf(vgx), by = floorf(vgy);
    s.tx = vgx - bx;
    s.ty = vgy - by;
    stencil_weights(s);
    int ix = trunc_x86(bx), iy = trunc_x86(by);
    s.idx[0] = v_index(ix, iy, W, H);
    s.idx[1] = v_index(ix + 1, iy, W, H);
    s.idx[2] = v_index(ix, iy + 1, W, H);
    s.idx[3] = v_index(ix + 1, iy + 1, W, H);
    stencil_offsets(s, dx);
}

// ---- bit masks (u32 words) ----
__device__ __forceinline__ uint32_t bit_at(const uint32_t* m, uint32_t i) { return (m[i >> 5] >> (i & 31)) & 1u; }
// Raw-index fluid test with the reference's index arithmetic; indices outside
// [0, cells) read as non-fluid (the padding rows of the padded layout are zero).
// (x, y) of raw index r on a grid w cells wide; shift = log2 w, or -1 when w
// is not a power of two (then a division).
__device__ __forceinline__ void raw_xy(uint32_t r, uint32_t w, int shift, uint32_t& x, uint32_t& y) {
    if (shift >= 0) {
        y = r >> shift;
        x = r & (w - 1u);
    } else {
        y = r / w;
        x = r - y * w;
    }
}
// Red cell of the checkerboard ((x + y) even, src/apic.rs list build).
__device__ __forceinline__ bool red_at(uint32_t r, uint32_t w, int shift) {
    uint32_t x, y;
    raw_xy(r, w, shift, x, y);
    return ((x + y) & 1u) == 0u;
}

// Checked build (-DAPIC_BOUNDS_CHECK): data-dependent indices (particle
// slots, cells, faces, sort destinations) are tested against their buffer
// before use; an index outside it sets kStatusBounds in *status (when
// given) and the access is skipped.  In the default build the test is
// `true` and compiles away: the index arithmetic is bounded by construction
// (clamped stencils, scans that sum to n).
#ifdef APIC_BOUNDS_CHECK
__device__ __forceinline__ bool in_bounds_checked(uint64_t i, uint64_t n, uint32_t* status) {
    if (i < n) return true;
    if (status) atomicOr(status, 16u);  // kStatusBounds
    return false;
}
#define APIC_IN_BOUNDS(i, n, status) ::apic::in_bounds_checked(uint64_t(i), uint64_t(n), (status))
#else
#define APIC_IN_BOUNDS(i, n, status) true
#endif

__device__ __forceinline__ uint32_t fluid_raw(const uint32_t* m, long long i, uint32_t cells) {
    if (i < 0 || i >= (long long)cells) return 0;
    return bit_at(m, uint32_t(i));
}
__device__ __forceinline__ uint32_t obstacle_raw(const uint32_t* m, long long i, uint32_t cells) {
    if (i < 0 || i >= (long long)cells) return 1;
    return bit_at(m, uint32_t(i));
}
// Apic::is_obstacle (src/apic.rs:994-1003): outside the grid is solid.
__device__ __forceinline__ uint32_t obstacle_xy(const uint32_t* m, int i, int j, int W, int H) {
    if (i < 0 || i >= W || j < 0 || j >= H) return 1;
    return bit_at(m, uint32_t(j * W + i));
}
// Apic::is_fluid (src/apic.rs:1015-1022).
__device__ __forceinline__ uint32_t fluid_xy(const uint32_t* m, int i, int j, int W, int H) {
    if (i < 0 || i >= W || j < 0 || j >= H) return 0;
    return bit_at(m, uint32_t(j * W + i));
}

// Programmatic dependent launch (sm_90+): wait until the kernel this one
// depends on has completed and its writes are visible (returns at once when
// the kernel was launched without the attribute), then let the next kernel's
// CTAs be scheduled.
__device__ __forceinline__ void pdl_wait() {
    asm volatile("griddepcontrol.wait;" ::: "memory");
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

// The GPU's global nanosecond timer (PTX %globaltimer).
__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// ---- block coordinates ----
// A block's index within its scene's grid and that grid's size in blocks.  A
// launch for one scene uses the hardware's values; a launch over many scenes
// (one grid whose blocks map to (scene, block) pairs through a table) gives
// each scene's blocks the indices that a launch of that scene alone would
// give them, so block partials and their sums come out the same bit for bit.
struct Blk {
    uint32_t id, n;
};
__device__ __forceinline__ Blk hw_blk() { return Blk{blockIdx.x, gridDim.x}; }
__device__ __forceinline__ uint32_t blk_warp(Blk b) { return (b.id * blockDim.x + threadIdx.x) >> 5; }
__device__ __forceinline__ uint32_t blk_nwarps(Blk b) { return (b.n * blockDim.x) >> 5; }

// ---- reductions ----
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ float warp_maxf(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

// Deterministic block sum into partials[bk.id]; returns true in the last
// block to finish, whose thread 0 receives the total of all partials (summed
// by a fixed strided pattern and tree, so the result does not depend on
// scheduling; no block waits on another).
template <int kThreads>
__device__ __forceinline__ bool block_sum_last(Blk bk, double v, double* partials, uint32_t* counter, double* total) {
    __shared__ double s_w[kThreads / 32];
    __shared__ bool s_last;
    v = warp_sum(v);
    int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) s_w[warp] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        double b = 0;
        for (int w = 0; w < kThreads / 32; ++w) b += s_w[w];
        partials[bk.id] = b;
        __threadfence();
        uint32_t prev = atomicAdd(counter, 1u);
        s_last = (prev == bk.n - 1);
    }
    __syncthreads();
    if (!s_last) return false;
    __threadfence();
    const volatile double* vp = partials;
    double t = 0;
    for (uint32_t b = threadIdx.x; b < bk.n; b += kThreads) t += vp[b];
    t = warp_sum(t);
    __syncthreads();
    if (lane == 0) s_w[warp] = t;
    __syncthreads();
    if (threadIdx.x == 0) {
        double a = 0;
        for (int w = 0; w < kThreads / 32; ++w) a += s_w[w];
        *total = a;
        *counter = 0;
    }
    return true;
}

// ---- double-float sums ---------------------------------------------------
// An unevaluated sum hi + lo of two floats (about 48 significant bits).  Sums
// of FP32 products accumulate in this form with FP32 instructions only:
// GB300 issues FP64 at a small fraction of the FP32 rate, and an FP64 add per
// cell plus five per warp shuffle level cost more than the sweep itself.
// Additions use Knuth's TwoSum for the high parts (exact error term) and
// fold the low parts in (the "sloppy" double-float add of Dekker/Bailey);
// -fmad=false keeps every operation as written.
struct F2 {
    float hi, lo;
};
__device__ __forceinline__ F2 f2_add(F2 a, F2 b) {
    float s = a.hi + b.hi;
    float v = s - a.hi;
    float e = (a.hi - (s - v)) + (b.hi - v);
    e = e + (a.lo + b.lo);
    float hi = s + e;
    return F2{hi, e - (hi - s)};
}
__device__ __forceinline__ F2 f2_add(F2 a, float b) { return f2_add(a, F2{b, 0.0f}); }
// a * a exactly (the FMA returns the rounding error of the product).
__device__ __forceinline__ F2 f2_square(float a) {
    float p = a * a;
    return F2{p, __fmaf_rn(a, a, -p)};
}
__device__ __forceinline__ double f2_value(F2 a) {
    return isfinite(a.hi) ? double(a.hi) + double(a.lo) : double(a.hi);
}
__device__ __forceinline__ F2 warp_sum(F2 v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        F2 w{__shfl_xor_sync(0xffffffffu, v.hi, o), __shfl_xor_sync(0xffffffffu, v.lo, o)};
        v = f2_add(v, w);
    }
    return v;
}

// block_sum_last for double-float sums; partials holds one F2 per block in
// the 8 bytes of a double.
template <int kThreads>
__device__ __forceinline__ bool block_sum_last(Blk bk, F2 v, double* partials, uint32_t* counter, double* total) {
    __shared__ F2 s_f[kThreads / 32];
    __shared__ bool s_last_f;
    float2* part = reinterpret_cast<float2*>(partials);
    v = warp_sum(v);
    int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) s_f[warp] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        F2 b{0.0f, 0.0f};
        for (int w = 0; w < kThreads / 32; ++w) b = f2_add(b, s_f[w]);
        part[bk.id] = make_float2(b.hi, b.lo);
        __threadfence();
        uint32_t prev = atomicAdd(counter, 1u);
        s_last_f = (prev == bk.n - 1);
    }
    __syncthreads();
    if (!s_last_f) return false;
    __threadfence();
    F2 t{0.0f, 0.0f};
    for (uint32_t b = threadIdx.x; b < bk.n; b += kThreads) {
        float2 q = __ldcg(part + b);  // from L2: written by other blocks
        t = f2_add(t, F2{q.x, q.y});
    }
    t = warp_sum(t);
    __syncthreads();
    if (lane == 0) s_f[warp] = t;
    __syncthreads();
    if (threadIdx.x == 0) {
        F2 a{0.0f, 0.0f};
        for (int w = 0; w < kThreads / 32; ++w) a = f2_add(a, s_f[w]);
        *total = f2_value(a);
        *counter = 0;
    }
    return true;
}

// ---- segment walks -------------------------------------------------------------
// A warp walks the segments s = warp, warp + nwarps, ... of a level (one
// non-zero 32-cell mask word each); the word of its next segment is loaded
// one step ahead, so a step's cell loads do not wait for their word (on
// large levels a warp has many segments).  w0: the first word if the caller
// loaded it already (else 0xFFFFFFFF).
__device__ __forceinline__ uint32_t seg_first(const uint32_t* seg, uint32_t nseg, uint32_t warp, uint32_t w0) {
    return w0 != 0xFFFFFFFFu ? w0 : (warp < nseg ? seg[warp] : 0u);
}
__device__ __forceinline__ uint32_t seg_next(const uint32_t* seg, uint32_t nseg, uint32_t s) {
    return s < nseg ? seg[s] : 0u;
}
// Returns the current word and loads the one of segment s into `next`.
__device__ __forceinline__ uint32_t seg_step(const uint32_t* seg, uint32_t nseg, uint32_t s, uint32_t& next) {
    const uint32_t cur = next;
    next = seg_next(seg, nseg, s);
    return cur;
}

// ---- split grid reductions ---------------------------------------------------
// The PCG loop's reductions stop at the block level: each block stores its
// partial, and the kernel that needs the total sums the partials itself after
// its dependency wait (the kernel boundary makes them visible), so no block
// fences, counts or waits at the end of the producing kernel.  The sums run
// in the order of block_sum_last's last block, so both forms give the same
// total.

// This block's F2 sum (and, with mx, its maximum) into slot bk.id.
template <int kThreads>
__device__ __forceinline__ void block_store(Blk bk, F2 v, float2* part) {
    __shared__ F2 s_bs[kThreads / 32];
    v = warp_sum(v);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) s_bs[warp] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        F2 b{0.0f, 0.0f};
        for (int w = 0; w < kThreads / 32; ++w) b = f2_add(b, s_bs[w]);
        part[bk.id] = make_float2(b.hi, b.lo);
    }
}

template <int kThreads>
__device__ __forceinline__ void block_store(Blk bk, F2 v, float mx, float4* part) {
    __shared__ F2 s_bs[kThreads / 32];
    __shared__ float s_bm[kThreads / 32];
    v = warp_sum(v);
    mx = warp_maxf(mx);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) {
        s_bs[warp] = v;
        s_bm[warp] = mx;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        F2 b{0.0f, 0.0f};
        float m = 0.0f;
        for (int w = 0; w < kThreads / 32; ++w) {
            b = f2_add(b, s_bs[w]);
            m = fmaxf(m, s_bm[w]);
        }
        part[bk.id] = make_float4(b.hi, b.lo, m, 0.0f);
    }
}

// Total of n partials, returned to every thread of the block.
template <int kThreads>
__device__ __forceinline__ double sum_partials(const float2* part, uint32_t n) {
    __shared__ F2 s_sp[kThreads / 32];
    __shared__ double s_tot;
    F2 t{0.0f, 0.0f};
#pragma unroll 4
    for (uint32_t b = threadIdx.x; b < n; b += kThreads) {
        const float2 q = __ldcg(part + b);
        t = f2_add(t, F2{q.x, q.y});
    }
    t = warp_sum(t);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) s_sp[warp] = t;
    __syncthreads();
    if (threadIdx.x == 0) {
        F2 a{0.0f, 0.0f};
        for (int w = 0; w < kThreads / 32; ++w) a = f2_add(a, s_sp[w]);
        s_tot = f2_value(a);
    }
    __syncthreads();
    return s_tot;
}

// Sum and maximum of n float4 partials (x, y: F2 sum; z: maximum).
template <int kThreads>
__device__ __forceinline__ void sum_max_partials(const float4* part, uint32_t n, double* sum, float* mx) {
    __shared__ F2 s_sp[kThreads / 32];
    __shared__ float s_mp[kThreads / 32];
    __shared__ double s_tot;
    __shared__ float s_max;
    F2 t{0.0f, 0.0f};
    float m = 0.0f;
#pragma unroll 4
    for (uint32_t b = threadIdx.x; b < n; b += kThreads) {
        const float4 q = __ldcg(part + b);
        t = f2_add(t, F2{q.x, q.y});
        m = fmaxf(m, q.z);
    }
    t = warp_sum(t);
    m = warp_maxf(m);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) {
        s_sp[warp] = t;
        s_mp[warp] = m;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        F2 a{0.0f, 0.0f};
        float b = 0.0f;
        for (int w = 0; w < kThreads / 32; ++w) {
            a = f2_add(a, s_sp[w]);
            b = fmaxf(b, s_mp[w]);
        }
        s_tot = f2_value(a);
        s_max = b;
    }
    __syncthreads();
    *sum = s_tot;
    *mx = s_max;
}

// Same pattern for a maximum of non-negative values (exact in any order).
template <int kThreads>
__device__ __forceinline__ bool block_max_last(float v, double* partials, uint32_t* counter, float* total) {
    __shared__ float s_m[kThreads / 32];
    __shared__ bool s_last;
    v = warp_maxf(v);
    int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) s_m[warp] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        float b = 0.0f;
        for (int w = 0; w < kThreads / 32; ++w) b = fmaxf(b, s_m[w]);
        partials[blockIdx.x] = double(b);
        __threadfence();
        s_last = atomicAdd(counter, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (!s_last) return false;
    __threadfence();
    const volatile double* vp = partials;
    float t = 0.0f;
    for (uint32_t b = threadIdx.x; b < gridDim.x; b += kThreads) t = fmaxf(t, float(vp[b]));
    t = warp_maxf(t);
    __syncthreads();
    if (lane == 0) s_m[warp] = t;
    __syncthreads();
    if (threadIdx.x == 0) {
        float a = 0.0f;
        for (int w = 0; w < kThreads / 32; ++w) a = fmaxf(a, s_m[w]);
        *total = a;
        *counter = 0;
    }
    return true;
}

}  // namespace apic
