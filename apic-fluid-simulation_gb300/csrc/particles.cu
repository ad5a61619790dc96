// particles.cu — particle <-> grid transfers on the GPU.
//
//   k_p2g       transfer_particles_to_grid's scatter (src/apic.rs:1237-1426):
//               APIC momentum and weight to the 4 u and 4 v faces, temporal
//               weight w_t (:1246-1248), cell-centred density (:1260-1284) and
//               the fluid bit of the particle's cell (:1358-1360).
//   k_g2p       transfer_grid_to_particles_and_advect (src/apic.rs:2057-2264)
//               over all padded lanes, fused with the max-speed reduction that
//               the next substep's CFL limit needs (get_max_particle_velocity,
//               :2412-2427) and a count of non-finite lanes.
//   k_vmax      stand-alone max speed (after the particle set is written).
//   k_permute   gather of the nine fields by the sorted `val` (:1068-1110).
//
// The reference sums P2G contributions with float CAS loops, so its sums come
// in thread-schedule order.  Here a CTA first sums its particles'
// contributions in shared memory (hardware float atomics) over the window of
// faces and cells they touch, then adds each touched entry to global memory
// once; both levels are likewise order-dependent at the last bit.  Every other result of these kernels is computed lane by lane with the
// reference's operation order.
#include <cuda_runtime.h>

#include <climits>

#include "apic_device.cuh"
#include "apic_internal.h"

namespace apic {
namespace {

// P2G accumulation window of one CTA: the faces and cells that its 256
// consecutive particles touch.  After the Morton sort consecutive slots are
// neighbouring cells, so the window is small; a CTA whose window (per grid)
// exceeds kP2gCap entries, e.g. across a jump of the Morton curve or with
// unsorted particles, adds straight to global memory instead.
constexpr int kP2gThreads = 256;
constexpr int kP2gCap = 512;
// Shared-memory float atomics are compare-and-swap loops, and consecutive
// lanes hold particles of the same cell, so the window arrays are kept in
// kP2gCopies interleaved copies (entry e, copy c at e * kP2gCopies + c, in
// different banks) and lane l adds into copy l % kP2gCopies.
constexpr int kP2gCopies = 4;

struct Box {
    int x0, y0, w, h;
};

__device__ __forceinline__ int warp_min_i(int v) { return __reduce_min_sync(0xffffffffu, v); }
__device__ __forceinline__ int warp_max_i(int v) { return __reduce_max_sync(0xffffffffu, v); }

__global__ void __launch_bounds__(kP2gThreads, 4) k_p2g(const PartPtrs* __restrict__ pp, uint32_t n, int W, int H,
                                                     float dx, const Ctl* __restrict__ ctl, float* __restrict__ acc_u,
                                                     float* __restrict__ acc_uw, float* __restrict__ acc_v,
                                                     float* __restrict__ acc_vw, float* __restrict__ dens,
                                                     uint32_t* __restrict__ fluid) {
    __shared__ float s_um[kP2gCap * kP2gCopies], s_uw[kP2gCap * kP2gCopies], s_vm[kP2gCap * kP2gCopies],
        s_vw[kP2gCap * kP2gCopies], s_d[kP2gCap * kP2gCopies];
    __shared__ uint8_t s_fl[kP2gCap];  // fluid cells of the density window
    __shared__ int s_red[kP2gThreads / 32][12];
    __shared__ Box s_box[3];
    __shared__ int s_tiled;
    pdl_wait();
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    const bool live = i < n;
    // bounds of the clamped node coordinates: u, v faces and density cells
    int b[12];
    float ua[4], wu[4], va[4], wv[4], cw[4];
    int ux[2], uy[2], vx2[2], vy2[2], cx[2], cy[2];
    int fx = 0, fy = 0;  // the particle's own cell (its fluid bit)
    if (live) {
        const float prev_dt = ctl->prev_dt;
        float px = pp->f[PX][i], py = pp->f[PY][i];
        float vx = pp->f[VX][i], vy = pp->f[VY][i];
        float cux = pp->f[CUX][i], cuy = pp->f[CUY][i];
        float cvx = pp->f[CVX][i], cvy = pp->f[CVY][i];
        float tr = pp->f[TR][i];

        float tau = (-tr) / prev_dt;
        float wt = temporal_w(tau);
        float gx = px / dx, gy = py / dx;

        // cell-centred density stencil
        float cgx = gx - 0.5f, cgy = gy - 0.5f;
        float cbx = floorf(cgx), cby = floorf(cgy);
        float ctx = cgx - cbx, cty = cgy - cby;
        cw[0] = ((1.0f - ctx) * (1.0f - cty)) * wt;
        cw[1] = (ctx * (1.0f - cty)) * wt;
        cw[2] = ((1.0f - ctx) * cty) * wt;
        cw[3] = (ctx * cty) * wt;
        int mx = W - 1, my = H - 1;
        int tbx = trunc_x86(cbx), tby = trunc_x86(cby);
        cx[0] = max(min(tbx, mx), 0); cx[1] = max(min(tbx + 1, mx), 0);
        cy[0] = max(min(tby, my), 0); cy[1] = max(min(tby + 1, my), 0);

        Stencil su, sv;
        u_stencil(gx, gy, W, H, dx, su);
        v_stencil(gx, gy, W, H, dx, sv);
        {
            // the same clamps as u_index / v_index
            int ix = trunc_x86(floorf(gx)), iy = trunc_x86(floorf(gy - 0.5f));
            ux[0] = max(min(ix, W), 0); ux[1] = max(min(ix + 1, W), 0);
            uy[0] = max(min(iy, H - 1), 0); uy[1] = max(min(iy + 1, H - 1), 0);
            int jx = trunc_x86(floorf(gx - 0.5f)), jy = trunc_x86(floorf(gy));
            vx2[0] = max(min(jx, W - 1), 0); vx2[1] = max(min(jx + 1, W - 1), 0);
            vy2[0] = max(min(jy, H), 0); vy2[1] = max(min(jy + 1, H), 0);
        }

        float clx = fmax_x86(fmin_x86(gx, float(W) - 1.0f), 0.0f);
        float cly = fmax_x86(fmin_x86(gy, float(H) - 1.0f), 0.0f);
        fx = trunc_x86(clx);
        fy = trunc_x86(cly);

#pragma unroll
        for (int k = 0; k < 4; ++k) {
            wu[k] = su.w[k] * wt;
            ua[k] = (vx + cux * su.ox[k] + cuy * su.oy[k]) * wu[k];
            wv[k] = sv.w[k] * wt;
            va[k] = (vy + cvx * sv.ox[k] + cvy * sv.oy[k]) * wv[k];
        }
        b[0] = ux[0]; b[1] = -ux[1]; b[2] = uy[0]; b[3] = -uy[1];
        b[4] = vx2[0]; b[5] = -vx2[1]; b[6] = vy2[0]; b[7] = -vy2[1];
        b[8] = min(cx[0], fx); b[9] = -max(cx[1], fx); b[10] = min(cy[0], fy); b[11] = -max(cy[1], fy);
    } else {
#pragma unroll
        for (int k = 0; k < 12; ++k) b[k] = INT_MAX;
    }
    // block minima of the lows and of the negated highs
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < 12; ++k) {
        int m = warp_min_i(b[k]);
        if (lane == 0) s_red[warp][k] = m;
    }
    __syncthreads();
    if (threadIdx.x < 3) {
        int lo_x = INT_MAX, hi_x = INT_MAX, lo_y = INT_MAX, hi_y = INT_MAX;
        for (int w = 0; w < kP2gThreads / 32; ++w) {
            lo_x = min(lo_x, s_red[w][4 * threadIdx.x + 0]);
            hi_x = min(hi_x, s_red[w][4 * threadIdx.x + 1]);
            lo_y = min(lo_y, s_red[w][4 * threadIdx.x + 2]);
            hi_y = min(hi_y, s_red[w][4 * threadIdx.x + 3]);
        }
        Box bx;
        bx.x0 = lo_x; bx.y0 = lo_y;
        bx.w = -hi_x - lo_x + 1; bx.h = -hi_y - lo_y + 1;
        s_box[threadIdx.x] = bx;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        bool ok = true;
        for (int g = 0; g < 3; ++g)
            ok = ok && s_box[g].w > 0 && s_box[g].h > 0 && (long long)s_box[g].w * s_box[g].h <= kP2gCap;
        s_tiled = ok ? 1 : 0;
    }
    __syncthreads();
    if (!s_tiled) {
        if (!live) return;
        const uint32_t fi = uint32_t(fy * W + fx);
        atomicOr(fluid + (fi >> 5), 1u << (fi & 31u));
        // node k = (x[k & 1], y[k >> 1]): the u_index / v_index of the stencils
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const uint32_t iu = uint32_t(uy[k >> 1]) * uint32_t(W + 1) + uint32_t(ux[k & 1]);
            if (ua[k] != 0.0f || wu[k] != 0.0f) { atomicAdd(acc_u + iu, ua[k]); atomicAdd(acc_uw + iu, wu[k]); }
        }
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const uint32_t iv = uint32_t(vy2[k >> 1]) * uint32_t(W) + uint32_t(vx2[k & 1]);
            if (va[k] != 0.0f || wv[k] != 0.0f) { atomicAdd(acc_v + iv, va[k]); atomicAdd(acc_vw + iv, wv[k]); }
        }
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const uint32_t ic = uint32_t(cy[k >> 1]) * uint32_t(W) + uint32_t(cx[k & 1]);
            if (cw[k] != 0.0f) atomicAdd(dens + ic, cw[k]);
        }
        return;
    }
    const Box bu = s_box[0], bv = s_box[1], bc = s_box[2];
    for (int e = threadIdx.x; e < bu.w * bu.h * kP2gCopies; e += kP2gThreads) { s_um[e] = 0.0f; s_uw[e] = 0.0f; }
    for (int e = threadIdx.x; e < bv.w * bv.h * kP2gCopies; e += kP2gThreads) { s_vm[e] = 0.0f; s_vw[e] = 0.0f; }
    for (int e = threadIdx.x; e < bc.w * bc.h * kP2gCopies; e += kP2gThreads) s_d[e] = 0.0f;
    for (int e = threadIdx.x; e < bc.w * bc.h; e += kP2gThreads) s_fl[e] = 0;
    __syncthreads();
    if (live) {
        const int c = lane % kP2gCopies;
        s_fl[(fy - bc.y0) * bc.w + (fx - bc.x0)] = 1;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const int lu = ((uy[k >> 1] - bu.y0) * bu.w + (ux[k & 1] - bu.x0)) * kP2gCopies + c;
            if (ua[k] != 0.0f || wu[k] != 0.0f) { atomicAdd(s_um + lu, ua[k]); atomicAdd(s_uw + lu, wu[k]); }
            const int lv = ((vy2[k >> 1] - bv.y0) * bv.w + (vx2[k & 1] - bv.x0)) * kP2gCopies + c;
            if (va[k] != 0.0f || wv[k] != 0.0f) { atomicAdd(s_vm + lv, va[k]); atomicAdd(s_vw + lv, wv[k]); }
            const int lc = ((cy[k >> 1] - bc.y0) * bc.w + (cx[k & 1] - bc.x0)) * kP2gCopies + c;
            if (cw[k] != 0.0f) atomicAdd(s_d + lc, cw[k]);
        }
    }
    __syncthreads();
    // one global add per touched face and cell (the copies summed in order)
    auto sum_copies = [](const float* a, int e) {
        float t = a[e * kP2gCopies];
#pragma unroll
        for (int c = 1; c < kP2gCopies; ++c) t += a[e * kP2gCopies + c];
        return t;
    };
    for (int e = threadIdx.x; e < bu.w * bu.h; e += kP2gThreads) {
        const float m = sum_copies(s_um, e), w = sum_copies(s_uw, e);
        if (m != 0.0f || w != 0.0f) {
            const uint32_t g = uint32_t(bu.y0 + e / bu.w) * uint32_t(W + 1) + uint32_t(bu.x0 + e % bu.w);
            atomicAdd(acc_u + g, m);
            atomicAdd(acc_uw + g, w);
        }
    }
    for (int e = threadIdx.x; e < bv.w * bv.h; e += kP2gThreads) {
        const float m = sum_copies(s_vm, e), w = sum_copies(s_vw, e);
        if (m != 0.0f || w != 0.0f) {
            const uint32_t g = uint32_t(bv.y0 + e / bv.w) * uint32_t(W) + uint32_t(bv.x0 + e % bv.w);
            atomicAdd(acc_v + g, m);
            atomicAdd(acc_vw + g, w);
        }
    }
    for (int e = threadIdx.x; e < bc.w * bc.h; e += kP2gThreads) {
        const float d = sum_copies(s_d, e);
        if (d != 0.0f) atomicAdd(dens + uint32_t(bc.y0 + e / bc.w) * uint32_t(W) + uint32_t(bc.x0 + e % bc.w), d);
    }
    // fluid bits: one OR per mask word that a window row overlaps (a row of
    // bc.w raw cells spans at most bc.w / 32 + 2 words)
    const int nw = bc.w / 32 + 2;
    for (int e = threadIdx.x; e < bc.h * nw; e += kP2gThreads) {
        const int r = e / nw, j = e % nw;
        const uint32_t first = uint32_t(bc.y0 + r) * uint32_t(W) + uint32_t(bc.x0);
        const uint32_t last = first + uint32_t(bc.w) - 1u;
        const uint32_t word = (first >> 5) + uint32_t(j);
        if (word > (last >> 5)) continue;
        const uint32_t lo = max(first, word << 5), hi = min(last, (word << 5) + 31u);
        uint32_t mask = 0;
        for (uint32_t c = lo; c <= hi; ++c)
            if (s_fl[r * bc.w + int(c - first)]) mask |= 1u << (c & 31u);
        if (mask) atomicOr(fluid + word, mask);
    }
}

// bilinear_interpolate, src/apic.rs:138-172.
__device__ __forceinline__ float bilinear(const float w[4], const float v[4]) {
    float ws = w[0] + w[1] + w[2] + w[3];
    float inv = 1.0f / fmax_x86(ws, 1e-6f);
    float vel = 0.0f;
#pragma unroll
    for (int k = 0; k < 4; ++k) vel += v[k] * w[k] * inv;
    return vel;
}

__device__ __forceinline__ void block_max_count(float m, uint32_t bad, Ctl* ctl) {
    __shared__ float sm[8];
    __shared__ uint32_t sb[8];
    m = warp_maxf(m);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) bad += __shfl_xor_sync(0xffffffffu, bad, o);
    int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) { sm[warp] = m; sb[warp] = bad; }
    __syncthreads();
    if (threadIdx.x == 0) {
        float bm = 0.0f;
        uint32_t bb = 0;
        for (int w = 0; w < int(blockDim.x / 32); ++w) { bm = fmaxf(bm, sm[w]); bb += sb[w]; }
        if (bm > 0.0f) atomicMax(&ctl->vmax_bits, __float_as_uint(bm));
        if (bb) atomicAdd(&ctl->nonfinite, bb);
    }
}

__global__ void __launch_bounds__(256) k_g2p(const PartPtrs* __restrict__ pp, uint32_t npad, int W, int H, float dx,
                                             float border_damping, Ctl* __restrict__ ctl,
                                             const float* __restrict__ gu, const float* __restrict__ gv,
                                             const uint32_t* __restrict__ u_open,
                                             const uint32_t* __restrict__ v_open) {
    pdl_wait();
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    float speed_out = 0.0f;
    uint32_t bad = 0;
    if (i < npad) {
        const float dt = ctl->dt;
        const uint32_t ts = ctl->timestamp;
        const float min_x = 1.001f * dx, max_x = (float(W) - 1.001f) * dx;
        const float min_y = 1.001f * dx, max_y = (float(H) - 1.001f) * dx;
        const float h2 = dx * dx, eps = 1e-6f, bd = -border_damping;
        float px = pp->f[PX][i], py = pp->f[PY][i];
        float gx = px / dx, gy = py / dx;
        Stencil su, sv;
        u_stencil(gx, gy, W, H, dx, su);
        v_stencil(gx, gy, W, H, dx, sv);
        float un[4], vn[4], uwm[4], vwm[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            un[k] = gu[su.idx[k]];
            vn[k] = gv[sv.idx[k]];
            uwm[k] = bit_at(u_open, su.idx[k]) ? su.w[k] : 0.0f;
            vwm[k] = bit_at(v_open, sv.idx[k]) ? sv.w[k] : 0.0f;
        }
        float nvx = bilinear(uwm, un), nvy = bilinear(vwm, vn);
        float res = pp->f[TR][i];
        float speed = sqrtf(nvx * nvx + nvy * nvy);
        float cfl_local = speed * dt / dx;
        float scale = fmin_x86(fmax_x86(cfl_local, 0.0f), 1.0f);
        float gam = scale * scale * (3.0f - (2.0f * scale));
        float jitter = gam * random_lane(i, ts) * dt;
        float dt_raw = dt + res + jitter;
        float dt_act = fmin_x86(fmax_x86(dt_raw, 0.0f), dt * 2.0f);
        float nres = dt + res - dt_act;
        float nx = px + dt_act * nvx, ny = py + dt_act * nvy;
        bool oxmin = nx < min_x, oxmax = nx > max_x, oymin = ny < min_y, oymax = ny > max_y;
        bool ovxmin = oxmin && nvx < 0.0f, ovxmax = oxmax && nvx > 0.0f;
        bool ovymin = oymin && nvy < 0.0f, ovymax = oymax && nvy > 0.0f;
        if (oxmin) nx = min_x;
        if (oxmax) nx = max_x;
        if (ovxmin) nvx = nvx * bd;
        if (ovxmax) nvx = nvx * bd;
        if (oymin) ny = min_y;
        if (oymax) ny = max_y;
        if (ovymin) nvy = nvy * bd;
        if (ovymax) nvy = nvy * bd;
        float udx = h2 * su.tx * (1.0f - su.tx), udy = h2 * su.ty * (1.0f - su.ty);
        float vdx = h2 * sv.tx * (1.0f - sv.tx), vdy = h2 * sv.ty * (1.0f - sv.ty);
        float uix = udx > eps ? 1.0f / udx : 0.0f, uiy = udy > eps ? 1.0f / udy : 0.0f;
        float vix = vdx > eps ? 1.0f / vdx : 0.0f, viy = vdy > eps ? 1.0f / vdy : 0.0f;
        float cux = 0.0f, cuy = 0.0f, cvx = 0.0f, cvy = 0.0f;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            cux += su.w[k] * un[k] * su.ox[k];
            cuy += su.w[k] * un[k] * su.oy[k];
        }
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            cvx += sv.w[k] * vn[k] * sv.ox[k];
            cvy += sv.w[k] * vn[k] * sv.oy[k];
        }
        float cu_x = cux * uix, cu_y = cuy * uiy, cv_x = cvx * vix, cv_y = cvy * viy;
        bool rx = ovxmin || ovxmax, ry = ovymin || ovymax;
        if (rx) { cu_y = cu_y * -1.0f; cv_x = cv_x * -1.0f; }
        if (ry) { cu_y = cu_y * -1.0f; cv_x = cv_x * -1.0f; }
        pp->f[PX][i] = nx;
        pp->f[PY][i] = ny;
        pp->f[VX][i] = nvx;
        pp->f[VY][i] = nvy;
        pp->f[CUX][i] = cu_x;
        pp->f[CUY][i] = cu_y;
        pp->f[CVX][i] = cv_x;
        pp->f[CVY][i] = cv_y;
        pp->f[TR][i] = nres;
        float m = sqrtf(nvx * nvx + nvy * nvy);  // Vec2x8::mag of the stored velocity
        speed_out = (m == m) ? m : 0.0f;
        bad = (isfinite(nx) && isfinite(ny)) ? 0u : 1u;
    }
    block_max_count(speed_out, bad, ctl);
}

__global__ void __launch_bounds__(256) k_vmax(const PartPtrs* __restrict__ pp, uint32_t npad, Ctl* __restrict__ ctl) {
    pdl_wait();
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    float m = 0.0f;
    if (i < npad) {
        float vx = pp->f[VX][i], vy = pp->f[VY][i];
        float mg = sqrtf(vx * vx + vy * vy);
        m = (mg == mg) ? mg : 0.0f;
    }
    block_max_count(m, 0u, ctl);
}

__global__ void k_zero_vmax(Ctl* ctl) {
    pdl_wait(); ctl->vmax_bits = 0; ctl->nonfinite = 0; }

__global__ void __launch_bounds__(256) k_permute(PartPtrs* __restrict__ pp, const uint32_t* __restrict__ vals,
                                                 uint32_t n, uint32_t npad) {
    pdl_wait();
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= npad) return;
    if (i < n) {
        uint32_t src = vals[i];
#pragma unroll
        for (int f = 0; f < NPF; ++f) pp->alt[f][i] = pp->f[f][src];
    } else {
#pragma unroll
        for (int f = 0; f < NPF; ++f) pp->alt[f][i] = 0.0f;
    }
}

__global__ void k_swap_tables(PartPtrs* pp) {
    pdl_wait();
    int f = threadIdx.x;
    if (f < NPF) {
        float* t = pp->f[f];
        pp->f[f] = pp->alt[f];
        pp->alt[f] = t;
    }
}

}  // namespace

cudaError_t launch_p2g(Scene& s) {
    if (s.n == 0) return cudaSuccess;
    launch(s.use_pdl, k_p2g, div_up(s.n, kP2gThreads), kP2gThreads, 0, s.stream, s.pp, s.n, int(s.W), int(s.H), s.dx, s.ctl, s.acc_u, s.acc_uw,
                                                    s.acc_v, s.acc_vw, s.density, s.lv[0].fluid);
    return cudaGetLastError();
}

cudaError_t launch_g2p(Scene& s) {
    if (s.npad == 0) return cudaSuccess;
    launch(s.use_pdl, k_g2p, div_up(s.npad, 256), 256, 0, s.stream, s.pp, s.npad, int(s.W), int(s.H), s.dx, s.props.border_damping,
                                                      s.ctl, s.u, s.v, s.u_open, s.v_open);
    return cudaGetLastError();
}

// Zero the running maximum, then reduce over the current velocities.
cudaError_t launch_vmax(Scene& s) {
    launch(s.use_pdl, k_zero_vmax, 1, 1, 0, s.stream, s.ctl);
    if (s.npad) launch(s.use_pdl, k_vmax, div_up(s.npad, 256), 256, 0, s.stream, s.pp, s.npad, s.ctl);
    return cudaGetLastError();
}

// Interleave two SoA particle fields into the reference's Vec2x8 layout
// (per chunk: 8 x lanes then 8 y lanes), for one contiguous copy to the host.
__global__ void __launch_bounds__(256) k_pack_vec2x8(const PartPtrs* __restrict__ pp, int fx, int fy, uint32_t nchunks,
                                                     float* __restrict__ out) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nchunks * 16u) return;
    const uint32_t c = i >> 4, j = i & 15u;
    out[i] = j < 8u ? pp->f[fx][c * 8u + j] : pp->f[fy][c * 8u + (j - 8u)];
}

cudaError_t launch_pack_vec2x8(Scene& s, int which, float* out) {
    if (s.nchunks == 0) return cudaSuccess;
    k_pack_vec2x8<<<div_up(uint64_t(s.nchunks) * 16, 256), 256, 0, s.stream>>>(s.pp, 2 * which, 2 * which + 1,
                                                                             s.nchunks, out);
    return cudaGetLastError();
}

cudaError_t launch_permute(Scene& s) {
    if (s.npad == 0) return cudaSuccess;
    launch(s.use_pdl, k_permute, div_up(s.npad, 256), 256, 0, s.stream, s.pp, s.vals, s.n, s.npad);
    launch(s.use_pdl, k_swap_tables, 1, 32, 0, s.stream, s.pp);
    return cudaGetLastError();
}

}  // namespace apic
