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
// in thread-schedule order; here each contribution is one hardware float
// atomic (red.global.add.f32), which is likewise order-dependent at the last
// bit.  Every other result of these kernels is computed lane by lane with the
// reference's operation order.
#include <cuda_runtime.h>

#include "apic_device.cuh"
#include "apic_internal.h"

namespace apic {
namespace {

__global__ void __launch_bounds__(256) k_p2g(const PartPtrs* __restrict__ pp, uint32_t n, int W, int H, float dx,
                                             const Ctl* __restrict__ ctl, float* __restrict__ acc_u,
                                             float* __restrict__ acc_uw, float* __restrict__ acc_v,
                                             float* __restrict__ acc_vw, float* __restrict__ dens,
                                             uint32_t* __restrict__ fluid) {
    pdl_wait();
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
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
    float cw[4];
    cw[0] = ((1.0f - ctx) * (1.0f - cty)) * wt;
    cw[1] = (ctx * (1.0f - cty)) * wt;
    cw[2] = ((1.0f - ctx) * cty) * wt;
    cw[3] = (ctx * cty) * wt;
    int mx = W - 1, my = H - 1;
    int tbx = trunc_x86(cbx), tby = trunc_x86(cby);
    int cx0 = max(min(tbx, mx), 0), cx1 = max(min(tbx + 1, mx), 0);
    int cy0 = max(min(tby, my), 0), cy1 = max(min(tby + 1, my), 0);
    uint32_t ci[4] = {uint32_t(cy0 * W + cx0), uint32_t(cy0 * W + cx1), uint32_t(cy1 * W + cx0),
                      uint32_t(cy1 * W + cx1)};

    Stencil su, sv;
    u_stencil(gx, gy, W, H, dx, su);
    v_stencil(gx, gy, W, H, dx, sv);

    float clx = fmax_x86(fmin_x86(gx, float(W) - 1.0f), 0.0f);
    float cly = fmax_x86(fmin_x86(gy, float(H) - 1.0f), 0.0f);
    uint32_t fi = uint32_t(trunc_x86(cly) * W + trunc_x86(clx));
    atomicOr(fluid + (fi >> 5), 1u << (fi & 31u));

#pragma unroll
    for (int k = 0; k < 4; ++k) {
        float wu = su.w[k] * wt;
        float ua = (vx + cux * su.ox[k] + cuy * su.oy[k]) * wu;
        if (ua != 0.0f || wu != 0.0f) {
            atomicAdd(acc_u + su.idx[k], ua);
            atomicAdd(acc_uw + su.idx[k], wu);
        }
    }
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        float wv = sv.w[k] * wt;
        float va = (vy + cvx * sv.ox[k] + cvy * sv.oy[k]) * wv;
        if (va != 0.0f || wv != 0.0f) {
            atomicAdd(acc_v + sv.idx[k], va);
            atomicAdd(acc_vw + sv.idx[k], wv);
        }
    }
#pragma unroll
    for (int k = 0; k < 4; ++k)
        if (cw[k] != 0.0f) atomicAdd(dens + ci[k], cw[k]);
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
    launch(s.use_pdl, k_p2g, div_up(s.n, 256), 256, 0, s.stream, s.pp, s.n, int(s.W), int(s.H), s.dx, s.ctl, s.acc_u, s.acc_uw,
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
